"""The reference's map cache files (receptor_cache::save / restore, grid.cpp:305-431)
through the library's host-side codec. No GPU calls here.

Parity is unpinned against Boost itself: Boost is not in this image and no file written
by the reference exists here. The bytes are checked against a second restatement of the
published Boost.Serialization layouts, written below with struct.pack, and the reader
is checked on the variations a Boost writer can produce (newer library versions, float
records, other bucket counts, newline delimiters).
"""
import struct

import numpy as np
import pytest

from pxdock_gb300 import mapcache, native

SIG = b"serialization::archive"


def boost_binary_vector(records, value_bytes=8, library=17):
    """std::vector<val_and_grad> in a Boost binary archive, restated from the format."""
    f = "<d" if value_bytes == 8 else "<f"
    out = struct.pack("<Q", len(SIG)) + SIG + struct.pack("<H", library)
    out += struct.pack("<BBBBi", 4, 8, 4, 8, 1)
    out += struct.pack("<BI", 0, 0)               # vector: tracking, class version
    out += struct.pack("<QI", len(records), 0)    # count, item version
    for i, (e, gx, gy, gz) in enumerate(records):
        if i == 0:
            out += struct.pack("<BI", 0, 0)       # val_and_grad preamble
        out += struct.pack(f, e)
        if i == 0:
            out += struct.pack("<BI", 0, 0)       # atom_position preamble
        out += struct.pack(f, gx) + struct.pack(f, gy) + struct.pack(f, gz)
    return out


@pytest.fixture(scope="module")
def lib():
    return native.load(auto_build=True)


def test_bdg_bytes_match_the_archive_layout(lib):
    rng = np.random.default_rng(0)
    rec = rng.normal(size=(7, 4)) * np.array([100.0, 1.0, 1.0, 1.0])
    rec[3] = [1e30, -1e30, 0.0, -0.0]
    assert mapcache.encode_bdg(rec) == boost_binary_vector(rec.tolist())
    assert mapcache.encode_bdg(rec, 4) == boost_binary_vector(rec.tolist(), 4)
    assert len(mapcache.encode_bdg(rec)) == 40 + 17 + 10 + 32 * 7


def test_bdg_round_trip_double_and_float(lib):
    rng = np.random.default_rng(1)
    rec = rng.normal(size=(55 ** 3, 4))
    back, vb = mapcache.decode_bdg(mapcache.encode_bdg(rec))
    assert vb == 8 and np.array_equal(back, rec)
    back, vb = mapcache.decode_bdg(boost_binary_vector(rec[:100].tolist(), 4, library=19))
    assert vb == 4 and np.array_equal(back, rec[:100].astype(np.float32).astype(np.float64))
    empty, vb = mapcache.decode_bdg(boost_binary_vector([]))
    assert empty.shape == (0, 4)


@pytest.mark.parametrize("damage", ["signature", "library", "sizes", "endian", "truncated", "trailing", "preamble"])
def test_bdg_reader_rejects_malformed_archives(lib, damage):
    good = bytearray(boost_binary_vector([[1.0, 2.0, 3.0, 4.0], [5.0, 6.0, 7.0, 8.0]]))
    if damage == "signature":
        good[8] = ord("S")
    elif damage == "library":
        good[30:32] = struct.pack("<H", 7)
    elif damage == "sizes":
        good[33] = 4  # sizeof(long) 4: another host's archive
    elif damage == "endian":
        good[36:40] = struct.pack(">i", 1)
    elif damage == "truncated":
        del good[-3:]
    elif damage == "trailing":
        good += b"\0"
    elif damage == "preamble":
        good[41:45] = struct.pack("<I", 3)  # a class version this layout does not have
    with pytest.raises(native.NativeError):
        mapcache.decode_bdg(bytes(good))


def test_meta_text_matches_the_archive_layout(lib):
    text = mapcache.encode_meta([-15.0, 1.25, 0.1], [81, 81, 49], 0.375, [12, 3, 40])
    expect = ("22 serialization::archive 17 20241030 3 -1.50000000000000000e+01 1.25000000000000000e+00 "
              "1.00000000000000006e-01 3 81 81 49 3.75000000000000000e-01 0 0 3 3 0 12 3 40\n")
    assert text == expect
    assert mapcache.encode_meta([0, 0, 0], [2, 2, 2], 1.0).endswith(" 0 0 0 1 0\n")


def test_meta_reader_round_trip_and_variants(lib):
    m = mapcache.decode_meta(mapcache.encode_meta([-15.0, 1.25, 0.1], [81, 81, 49], 0.375, [12, 3, 40]))
    assert m == dict(version=20241030, init_xyz=[-15.0, 1.25, 0.1], npoints=[81, 81, 49], spacing=0.375,
                     excluded=[12, 3, 40])
    # a newer Boost, newline delimiters, another bucket count and digits
    other = ("22 serialization::archive 20\n20241030\n3 -1.5e+01 1.25 0.1\n3 81 81 49\n0.375\n"
             "0 0 2 13 0\n7\n5\n")
    m = mapcache.decode_meta(other)
    assert m["npoints"] == [81, 81, 49] and m["excluded"] == [7, 5] and m["spacing"] == 0.375
    assert mapcache.decode_meta("22 serialization::archive 17 20240101 3 0 0 0")["version"] == 20240101


@pytest.mark.parametrize("text", ["", "22 serialization::archive", "21 serialization::archive 17 20241030",
                                  "22 serialization::archive 7 20241030 3 0 0 0 3 2 2 2 1 0 0 0 1 0",
                                  "22 serialization::archive 17 20241030 3 0 0 0 3 2 2 2 -1 0 0 0 1 0",
                                  "22 serialization::archive 17 20241030 3 0 0 0 3 2 1 2 1 0 0 0 1 0",
                                  "22 serialization::archive 17 20241030 3 0 0 0 3 2 2 2 1 0 0 2 3 0 1"])
def test_meta_reader_rejects_malformed_text(lib, text):
    with pytest.raises(native.NativeError):
        mapcache.decode_meta(text)
