"""The engine's JSON reader (protenix-dock_gb300/csrc/json.cpp), compiled here with g++:
values, escapes and numbers as Python's json module reads them, key order kept (the
reference walks rotor batches and fragment levels in file order), and errors on bad
input."""
import json
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "protenix-dock_gb300", "csrc")


@pytest.fixture(scope="module")
def reader(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("json") / "json_main")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "native", "json_main.cpp"),
                    os.path.join(CSRC, "json.cpp"), "-o", exe], check=True)

    def run(text):
        r = subprocess.run([exe], input=text.encode(), capture_output=True)
        return r.returncode, r.stdout.decode()

    return run


def test_values_round_trip(reader):
    doc = {"b": [1, -2.5, 1e-7, 6.02214076e23, 0.1],
           "a": {"z": True, "y": None, "x": 's"q\\\né'},
           "empty": [], "nested": [[[]], {}]}
    text = json.dumps(doc, ensure_ascii=True)
    rc, out = reader(text)
    assert rc == 0, out
    back = json.loads(out)
    assert back == doc
    assert list(back) == ["b", "a", "empty", "nested"]  # key order kept
    assert list(back["a"]) == ["z", "y", "x"]


def test_golden_files_parse_like_python(reader):
    golden = os.path.join(HERE, "golden")
    for name in ("utest_interaction_receptor.json", "scoring_function.json", os.path.join("engine", "ligand.json")):
        text = open(os.path.join(golden, name)).read()
        rc, out = reader(text)
        assert rc == 0, out
        assert json.loads(out) == json.loads(text)


@pytest.mark.parametrize("bad", ['{', '[1,]', '{"a" 1}', 'tru', '"abc', '[1] x', '{"a":"\\q"}'])
def test_bad_input_is_an_error(reader, bad):
    rc, out = reader(bad)
    assert rc == 1 and out.startswith("ERROR JSON parse error"), out
