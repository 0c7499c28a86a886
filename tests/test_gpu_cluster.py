"""Pose clustering on the GPU (pxd_cluster_poses_batch, pose_cluster::preprocess of
writer.cpp:99-177, one warp per ligand) against the host rule (pxd_cluster_poses) ligand by
ligand: the same kept poses in the same order. The candidates mix failed walkers
(nevals 0), near-duplicates of earlier poses (RMSD below min_rmsd, so the better one
replaces the closest mode) and more distinct poses than modes (the worst mode is
replaced by a better newcomer)."""
import ctypes as C

import numpy as np
import pytest

from pxdock_gb300 import abi, native

pytestmark = pytest.mark.gpu


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def test_device_clustering_matches_host_rule():
    lib = native.load(auto_build=True)
    i32p, f64p = C.POINTER(C.c_int32), C.POINTER(C.c_double)
    lib.pxd_cluster_poses.argtypes = [C.c_int32, C.c_int32, f64p, f64p, C.POINTER(C.c_int64), C.c_int32,
                                      C.c_double, i32p, i32p]
    lib.pxd_cluster_poses_batch.argtypes = [C.c_void_p, C.c_int32, i32p, i32p, C.c_int32, f64p, f64p, i32p,
                                            C.c_int32, C.c_double, i32p, i32p]
    rng = np.random.default_rng(7)
    n_groups, W, stride, modes, min_rmsd = 96, 48, 40, 8, 1.0
    atoms = rng.integers(8, stride + 1, size=n_groups).astype(np.int32)
    xyz = np.zeros((n_groups * W, stride, 3))
    ps = rng.normal(size=n_groups * W) * 10.0
    nev = rng.integers(1, 500, size=n_groups * W).astype(np.int32)
    nev[rng.random(n_groups * W) < 0.1] = 0
    for g in range(n_groups):
        base = rng.normal(size=(atoms[g], 3)) * 3.0
        for w in range(W):
            r = g * W + w
            src = rng.integers(0, 12)  # twelve basins: near-duplicates, and more basins than modes
            xyz[r, : atoms[g]] = base + src * 2.0 + rng.normal(scale=0.3, size=(atoms[g], 3))
    xyz = xyz.astype(np.float32).astype(np.float64)  # search outputs are FP32 values
    start = (np.arange(n_groups + 1) * W).astype(np.int32)
    ctx = native.Context(0)
    kept = np.full(n_groups * modes, -2, np.int32)
    n_kept = np.zeros(n_groups, np.int32)
    for _ in range(2):  # twice: the same lists
        rc = lib.pxd_cluster_poses_batch(ctx.h, n_groups, _p(start, C.c_int32), _p(atoms, C.c_int32), stride,
                                         _p(xyz, C.c_double), _p(ps, C.c_double), _p(nev, C.c_int32), modes,
                                         min_rmsd, _p(kept, C.c_int32), _p(n_kept, C.c_int32))
        assert rc == 0
        replaced = 0
        for g in range(n_groups):
            rows = slice(g * W, (g + 1) * W)
            hx = np.ascontiguousarray(xyz[rows, : atoms[g]])
            hk = np.zeros(modes, np.int32)
            hn = np.zeros(1, np.int32)
            ev = nev[rows].astype(np.int64)
            assert lib.pxd_cluster_poses(W, int(atoms[g]), _p(hx, C.c_double), _p(np.ascontiguousarray(ps[rows]),
                                         C.c_double), _p(ev, C.c_int64), modes, min_rmsd,
                                         _p(hk, C.c_int32), _p(hn, C.c_int32)) == 0
            got = kept[g * modes:(g + 1) * modes]
            assert n_kept[g] == hn[0]
            assert np.array_equal(got[: hn[0]] - g * W, hk[: hn[0]]), g
            assert np.all(got[hn[0]:] == -1)
            replaced += hn[0] == modes
        assert replaced > 0  # some ligands filled every mode
    with pytest.raises(native.NativeError):
        ctx._check(lib.pxd_cluster_poses_batch(ctx.h, 1, _p(start, C.c_int32), _p(atoms, C.c_int32), stride,
                                               _p(xyz, C.c_double), _p(ps, C.c_double), _p(nev, C.c_int32), 33,
                                               min_rmsd, _p(kept, C.c_int32), _p(n_kept, C.c_int32)))
    ctx.close()
