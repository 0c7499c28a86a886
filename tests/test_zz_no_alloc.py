"""pxd_lbfgs_dev_noalloc: the batched optimiser with its scratch in a static device
array gives exactly what pxd_lbfgs_dev gives, on two calls in a row.

Each pose's optimisation runs within one warp and depends on nothing but the pose, so
the two entry points (different scratch, possibly a different grid) agree bit for bit.
"""
import numpy as np
import pytest

from pxdock_gb300 import model, native, synth

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point():
    import torch

    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=400, cube=18.0, cavity=5.0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (10.0, 10.0, 10.0), 0.5)
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)))
    ctx.set_slope(1e6)
    lid = ctx.add_ligand(lig)
    n, N = 512, lig.n_atoms
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    poses = synth.random_poses(lig, lo + 2.0, hi - 2.0, n, seed=9)
    dev = torch.device("cuda:0")
    start = torch.from_numpy(poses.astype(np.float32)).to(dev)
    ids = torch.full((n,), lid, dtype=torch.int32, device=dev)
    tors = torch.zeros(1, device=dev)
    p = native.lbfgs_params(max_iter=100, history=8, tolerance_grad=1e-3)

    def run(fn):
        xyz = start.clone()
        e = torch.zeros(n, dtype=torch.float64, device=dev)
        nev = torch.zeros(n, dtype=torch.int32, device=dev)
        st = torch.full((n,), -1, dtype=torch.int32, device=dev)
        fn(p, n, N, ids.data_ptr(), xyz.data_ptr(), tors.data_ptr(), e.data_ptr(), nev.data_ptr(),
           st.data_ptr())
        torch.cuda.synchronize()
        return xyz.cpu().numpy(), e.cpu().numpy(), nev.cpu().numpy(), st.cpu().numpy()

    ref = run(ctx.lbfgs_dev)
    assert np.all(ref[3] >= 0) and np.all(ref[2] > 0)
    for _ in range(2):
        got = run(ctx.lbfgs_dev_noalloc)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    ctx.close()
