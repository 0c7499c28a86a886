"""pxd_lbfgs_dev_noalloc: the batched optimiser with its scratch in a static device
array gives exactly what pxd_lbfgs_dev gives, on two calls in a row.

Each pose's optimisation runs within one warp and depends on nothing but the pose, so
the two entry points (different scratch, possibly a different grid) agree bit for bit.
That holds too when the static array holds fewer warps' history than the grid wants and
the no-alloc launch runs on a trimmed grid. The entry point refuses, rather than
allocates, when the device ligand table would have to grow, and it leaves the device's
free memory unchanged.
"""
import numpy as np
import pytest

from pxdock_gb300 import model, native, synth

pytestmark = pytest.mark.gpu

PXD_ERR_INVALID, PXD_ERR_STATE = 1, 2


@pytest.fixture(scope="module")
def system():
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=400, cube=18.0, cavity=5.0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (10.0, 10.0, 10.0), 0.5)
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    return rec, lig, box, synth.random_poses(lig, lo + 2.0, hi - 2.0, 512, seed=9)


def make_ctx(system):
    rec, lig, box, _ = system
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)))
    ctx.set_slope(1e6)
    return ctx, ctx.add_ligand(lig)


def runner(ctx, lid, poses, stride, p):
    """Runs an entry point on copies of `poses` laid out at `stride` atoms per pose."""
    import torch

    n, N = poses.shape[0], poses.shape[1]
    dev = torch.device("cuda:0")
    buf = np.zeros((n, stride, 3), np.float32)
    buf[:, :N] = poses
    start = torch.from_numpy(buf).to(dev)
    ids = torch.full((n,), lid, dtype=torch.int32, device=dev)
    tors = torch.zeros(1, device=dev)

    def run(fn):
        xyz = start.clone()
        e = torch.zeros(n, dtype=torch.float64, device=dev)
        nev = torch.zeros(n, dtype=torch.int32, device=dev)
        st = torch.full((n,), -1, dtype=torch.int32, device=dev)
        fn(p, n, stride, ids.data_ptr(), xyz.data_ptr(), tors.data_ptr(), e.data_ptr(), nev.data_ptr(),
           st.data_ptr())
        torch.cuda.synchronize()
        return xyz.cpu().numpy(), e.cpu().numpy(), nev.cpu().numpy(), st.cpu().numpy()

    return run


def test_noalloc_matches_allocating_entry_point(system):
    ctx, lid = make_ctx(system)
    poses = system[3]
    p = native.lbfgs_params(max_iter=100, history=8, tolerance_grad=1e-3)
    run = runner(ctx, lid, poses, poses.shape[1], p)
    ref = run(ctx.lbfgs_dev)
    assert np.all(ref[3] >= 0) and np.all(ref[2] > 0)
    for _ in range(2):
        got = run(ctx.lbfgs_dev_noalloc)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    ctx.close()


def test_noalloc_trimmed_grid_matches(system):
    """History 64 at a 256-atom pose stride: one block's history is 1.5 MiB, so the
    32 MiB array holds 21 blocks, fewer than the 152 the persistent grid wants; the
    trimmed grid still ends every pose where pxd_lbfgs_dev ends it."""
    ctx, lid = make_ctx(system)
    poses = system[3][:256]
    p = native.lbfgs_params(max_iter=60, history=64, tolerance_grad=1e-3)
    run = runner(ctx, lid, poses, 256, p)
    ref = run(ctx.lbfgs_dev)
    assert np.all(ref[3] >= 0) and np.all(ref[2] > 0)
    for _ in range(2):
        got = run(ctx.lbfgs_dev_noalloc)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    ctx.close()


def test_noalloc_refusals(system):
    """A context whose device ligand table was never allocated, or would have to grow
    (it holds 16 entries after the first allocating launch), is refused with
    PXD_ERR_STATE, and one allocating call makes room; parameters beyond the limits are
    refused with PXD_ERR_INVALID."""
    ctx, lid = make_ctx(system)
    poses = system[3][:64]
    lig = system[1]
    p = native.lbfgs_params(max_iter=20, history=8)
    run = runner(ctx, lid, poses, poses.shape[1], p)
    with pytest.raises(native.NativeError) as e:
        run(ctx.lbfgs_dev_noalloc)
    assert e.value.code == PXD_ERR_STATE
    run(ctx.lbfgs_dev)
    run(ctx.lbfgs_dev_noalloc)
    with pytest.raises(native.NativeError) as e:
        run_big = runner(ctx, lid, poses, poses.shape[1], native.lbfgs_params(max_iter=20, history=129))
        run_big(ctx.lbfgs_dev_noalloc)
    assert e.value.code == PXD_ERR_INVALID
    for _ in range(16):
        ctx.add_ligand(lig)
    with pytest.raises(native.NativeError) as e:
        run(ctx.lbfgs_dev_noalloc)
    assert e.value.code == PXD_ERR_STATE
    ref = run(ctx.lbfgs_dev)  # grows the table
    got = run(ctx.lbfgs_dev_noalloc)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    ctx.close()


def test_noalloc_leaves_free_memory_unchanged(system):
    import torch

    ctx, lid = make_ctx(system)
    poses = system[3]
    p = native.lbfgs_params(max_iter=50, history=8)
    run = runner(ctx, lid, poses, poses.shape[1], p)
    # an allocating call sizes the ligand table, the first no-alloc call resolves the
    # array's address; the runner's torch buffers of later calls come from torch's
    # cache, so only the entry point could change the free memory
    run(ctx.lbfgs_dev)
    run(ctx.lbfgs_dev_noalloc)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(3):
        run(ctx.lbfgs_dev_noalloc)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0
    ctx.close()
