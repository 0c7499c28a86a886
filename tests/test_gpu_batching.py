"""The batched L-BFGS launch over uneven ligands: poses are split into size classes on
the device and each class runs with shared memory sized for its own ligands. A pose's
result does not depend on that, so one mixed launch must equal per-ligand launches bit
for bit, in any pose order."""
import numpy as np
import pytest

from pxdock_gb300 import model, native, synth

pytestmark = pytest.mark.gpu


def test_size_classes_match_single_ligand_launches():
    import torch

    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=500, cube=18.0, cavity=6.0))
    ligs = [model.Ligand.from_json(synth.make_ligand(seed=s, n_heavy=h, n_rot=r, n_n=1, n_o=2))
            for s, h, r in ((3, 12, 2), (4, 22, 4), (6, 48, 7))]
    assert [l.n_atoms for l in ligs][0] <= 32 < ligs[1].n_atoms <= 64 < ligs[2].n_atoms
    box = model.make_box((0.0, 0.0, 0.0), (12.0, 12.0, 12.0), 0.5)
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, sorted(set(int(t) for l in ligs for t in l.vdw_type)))
    ctx.set_slope(1e6)
    ids = [ctx.add_ligand(l) for l in ligs]
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    per = 400
    maxN = max(l.n_atoms for l in ligs)
    dev = torch.device("cuda:0")
    p = native.lbfgs_params(max_iter=60, history=8, tolerance_grad=1e-3)
    tors = torch.zeros(1, device=dev)

    def run(xyz, lig_ids, N, params=None):
        n = len(lig_ids)
        x = torch.from_numpy(np.ascontiguousarray(xyz, np.float32)).to(dev)
        d_ids = torch.from_numpy(np.asarray(lig_ids, np.int32)).to(dev)
        e = torch.zeros(n, dtype=torch.float64, device=dev)
        nev = torch.zeros(n, dtype=torch.int32, device=dev)
        st = torch.full((n,), -1, dtype=torch.int32, device=dev)
        ctx.lbfgs_dev(params or p, n, N, d_ids.data_ptr(), x.data_ptr(), tors.data_ptr(), e.data_ptr(), nev.data_ptr(),
                      st.data_ptr())
        torch.cuda.synchronize()
        return x.cpu().numpy(), e.cpu().numpy(), nev.cpu().numpy(), st.cpu().numpy()

    starts = [synth.random_poses(l, lo + 1.0, hi - 1.0, per, seed=20 + k) for k, l in enumerate(ligs)]
    # one mixed launch, ligands interleaved
    n = per * len(ligs)
    xyz = np.zeros((n, maxN, 3), np.float32)
    lig_ids = np.zeros(n, np.int32)
    owner = np.zeros(n, int)
    perm = np.random.default_rng(1).permutation(n)
    for k, l in enumerate(ligs):
        rows = perm[k * per:(k + 1) * per]
        xyz[rows, : l.n_atoms] = starts[k]
        lig_ids[rows] = ids[k]
        owner[rows] = k
    mixed = run(xyz, lig_ids, maxN)
    assert np.all(mixed[3] >= 0) and np.all(mixed[2] > 0)
    for k, l in enumerate(ligs):
        single = run(starts[k], np.full(per, ids[k]), l.n_atoms)
        rows = perm[k * per:(k + 1) * per]
        assert np.array_equal(mixed[0][rows, : l.n_atoms], single[0])
        for a, b in zip(mixed[1:], single[1:]):
            assert np.array_equal(a[rows], b)
    # the history in shared memory instead of the global slab changes where S and Y live,
    # not the arithmetic: the same launch, bit for bit
    for b in (32, 64, 96):
        ctx.lbfgs_set_variant(b, 4 | native.LBFGS_HIST_SMEM)
    smem_hist = run(xyz, lig_ids, maxN)
    for a, b in zip(smem_hist, mixed):
        assert np.array_equal(a, b)
    for b in (32, 64, 96):
        ctx.lbfgs_set_variant(b, -1)
    # at history 100 the shared-memory history of the largest class does not fit: the
    # pinned variant falls back to the global slab, and the launch is the default one
    p100 = native.lbfgs_params(max_iter=20, history=100, tolerance_grad=1e-3)
    big = starts[2].astype(np.float32)
    ids_big = np.full(per, ids[2], np.int32)
    plain = run(big, ids_big, ligs[2].n_atoms, p100)
    ctx.lbfgs_set_variant(96, 4 | native.LBFGS_HIST_SMEM)
    pinned = run(big, ids_big, ligs[2].n_atoms, p100)
    ctx.lbfgs_set_variant(96, -1)
    for a, b in zip(pinned, plain):
        assert np.array_equal(a, b)
    with pytest.raises(native.NativeError):
        ctx.lbfgs_set_variant(48, 4)
    with pytest.raises(native.NativeError):
        ctx.lbfgs_set_variant(64, 7)
    # the autotuner picks a variant per size class from timed probes on copies; the
    # caller's poses are untouched and the tuned launch optimises to the same results
    x = torch.from_numpy(np.ascontiguousarray(xyz, np.float32)).to(dev)
    d_ids = torch.from_numpy(lig_ids).to(dev)
    chosen = ctx.lbfgs_autotune_dev(p, n, maxN, d_ids.data_ptr(), x.data_ptr(), tors.data_ptr(), sample=256,
                                    probe_iters=10)
    assert sorted(chosen) == [32, 64, 96] and all(v & 255 in (0, 3, 4, 5, 6) and v >> 8 in (0, 1) for v in chosen.values())
    assert np.array_equal(x.cpu().numpy(), xyz)
    tuned = run(xyz, lig_ids, maxN)
    if all(v == 5 for v in chosen.values()):  # the default variant: the same launch
        assert np.array_equal(tuned[1], mixed[1])
    else:  # another register budget may round differently; trajectories then part
        assert abs(np.median(tuned[1]) - np.median(mixed[1])) <= 0.01 * abs(np.median(mixed[1])) + 1e-3
    ctx.close()


def test_inplace_host_call_matches_copying_wrapper():
    """Context.lbfgs_inplace (pxd_lbfgs on the caller's arrays, as bench.py's end-to-end leg
    times it) ends where Context.lbfgs (which copies its inputs) ends, bit for bit, and
    leaves the results in the caller's arrays."""
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=400, cube=16.0, cavity=5.0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=5))
    box = model.make_box((0.0, 0.0, 0.0), (12.0, 12.0, 12.0), 0.5)
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)))
    ctx.set_slope(1e6)
    lid = ctx.add_ligand(lig)
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    poses = synth.random_poses(lig, lo, hi, 64, seed=9)
    p = native.lbfgs_params(max_iter=40, history=8)
    ref = ctx.lbfgs(p, lid, poses)
    xyz = np.ascontiguousarray(poses, np.float64).copy()
    tors = np.zeros((64, ctx.n_rotors))
    e, nev, st = np.zeros(64), np.zeros(64, np.int32), np.zeros(64, np.int32)
    ctx.lbfgs_inplace(p, lid, xyz, tors, e, nev, st)
    assert np.array_equal(xyz, ref["xyz"]) and np.array_equal(e, ref["energy"])
    assert np.array_equal(nev, ref["nevals"]) and np.array_equal(st, ref["status"])
    with pytest.raises(ValueError):
        ctx.lbfgs_inplace(p, lid, xyz.astype(np.float32), tors, e, nev, st)
    ctx.close()
