"""The batched optimiser at its full workload size: 65,536 random poses of the 42-atom,
5-torsion ligand in a 30 A box at 0.375 A (81^3 maps over a 1,500-heavy-atom pocket),
m = 8, max_iter = 300, tol_grad = 1e-3, all in one persistent launch. At this size the
FP64 optimiser cannot follow every pose, so the batch is checked through properties that
do not depend on its size:

- determinism: the same batch twice ends bit for bit the same;
- independence: the batch in reverse order ends, pose by pose, bit for bit the same (a
  pose's result does not depend on its neighbours, its place in the queue or its warp);
- every pose ends converged or at the iteration cap with a finite energy, but for at most
  1e-4 of them that stop on a NaN loss (the reference's status for it, optimizer.cpp:532):
  from one start of the 65,536 the FP32 trajectory is flung ~1e11 A out of the box along the
  1e6 kcal/mol/A penalty slope until a trial point leaves the FP32 range (the FP64
  optimiser from the same start converges); no bad input;
- the batch goes downhill: the median energy falls, and nine in ten poses end no higher
  than they started. Not all of them: like the reference (optimizer.cpp:258-263), the line
  search accepts its first trial step outright when the directional derivative there
  exceeds 1e5 in magnitude, which clash poses (start energies up to 1e16) do;
- the reported energy is the FP64 objective at the returned pose (the oracle, with its maps
  built in FP64) within 1e-3 kcal/mol + 1e-9 relative, for 128 poses: the 32 lowest, 32
  drawn from those below 100 kcal/mol, 32 drawn from the strained poses between 100 and
  1e4 kcal/mol and the 32 highest (clashes up to ~1e9 kcal/mol). The optimiser reports
  the FP64 evaluation of its final pose (energy64.cuh), over map energies kept in FP64
  beside the FP32 records.
"""
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import model, native, synth

pytestmark = pytest.mark.gpu

N_POSES = 65536


def test_full_size_batch_properties():
    import torch

    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (30.0, 30.0, 30.0), 0.375)
    assert list(box.npoints) == [81, 81, 81] and lig.n_atoms == 42
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    poses = synth.random_poses(lig, lo, hi, N_POSES, seed=2).astype(np.float32)
    types = sorted(set(int(t) for t in lig.vdw_type))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, types)
    ctx.set_slope(1e6)
    lid = ctx.add_ligand(lig)
    N = lig.n_atoms
    dev = torch.device("cuda:0")
    p = native.lbfgs_params(max_iter=300, history=8, tolerance_grad=1e-3)
    tors = torch.zeros(1, device=dev)

    def run(xyz):
        x = torch.from_numpy(np.ascontiguousarray(xyz)).to(dev)
        ids = torch.full((N_POSES,), lid, dtype=torch.int32, device=dev)
        e = torch.zeros(N_POSES, dtype=torch.float64, device=dev)
        nev = torch.zeros(N_POSES, dtype=torch.int32, device=dev)
        st = torch.full((N_POSES,), -1, dtype=torch.int32, device=dev)
        ctx.lbfgs_dev(p, N_POSES, N, ids.data_ptr(), x.data_ptr(), tors.data_ptr(), e.data_ptr(),
                      nev.data_ptr(), st.data_ptr())
        torch.cuda.synchronize()
        return x.cpu().numpy(), e.cpu().numpy(), nev.cpu().numpy(), st.cpu().numpy()

    first = run(poses)
    again = run(poses)
    for a, b in zip(first, again):
        assert np.array_equal(a, b)
    rev = run(poses[::-1])
    for a, b in zip(first, rev):
        assert np.array_equal(a, b[::-1])

    xyz, energy, nevals, status = first
    # converged or at the cap; a NaN stop (the reference's own outcome, optimizer.cpp:532)
    # is left to at most 1e-4 of the poses: a trajectory that the 1e6 out-of-box slope flings
    # beyond the FP32 range. Its reported energy is that of its last accepted pose.
    assert set(np.unique(status)) <= {0, 1, 2}
    assert np.sum(status == 2) <= 1e-4 * N_POSES
    assert np.all(np.isfinite(energy)) and np.all(nevals > 0)
    e_start, _, _ = ctx.score_grad(lid, poses.astype(np.float64))
    assert np.median(energy) < np.median(e_start)
    assert np.mean(energy <= e_start + 1e-3 + 1e-6 * np.abs(e_start)) >= 0.9

    port = O.PortSystem(rec, lig)
    port.build_grid(box, types, nthreads=os.cpu_count() or 1)
    port.set_slope(1e6)
    rng = np.random.default_rng(3)
    low = np.where(energy < 100.0)[0]
    strained = np.where((energy >= 100.0) & (energy < 1e4))[0]
    assert len(low) >= 32 and len(strained) >= 32, (len(low), len(strained))
    checks = [np.argsort(energy)[:32], rng.choice(low, 32, replace=False),
              rng.choice(strained, 32, replace=False), np.argsort(energy)[-32:]]
    for rows in checks:
        for i in rows:
            e_ref, _, _ = port.score_grad([], xyz[i].astype(np.float64))
            assert abs(energy[i] - e_ref) <= 1e-3 + 1e-9 * abs(e_ref), (i, energy[i], e_ref)
    port.close()
    ctx.close()
