"""Optimiser outcomes at the headline configuration: GPU against the FP64 optimiser.

Configuration (the bench's workload): the seeded 1,500-heavy-atom pocket, the
24-heavy-atom / 5-torsion ligand (42 atoms with H), a 30 A box at 0.375 A (81^3 maps),
random starts (centre uniform in the box, uniform orientation, torsions U[-pi, pi)),
L-BFGS with m = 8, at most 300 iterations, tolerance_grad 1e-3, out-of-box slope 1e6,
on the first 2,048 of the bench's 65,536 starts (seed 2). The FP64 optimiser is the port
of lbfgs_step::apply (optimizer.cpp:429-560), pinned to the reference engine.

From random starts the flexible ligand's Cartesian L-BFGS is chaotic: the FP64 optimiser
started from the same poses rounded to FP32 (the control, a 1e-7 relative change) ends
within 0.05 A of its own unrounded run for only ~30 % of them, and its final-energy
quartiles move by up to ~12 % (most starts overlap the pocket or leave the box, so final
energies reach 1e5 kcal/mol). The GPU optimises in FP32 from the FP32-rounded starts
(the host call narrows the caller's FP64 coordinates), and is held to the control's
reproducibility:

- per pose, the reported energy is the FP64 objective at the returned pose, for 64
  poses (1e-3 kcal/mol + 1e-6 relative, + 4e-6 relative above 100 kcal/mol where the
  FP32 map values set the error);
- poses within 0.05 A of the FP64 run: at least the control's fraction less 8 points;
- evaluations per pose: mean within 3 % of the FP64 run's;
- converged fraction within 3 points of the FP64 run's;
- final-energy quartiles: off the FP64 run's by at most three times the control's
  offset or 2 % of the quartile, whichever is larger.
"""
import json

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, model, native, synth

pytestmark = pytest.mark.gpu

N_POSES = 2048


@pytest.fixture(scope="module")
def headline():
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (30.0, 30.0, 30.0), 0.375)
    assert list(box.npoints) == [81, 81, 81] and lig.n_atoms == 42
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    poses = synth.random_poses(lig, lo, hi, N_POSES, seed=2)
    types = sorted(set(int(t) for t in lig.vdw_type))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, types)
    ctx.set_slope(1e6)
    lid = ctx.add_ligand(lig)
    p = native.lbfgs_params(max_iter=300, history=8, tolerance_grad=1e-3)
    gpu = ctx.lbfgs(p, lid, poses)
    ctx.close()
    port = O.PortSystem(rec, lig)
    port.build_grid(box, types, nthreads=host_threads())
    port.set_slope(1e6)
    pp = abi.lbfgs_params(max_iter=300, history=8, tolerance_grad=1e-3)
    none = np.zeros((N_POSES, 0))
    ref = port.lbfgs_batch(pp, none, poses, host_threads())
    ctl = port.lbfgs_batch(pp, none, poses.astype(np.float32).astype(np.float64), host_threads())
    return port, gpu, ref, ctl


def host_threads():
    import os

    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def test_reported_energy_is_the_fp64_objective(headline):
    port, gpu, _, _ = headline
    rng = np.random.default_rng(0)
    for i in rng.choice(N_POSES, 64, replace=False):
        e, _, _ = port.score_grad([], gpu["xyz"][i])
        rel = 1e-6 if abs(e) < 100.0 else 4e-6
        assert abs(gpu["energy"][i] - e) <= 1e-3 + rel * abs(e), (i, gpu["energy"][i], e)


def test_outcomes_match_the_fp64_optimiser(headline):
    _, gpu, ref, ctl = headline
    g = O.compare_outcomes(gpu, ref)
    c = O.compare_outcomes(ctl, ref)
    print(json.dumps({"gpu_vs_fp64": g, "control_vs_fp64": c}))
    assert g["run"]["status"]["nan"] == 0 and g["run"]["status"]["bad_input"] == 0
    assert g["within_rmsd"] >= c["within_rmsd"] - 0.08, (g["within_rmsd"], c["within_rmsd"])
    e_gpu, e_ref = g["run"]["evals_per_pose"], g["ref"]["evals_per_pose"]
    assert abs(e_gpu - e_ref) <= 0.03 * e_ref, (e_gpu, e_ref)
    conv = lambda s: s["status"]["converged"] / N_POSES  # noqa: E731
    assert abs(conv(g["run"]) - conv(g["ref"])) <= 0.03, (g["run"]["status"], g["ref"]["status"])
    q_gpu, q_ref, q_ctl = (np.array(x) for x in (g["run"]["energy_quartiles"], g["ref"]["energy_quartiles"],
                                                   c["run"]["energy_quartiles"]))
    slack = np.maximum(3.0 * np.abs(q_ctl - q_ref), 0.02 * np.abs(q_ref))
    assert np.all(np.abs(q_gpu - q_ref) <= slack), (q_gpu, q_ref, q_ctl)
