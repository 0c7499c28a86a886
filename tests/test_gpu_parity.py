"""GPU parity: the CUDA path through the C ABI against the FP64 port (the oracle).

Tolerances (the parity bar of the path, written here once):
  energy   |dE| <= 1e-3 kcal/mol on physically visited poses (ligand inside the pocket,
           no atom overlaps), relative 1e-6 of |E| elsewhere;
  gradient max|dg| <= 1e-4 * max|g| (relative to the largest component of the pose), and
           |dg_i| <= 1e-3 |g_i| for every component above 1 kcal/mol/A;
  final L-BFGS poses from identical starts: RMSD <= 0.05 A as often as the FP64
           optimiser reproduces itself from FP32-rounded starts (the trajectories are
           chaotic), with the same distribution of final energies;
  integer / index work (nevals, status) exact where trajectories coincide.
"""
import json
import math
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, model, native, synth

pytestmark = pytest.mark.gpu

E_ABS = 1e-3
G_REL = 1e-4
G_COMP = 1e-3  # per component, where |component| > 1 kcal/mol/A


@pytest.fixture(scope="module")
def lib():
    native.load(auto_build=True)
    return native


@pytest.fixture(scope="module")
def complex_small(lib):
    # a pocket the ligand fits in: E(input pose) ~ -90 kcal/mol
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=1000, cube=26.0, cavity=8.5))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (16.0, 16.0, 16.0), 0.375)
    types = sorted(set(int(t) for t in lig.vdw_type))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, types)
    lid = ctx.add_ligand(lig)
    port = O.PortSystem(rec, lig)
    port.build_grid(box, types, nthreads=os.cpu_count() or 1)
    yield dict(rec=rec, lig=lig, box=box, types=types, ctx=ctx, lid=lid, port=port)
    ctx.close()


def near_poses(lig, n, seed, scale=0.15):
    rng = np.random.default_rng(seed)
    return lig.poses[0][None] + rng.normal(scale=scale, size=(n,) + lig.poses[0].shape)


def test_maps_match_oracle(complex_small):
    c = complex_small
    for m in c["types"] + [abi.COULOMB_MAP]:
        gpu = c["ctx"].read_map(m).astype(np.float64)
        ref = c["port"].grid_map(m, c["box"])
        visited = np.abs(ref[:, 0]) < 1e3  # points a ligand atom can occupy
        err = np.max(np.abs(gpu[visited] - ref[visited]), axis=1)
        # FP32 records: error relative to the record's largest component
        scale = np.maximum(1.0, np.max(np.abs(ref[visited]), axis=1))
        assert np.max(err / scale) < 2e-5, (m, np.max(err / scale))
        # where the physics is mild (|E| < 10), the absolute error is tiny
        mild = np.abs(ref[:, 0]) < 10.0
        assert np.max(np.abs(gpu[mild, 0] - ref[mild, 0])) < 1e-4
        # everywhere else the records agree to FP32 relative precision
        hi = ~visited
        if hi.any():
            rel = np.abs(gpu[hi, 0] - ref[hi, 0]) / np.abs(ref[hi, 0])
            assert np.max(rel) < 1e-4


@pytest.mark.parametrize("slope", [0.0, 1e6])
def test_score_grad_grid(complex_small, slope):
    c = complex_small
    c["ctx"].set_slope(slope)
    c["port"].set_slope(slope)
    poses = near_poses(c["lig"], 32, 11)
    e, g, _ = c["ctx"].score_grad(c["lid"], poses)
    worst = 0.0
    for i in range(len(poses)):
        er, _, gr = c["port"].score_grad([], poses[i])
        assert abs(e[i] - er) <= E_ABS, (i, e[i], er)
        assert np.max(np.abs(g[i] - gr)) <= G_REL * np.max(np.abs(gr)), i
        # component by component where the component is at least 1 kcal/mol/A
        big = np.abs(gr) > 1.0
        rel = np.abs(g[i] - gr)[big] / np.abs(gr)[big]
        worst = max(worst, float(rel.max()) if rel.size else 0.0)
        assert np.all(rel <= G_COMP), (i, rel.max())
    print("largest relative error of a gradient component above 1 kcal/mol/A: %.2e" % worst)


def box_penalty(box, slope, x):
    """The out-of-box part of the objective (grid.cpp:211-236): slope * spacing * the
    distance outside the box in grid units, summed over atoms."""
    lo = np.array(box.init_xyz)
    top = np.array(box.npoints, np.float64) - 1
    f = (x - lo) / box.spacing
    out = np.where(f < 0, -f, 0.0) + np.where(f > top, f - top, 0.0)
    return slope * box.spacing * out.sum()


def test_score_grad_out_of_box_penalty(complex_small):
    c = complex_small
    c["ctx"].set_slope(1e6)
    c["port"].set_slope(1e6)
    poses = near_poses(c["lig"], 4, 12) + np.array([9.5, 0.0, -9.0])  # partly outside
    # the call evaluates the FP32-rounded coordinates: on these LJ walls (gradients of
    # 1e12 kcal/mol/A) the rounding alone moves the energy by 1e5, so the oracle gets them too
    poses = poses.astype(np.float32).astype(np.float64)
    e, g, _ = c["ctx"].score_grad(c["lid"], poses)
    for i in range(len(poses)):
        er, _, gr = c["port"].score_grad([], poses[i])
        pen = box_penalty(c["box"], 1e6, poses[i])
        assert pen > 1e6
        # the reported energy is the FP64 evaluation: penalty and the maps read at the
        # clamped boundary (here inside receptor atoms, E ~ 1e11) to FP64 precision
        assert abs(e[i] - er) <= E_ABS + 1e-9 * abs(er), (e[i], er, pen)
        assert np.max(np.abs(g[i] - gr)) <= G_REL * np.max(np.abs(gr))


def test_random_poses_relative(complex_small):
    """Uniform random poses clash with the receptor: energies up to ~1e15 on the steep
    LJ walls. The reported energy is the FP64 evaluation over the maps' FP64 energies,
    within 1e-3 kcal/mol + 1e-9 relative at any size."""
    c = complex_small
    c["ctx"].set_slope(1e6)
    c["port"].set_slope(1e6)
    lo = np.array(c["box"].init_xyz)
    hi = lo + (np.array(c["box"].npoints) - 1) * c["box"].spacing
    poses = synth.random_poses(c["lig"], lo, hi, 32, seed=5).astype(np.float32).astype(np.float64)
    e, g, _ = c["ctx"].score_grad(c["lid"], poses)
    for i in range(len(poses)):
        er, _, gr = c["port"].score_grad([], poses[i])
        assert abs(e[i] - er) <= 1e-9 * abs(er) + E_ABS, (e[i], er)


def test_brute_force_with_receptor_rotors(lib, golden):
    """test_interaction.cpp:280-454 system (3 rotors, no maps) on the GPU."""
    rec = model.Receptor.from_file(os.path.join(golden, "utest_interaction_receptor.json"))
    lig = model.Ligand.from_file(os.path.join(golden, "utest_interaction_ligand.json"))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    lid = ctx.add_ligand(lig)
    x = lig.poses[0][None]
    e, g, tg = ctx.score_grad(lid, x, np.zeros((1, 3)))
    assert abs(e[0] - -24.8695) < 4e-5 + 1e-4
    np.testing.assert_allclose(tg[0], [-1.6258, 0.1114, -0.0144], atol=3e-4)
    t = np.array([[math.radians(i * 120.0) for i in range(3)]])
    e, g, tg = ctx.score_grad(lid, x, t)
    assert abs(e[0] - -25.51645) < 2e-4
    np.testing.assert_allclose(tg[0], [-1.6258, -0.5845, -0.0027], atol=3e-4)
    port = O.PortSystem(rec, lig)
    er, tgr, gr = port.score_grad(t[0], x[0])
    assert abs(e[0] - er) <= E_ABS
    assert np.max(np.abs(g[0] - gr)) <= G_REL * np.max(np.abs(gr))
    assert np.max(np.abs(tg[0] - tgr)) <= G_REL * max(1.0, np.max(np.abs(tgr)))
    ctx.close()


@pytest.mark.parametrize("iters,evals,t0,E,tors,e_tol,t_tol", [
    (1, 8, [0.0, 0.0, 0.0], -65.1168, [1.7078, -0.1169, 0.0151], 1e-3, 2e-3),
    # Stopped after 2 iterations mid-line-search: with FP32 coordinates the search
    # resolves steps to ~2e-6 A at these 25 A positions and takes 18 evaluations
    # where the FP64 reference takes 11 (the FP32 restatement of the reference gives
    # -75.2588 as well); the run stays in the reference's basin.
    (2, 12, [1.0, 2.0, 3.0], -75.4551, [0.3757, 2.6070, 2.9846], 0.25, 0.05),
])
def test_lbfgs_reference_fixtures(lib, golden, iters, evals, t0, E, tors, e_tol, t_tol):
    """test_optimizer.cpp:177-221 on the GPU (reference constants, m = 100)."""
    rec = model.Receptor.from_file(os.path.join(golden, "utest_optimizer_receptor.json"))
    lig = model.Ligand.from_file(os.path.join(golden, "utest_optimizer_ligand.json"))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    lid = ctx.add_ligand(lig)
    p = native.lbfgs_params(max_iter=iters, max_eval=evals)
    out = ctx.lbfgs(p, lid, lig.poses[0][None], np.array([t0]))
    assert abs(out["energy"][0] - E) < e_tol
    np.testing.assert_allclose(out["torsions"][0], tors, atol=t_tol)
    ctx.close()


def rmsd(a, b):
    return float(np.sqrt(np.mean(np.sum((a - b) ** 2, axis=-1))))


@pytest.mark.parametrize("history", [100, 8])
def test_lbfgs_with_receptor_rotors_follows_port(lib, golden, history):
    """The reference engine's own optimize inputs (a pocket with two receptor rotors, three
    clashing starts at 1e6-1e10 kcal/mol), 30 iterations: a descent that FP32 follows
    closely, so every pose ends within 0.01 kcal/mol of the FP64 port with the same
    evaluation count and status. (A racy line-search state once advanced its counter twice
    here and ended pose 2 at -9.6 instead of -18.8 kcal/mol.)"""
    eng = os.path.join(golden, "engine")
    calls = json.load(open(os.path.join(eng, "calls.json")))
    rec = model.Receptor.from_file(os.path.join(eng, "receptor.json"))
    lig = model.Ligand.from_file(os.path.join(eng, "ligand.json"))
    assert rec.n_rotors > 0
    box = model.make_box(calls["box"][:3], calls["box"][3:], calls["spacing"])
    types = sorted(set(int(t) for t in lig.vdw_type))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, types)
    ctx.set_slope(1e6)
    lid = ctx.add_ligand(lig)
    port = O.PortSystem(rec, lig)
    port.build_grid(box, types, nthreads=os.cpu_count() or 1)
    port.set_slope(1e6)
    out = ctx.lbfgs(native.lbfgs_params(max_iter=30, history=history), lid, lig.poses)
    pp = abi.lbfgs_params(max_iter=30, history=history)
    for k in range(len(lig.poses)):
        r = port.lbfgs(pp, np.zeros(rec.n_rotors), lig.poses[k])
        assert abs(out["energy"][k] - r["energy"]) <= 1e-2, (k, out["energy"][k], r["energy"])
        assert out["nevals"][k] == r["nevals"] and out["status"][k] == r["status"], k
    ctx.close()


def test_lbfgs_matches_oracle_trajectories(complex_small):
    """Identical starting poses, GPU against the FP64 optimiser.

    Per pose, the reported energy is the FP64 objective at the returned pose. Per
    trajectory, the flexible ligand's Cartesian L-BFGS is chaotic: the FP64 optimiser
    started from the same poses rounded to FP32 (a 1e-7 relative change) ends within
    0.05 A of its unrounded run for only ~40 % of these starts. So the GPU is held to
    the FP64 optimiser's own reproducibility: as many poses within 0.05 A as that
    control (less a small-sample margin) and the same distribution of final energies.
    """
    c = complex_small
    c["ctx"].set_slope(1e6)
    c["port"].set_slope(1e6)
    poses = near_poses(c["lig"], 48, 21, scale=0.25)
    p = native.lbfgs_params(max_iter=240, history=100)
    out = c["ctx"].lbfgs(p, c["lid"], poses)
    pp = abi.lbfgs_params(max_iter=240, history=100)
    close, close_ctl, energy_ok = 0, 0, 0
    e_gpu, e_ref, e_ctl = [], [], []
    for i in range(len(poses)):
        r = c["port"].lbfgs(pp, [], poses[i])
        ctl = c["port"].lbfgs(pp, [], poses[i].astype(np.float32).astype(np.float64))
        close += rmsd(out["xyz"][i], r["xyz"]) <= 0.05
        close_ctl += rmsd(ctl["xyz"], r["xyz"]) <= 0.05
        # the GPU's final energy is the FP64 objective at the GPU's final pose
        er, _, _ = c["port"].score_grad([], out["xyz"][i])
        energy_ok += abs(out["energy"][i] - er) <= E_ABS
        e_gpu.append(out["energy"][i])
        e_ref.append(r["energy"])
        e_ctl.append(ctl["energy"])
    assert energy_ok == len(poses)
    print("within 0.05 A: gpu %d, fp64 control %d of %d" % (close, close_ctl, len(poses)))
    assert close >= close_ctl - 8, (close, close_ctl)
    # final-energy distributions: medians and quartiles agree as well as the control's
    q_gpu, q_ref, q_ctl = (np.percentile(e, [25, 50, 75]) for e in (e_gpu, e_ref, e_ctl))
    assert np.all(np.abs(q_gpu - q_ref) <= np.abs(q_ctl - q_ref) + 1.0), (q_gpu, q_ref, q_ctl)


def test_lbfgs_batch_uneven_ligands(lib):
    """Several ligands of different sizes in one persistent launch."""
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=500, cube=18.0, cavity=6.0))
    ligs = [model.Ligand.from_json(synth.make_ligand(seed=s, n_heavy=h, n_rot=r, n_n=1, n_o=2))
            for s, h, r in ((3, 12, 2), (4, 20, 4), (5, 30, 6))]
    box = model.make_box((0.0, 0.0, 0.0), (12.0, 12.0, 12.0), 0.5)
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box)
    ctx.set_slope(1e6)
    ids = [ctx.add_ligand(l) for l in ligs]
    maxN = max(l.n_atoms for l in ligs)
    import torch

    dev = torch.device("cuda:0")
    per = 16
    n = per * len(ligs)
    xyz = np.zeros((n, maxN, 3), np.float32)
    lig_ids = np.zeros(n, np.int32)
    for k, (l, i) in enumerate(zip(ligs, ids)):
        for j in range(per):
            xyz[k * per + j, : l.n_atoms] = l.poses[0] + np.random.default_rng(j).normal(scale=0.1, size=l.poses[0].shape)
            lig_ids[k * per + j] = i
    d_xyz = torch.from_numpy(xyz).to(dev)
    d_ids = torch.from_numpy(lig_ids).to(dev)
    d_t = torch.zeros(1, device=dev)
    d_e = torch.zeros(n, dtype=torch.float64, device=dev)
    d_n = torch.zeros(n, dtype=torch.int32, device=dev)
    d_s = torch.zeros(n, dtype=torch.int32, device=dev)
    p = native.lbfgs_params(max_iter=100, history=8)
    torch.cuda.synchronize()
    ctx.lbfgs_dev(p, n, maxN, d_ids.data_ptr(), d_xyz.data_ptr(), d_t.data_ptr(), d_e.data_ptr(),
                  d_n.data_ptr(), d_s.data_ptr(), ctx.stream)
    torch.cuda.synchronize()
    out_xyz = d_xyz.cpu().numpy().astype(np.float64)
    e = d_e.cpu().numpy()
    # each pose equals the single-ligand run of the same start
    for k, (l, i) in enumerate(zip(ligs, ids)):
        single = ctx.lbfgs(p, i, xyz[k * per:(k + 1) * per, : l.n_atoms].astype(np.float64))
        np.testing.assert_allclose(e[k * per:(k + 1) * per], single["energy"], rtol=1e-9, atol=1e-6)
        np.testing.assert_allclose(out_xyz[k * per:(k + 1) * per, : l.n_atoms], single["xyz"], atol=1e-5)
    ctx.close()


def test_bad_ligand_id_and_empty_batch(lib):
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=200, cube=14.0, cavity=4.0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    lid = ctx.add_ligand(lig)
    import torch

    dev = torch.device("cuda:0")
    N = lig.n_atoms
    d_xyz = torch.from_numpy(np.tile(lig.poses[0].astype(np.float32), (2, 1, 1))).to(dev)
    d_ids = torch.tensor([lid, 7], dtype=torch.int32, device=dev)
    d_t = torch.zeros(1, device=dev)
    d_e = torch.zeros(2, dtype=torch.float64, device=dev)
    d_n = torch.zeros(2, dtype=torch.int32, device=dev)
    d_s = torch.zeros(2, dtype=torch.int32, device=dev)
    p = native.lbfgs_params(max_iter=5, history=4)
    ctx.lbfgs_dev(p, 2, N, d_ids.data_ptr(), d_xyz.data_ptr(), d_t.data_ptr(), d_e.data_ptr(),
                  d_n.data_ptr(), d_s.data_ptr(), ctx.stream)
    torch.cuda.synchronize()
    assert int(d_s[1]) == abi.POSE_BAD_INPUT and int(d_n[1]) == 0
    assert int(d_n[0]) > 0
    ctx.lbfgs_dev(p, 0, N, d_ids.data_ptr(), d_xyz.data_ptr(), d_t.data_ptr(), d_e.data_ptr(),
                  d_n.data_ptr(), d_s.data_ptr(), ctx.stream)
    with pytest.raises(native.NativeError):
        ctx.lbfgs_dev(p, 2, 0, d_ids.data_ptr(), d_xyz.data_ptr(), d_t.data_ptr(), d_e.data_ptr(),
                      d_n.data_ptr(), d_s.data_ptr(), ctx.stream)
    # maps missing a registered ligand's type are refused and dropped
    box = model.make_box((0.0, 0.0, 0.0), (8.0, 8.0, 8.0), 1.0)
    with pytest.raises(native.NativeError):
        ctx.build_grid(box, [int(lig.vdw_type[0])])
    # a ligand type without a map is refused once maps exist
    ctx.clear_ligands()
    ctx.build_grid(box, [int(lig.vdw_type[0])])
    with pytest.raises(native.NativeError):
        ctx.add_ligand(lig)
    ctx.close()


def test_kinematics_match_oracle(lib, golden):
    rec = model.Receptor.from_file(os.path.join(golden, "utest_conformer_receptor.json"))
    lig = model.Ligand.from_file(os.path.join(golden, "utest_conformer_ligand.json"))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    lid = ctx.add_ligand(lig)
    port = O.PortSystem(rec, lig)
    rng = np.random.default_rng(2)
    n = 16
    q = synth.random_quaternions(rng, n)
    R = synth.quaternion_matrix(q)
    C = rng.normal(size=(n, 3)) * 5
    T = rng.uniform(-math.pi, math.pi, size=(n, lig.n_torsions))
    out = ctx.ligand_kinematics(lid, lig.poses[0], C, R, T)
    for i in range(n):
        ref = port.ligand_apply(lig.poses[0], C[i], R[i], T[i])
        assert np.max(np.abs(out[i] - ref)) < 2e-5
    t = rng.uniform(-3, 3, size=(4, 3))
    outr = ctx.receptor_kinematics(t)
    for i in range(4):
        assert np.max(np.abs(outr[i] - port.receptor_apply(t[i]))) < 2e-5
    ctx.close()
