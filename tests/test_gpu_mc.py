"""GPU Monte-Carlo search (monte_carlo_searcher, searcher.cpp:46-223) against the FP64
port of the reference walker.

- The device walker generator reproduces mt19937 and the libstdc++ distributions the
  reference draws from: integers and uniform reals bit for bit, orientations to 1e-15
  (CUDA's and glibc's sin/cos may differ in the last ulp).
- A walker's random start (centre, orientation, torsions, the in-box and clash tests)
  equals the port's pose to FP32 coordinate precision (1e-4 A).
- Every reported energy and pose score is the FP64 objective / score at the returned
  pose: |dE| <= 1e-3 kcal/mol, |d pscore| <= 1e-3 + 1e-5 |pscore|.
- Walks themselves are chaotic (so are the port's against the reference's), so the
  populations of best scores are compared, as in the port-versus-reference test.
"""
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, model, native, synth

pytestmark = pytest.mark.gpu

E_ABS = 1e-3


@pytest.fixture(scope="module")
def mc(golden):
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=500, cube=24.0, cavity=8.0,
                                                       n_rotors=3))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (16.0, 16.0, 16.0), 0.5)
    types = sorted(set(int(t) for t in lig.vdw_type))
    pose_sf, aff_sf = model.load_scoring_function(os.path.join(golden, "scoring_function.json"))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, types)
    ctx.set_slope(1e6)
    ctx.set_scoring_function(0, pose_sf)
    lid = ctx.add_ligand(lig)
    port = O.PortSystem(rec, lig)
    port.build_grid(box, types, nthreads=os.cpu_count() or 1)
    port.set_slope(1e6)
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    yield dict(ctx=ctx, lid=lid, port=port, rec=rec, lig=lig, sf=pose_sf, lo=lo, hi=hi)
    ctx.close()


def test_rng_draws_match_reference_generator(mc):
    rng = np.random.default_rng(0)
    kinds = rng.integers(0, 5, size=3000)
    ints = rng.integers(0, 40, size=3000)
    for seed in (0, 7, 123456789):
        dev = mc["ctx"].rng_draws(seed, kinds, ints)
        ref = O.port_rng_draws(seed, kinds, ints)
        assert dev.shape == ref.shape
        o = 0
        for k in kinds:
            w = 3 if k == 3 else 4 if k == 4 else 1
            if k == 4:
                np.testing.assert_allclose(dev[o:o + w], ref[o:o + w], rtol=0, atol=1e-15)
            else:
                assert np.array_equal(dev[o:o + w], ref[o:o + w]), (seed, o, k)
            o += w


@pytest.mark.parametrize("first_pose", [True, False])
def test_random_starts_match_port(mc, first_pose):
    c = mc
    W = 32
    p = native.mc_params(c["lo"], c["hi"], seed=11, max_nsteps=0, full_nsteps=0)
    starts = np.repeat(c["lig"].poses[0][None], W, axis=0)
    out = c["ctx"].mc_search(p, c["lid"], starts, np.arange(1, W + 1), [first_pose] * W)
    same = 0
    for w in range(W):
        ref = c["port"].mc_randomize(c["sf"], c["lo"], c["hi"], 11, w + 1, starts[w], first_pose)
        same += np.max(np.abs(out["xyz"][w] - ref)) < 1e-4
    # a start whose clash test sits within FP32 rounding of the threshold may differ
    assert same >= W - 1, same


def consistent(c, out, w):
    x, t = out["xyz"][w], out["torsions"][w]
    er, _, _ = c["port"].score_grad(t, x)
    assert abs(out["energy"][w] - er) <= E_ABS, (w, out["energy"][w], er)
    ps, _ = c["port"].score(c["sf"], c["port"].receptor_apply(t), x)
    assert abs(out["pscore"][w] - ps) <= 1e-3 + 1e-5 * abs(ps), (w, out["pscore"][w], ps)


def test_walker_zero_relaxes_only(mc):
    c = mc
    p = native.mc_params(c["lo"], c["hi"], seed=7, max_nsteps=12, relax_nsteps=15)
    out = c["ctx"].mc_search(p, c["lid"], c["lig"].poses[0][None], [0])
    assert out["status"][0] == 0
    consistent(c, out, 0)
    ref = c["port"].mc_walker(c["sf"], c["lo"], c["hi"], 7, 0, c["lig"].poses[0], True, 12, 15)
    # one full relaxation of the same start: same basin to within the optimiser's tolerance
    assert abs(out["energy"][0] - ref["energy"]) < 1.0 + 0.01 * abs(ref["energy"])


def test_walker_population_matches_port(mc):
    c = mc
    W = 24
    p = native.mc_params(c["lo"], c["hi"], seed=7, max_nsteps=6, relax_nsteps=15)
    starts = np.repeat(c["lig"].poses[0][None], W, axis=0)
    ids = np.arange(1, W + 1)
    out = c["ctx"].mc_search(p, c["lid"], starts, ids)
    ps_gpu, ps_port, same_class = [], [], 0
    for w in range(W):
        ref = c["port"].mc_walker(c["sf"], c["lo"], c["hi"], 7, int(ids[w]), starts[w], True, 6, 15)
        same_class += (out["status"][w] == 0) == (ref["status"] == 0)
        if out["status"][w] == 0:
            # no box check: a new best is fully relaxed after its in-box test and may
            # leave the box, as in the reference (searcher.cpp:168-172)
            consistent(c, out, w)
            ps_gpu.append(out["pscore"][w])
        if ref["status"] == 0:
            ps_port.append(ref["pscore"])
    assert same_class >= W - 2
    assert len(ps_gpu) >= W // 2
    m_g, m_p = np.median(ps_gpu), np.median(ps_port)
    assert abs(m_g - m_p) < 0.5 + 0.1 * abs(m_p), (m_g, m_p)


def test_pruning_threshold_runs(mc):
    c = mc
    W = 8
    p = native.mc_params(c["lo"], c["hi"], seed=3, max_nsteps=6, relax_nsteps=10,
                         mc_mmenergy_threshold=50.0)
    starts = np.repeat(c["lig"].poses[0][None], W, axis=0)
    out = c["ctx"].mc_search(p, c["lid"], starts, np.arange(W))
    for w in range(W):
        if out["status"][w] == 0:
            consistent(c, out, w)


def test_team_barrier_timeout_is_reported_and_the_context_recovers(mc):
    """Failure detection of team mode without a GPU fault: with PXD_TEST_TEAM_DROPOUT=1 the
    last member of every team leaves before its first barrier, so the other members' waits
    run out (a bounded spin, about 0.1 s), the team stops and the host reports
    PXD_ERR_DEVICE_FLAG. The next launch on the same context runs normally."""
    c = mc
    W = 4  # at most one walker per SM: team mode
    p = native.mc_params(c["lo"], c["hi"], seed=4, max_nsteps=2, relax_nsteps=5)
    starts = np.repeat(c["lig"].poses[0][None], W, axis=0)
    os.environ["PXD_TEST_TEAM_DROPOUT"] = "1"
    try:
        with pytest.raises(native.NativeError, match="stopped waiting") as err:
            c["ctx"].mc_search(p, c["lid"], starts, np.arange(W))
        assert err.value.code == 6  # PXD_ERR_DEVICE_FLAG
    finally:
        del os.environ["PXD_TEST_TEAM_DROPOUT"]
    out = c["ctx"].mc_search(p, c["lid"], starts, np.arange(W))
    assert np.all(out["status"] <= 2) and np.sum(out["status"] == 0) >= 1
    for w in range(W):
        if out["status"][w] == 0:
            consistent(c, out, w)


def test_bad_parameters_rejected(mc):
    c = mc
    p = native.mc_params(c["lo"], c["hi"], temperature=0.0)
    with pytest.raises(native.NativeError):
        c["ctx"].mc_search(p, c["lid"], c["lig"].poses[0][None], [1])
    p = native.mc_params(c["hi"], c["lo"])
    with pytest.raises(native.NativeError):
        c["ctx"].mc_search(p, c["lid"], c["lig"].poses[0][None], [1])


def test_mixed_ligand_launch_matches_single_ligand_launches(golden):
    """Walkers of three ligands of 24, 54 and 81 atoms in one launch of 1,056 walkers
    (per-warp slices sized for the largest) end bit for bit where one launch per ligand
    (slices of its own size) ends."""
    rec = model.Receptor.from_json(synth.make_receptor(seed=2, n_heavy=500, cube=24.0, cavity=8.0))
    ligs = [model.Ligand.from_json(synth.make_ligand(seed=s, n_heavy=h, n_rot=r, n_n=1, n_o=2))
            for s, h, r in ((21, 12, 2), (22, 28, 5), (23, 44, 7))]
    box = model.make_box((0.0, 0.0, 0.0), (16.0, 16.0, 16.0), 0.5)
    types = sorted(set(int(t) for l in ligs for t in l.vdw_type))
    pose_sf, _ = model.load_scoring_function(os.path.join(golden, "scoring_function.json"))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, types)
    ctx.set_slope(1e6)
    ctx.set_scoring_function(0, pose_sf)
    lids = [ctx.add_ligand(l) for l in ligs]
    assert [l.n_atoms <= b for l, b in zip(ligs, (32, 64, 96))] == [True] * 3
    assert ligs[0].n_atoms > 0 and ligs[1].n_atoms > 32 and ligs[2].n_atoms > 64
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    p = native.mc_params(lo, hi, seed=11, max_nsteps=2, relax_nsteps=5, full_nsteps=20)
    per = 352
    maxN = max(l.n_atoms for l in ligs)
    n = per * len(ligs)
    starts = np.zeros((n, maxN, 3))
    ids = np.repeat(np.array(lids, np.int32), per)
    wid = np.tile(np.arange(1, per + 1, dtype=np.int32), len(ligs))
    for k, l in enumerate(ligs):
        starts[k * per:(k + 1) * per, : l.n_atoms] = l.poses[0]
    mixed = ctx.mc_search_multi(p, ids, starts, wid, np.ones(n, np.int32))
    for k, (l, lid) in enumerate(zip(ligs, lids)):
        rows = slice(k * per, (k + 1) * per)
        single = ctx.mc_search(p, lid, starts[rows, : l.n_atoms], wid[rows])
        for key in ("energy", "pscore", "nevals", "status"):
            assert np.array_equal(mixed[key][rows], single[key]), key
        assert np.array_equal(mixed["xyz"][rows, : l.n_atoms], single["xyz"])
        assert np.sum(single["status"] == 0) >= per // 2
    ctx.close()
