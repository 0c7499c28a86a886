"""The FP64 differentiable empirical score of the port (po_score_diff): its value equals
the port's root_scorer restatement (po_score, itself pinned to the reference engine),
and its analytic adjoint equals central FP64 finite differences.

The score is piecewise smooth: ramps, the LJ clamp and the pair table (linear between
bins 0.03125 A apart) have kinks. Finite differences that straddle a kink measure the
average of the two one-sided slopes, so the coordinate check uses h = 1e-6 (straddles
are then rare: at most one coordinate per pose may miss) and, at h = 1e-4, requires 95 %
of coordinates to agree; the score is linear in every weight and table value, so those
differences are exact at h = 1e-4."""
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import abi, model, synth


@pytest.fixture(scope="module")
def system(golden):
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=700, cube=20.0, cavity=6.0, n_rotors=3))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    pose_sf, _ = model.load_scoring_function(os.path.join(golden, "scoring_function.json"))
    port = O.PortSystem(rec, lig)
    rng = np.random.default_rng(0)
    w = abi.sf_weights(pose_sf) * rng.uniform(0.5, 1.5, size=abi.NUM_SF_WEIGHTS)
    yield dict(rec=rec, lig=lig, sf=pose_sf, port=port, w=w, tab=abi.smooth_pair_tables(1),
               rx=port.receptor_apply(np.array([0.2, -0.4, 1.1])))


def score(s, x, w=None, tab=None):
    return O.port_score_diff(s["sf"], s["rec"], s["lig"], s["rx"], x, s["w"] if w is None else w,
                             s["tab"] if tab is None else tab, grads=False)[0]


def test_features_combine_to_the_port_score(system):
    s = system
    x = s["lig"].poses[0]
    for k in range(3):
        xk = x + np.random.default_rng(k).normal(scale=0.4, size=x.shape)
        v, f = O.port_score_diff(s["sf"], s["rec"], s["lig"], s["rx"], xk, abi.sf_weights(s["sf"]), None,
                                 grads=False)
        ref, _ = s["port"].score(s["sf"], s["rx"], xk)
        assert abs(v - ref) <= 1e-9 * max(1.0, abs(ref)), (v, ref)
        assert f[27] == 0.0
    # the synthetic complex reaches most feature families
    _, f = O.port_score_diff(s["sf"], s["rec"], s["lig"], s["rx"], x, s["w"], s["tab"], grads=False)
    assert np.count_nonzero(f) >= 9 and f[27] != 0.0


def test_coordinate_adjoint_matches_small_step_differences(system):
    s = system
    h = 1e-6
    for k in range(2):
        x = s["lig"].poses[0] + np.random.default_rng(10 + k).normal(scale=0.3, size=s["lig"].poses[0].shape)
        _, _, gx, _, _ = O.port_score_diff(s["sf"], s["rec"], s["lig"], s["rx"], x, s["w"], s["tab"], g=1.0)
        err = []
        for i in range(x.shape[0]):
            for d in range(3):
                xp, xm = x.copy(), x.copy()
                xp[i, d] += h
                xm[i, d] -= h
                fd = (score(s, xp) - score(s, xm)) / (2 * h)
                err.append(abs(fd - gx[i, d]) / max(1.0, abs(fd)))
        err = np.array(err)
        # a step that straddles a kink is rare at h = 1e-6; allow one per pose
        assert np.mean(err <= 1e-6) >= 0.97, np.sort(err)[-5:]
        assert np.sum(err > 1e-4) <= 1, np.sort(err)[-5:]


def test_adjoint_matches_h1e4_differences(system):
    s = system
    h = 1e-4
    x = s["lig"].poses[0] + np.random.default_rng(20).normal(scale=0.3, size=s["lig"].poses[0].shape)
    g = 0.7
    v, _, gx, gw, gt = O.port_score_diff(s["sf"], s["rec"], s["lig"], s["rx"], x, s["w"], s["tab"], g=g)
    ok = 0
    for i in range(x.shape[0]):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[i, d] += h
            xm[i, d] -= h
            fd = g * (score(s, xp) - score(s, xm)) / (2 * h)
            ok += abs(fd - gx[i, d]) <= 1e-4 * max(1.0, abs(fd))
    assert ok >= 0.95 * 3 * x.shape[0]
    for k in range(abi.NUM_SF_WEIGHTS):
        wp, wm = s["w"].copy(), s["w"].copy()
        wp[k] += h
        wm[k] -= h
        fd = g * (score(s, x, w=wp) - score(s, x, w=wm)) / (2 * h)
        assert abs(fd - gw[k]) <= 1e-8 * max(1.0, abs(fd)), (k, fd, gw[k])
    nz = np.flatnonzero(gt)
    assert nz.size > 100
    for k in np.random.default_rng(1).choice(nz, size=24, replace=False):
        tp, tm = s["tab"].reshape(-1).copy(), s["tab"].reshape(-1).copy()
        tp[k] += h
        tm[k] -= h
        fd = g * (score(s, x, tab=tp) - score(s, x, tab=tm)) / (2 * h)
        assert abs(fd - gt[k]) <= 1e-8 * max(1.0, abs(fd)), (k, fd, gt[k])


def test_host_weight_gradient_matches_the_oracle(system):
    """abi.weights_grad (the autograd backward's weight gradient from summed features)
    equals the port's po_combine_grad, on numpy and torch inputs."""
    import ctypes as C
    f = np.random.default_rng(4).normal(size=abi.NUM_SCORE_FEATURES)
    ref = np.zeros(abi.NUM_SF_WEIGHTS)
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    O.port_lib().po_combine_grad(p(system["w"]), p(f), 1.0, p(ref))
    np.testing.assert_allclose(abi.weights_grad(system["w"], f), ref, rtol=1e-14, atol=1e-14)
    torch = pytest.importorskip("torch")
    got = abi.weights_grad(torch.tensor(system["w"]), torch.tensor(f)).numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-14, atol=1e-14)
