"""The FP64 rigid-body + torsion optimiser of oracle/dof_ref.py, pinned before it checks the
device mode:
  - its L-BFGS + strong-Wolfe restatement, run over the Cartesian closure, reproduces the
    C port's optimiser (pinned against the reference's optimiser fixtures) on short runs;
  - its DOF gradient is the Cartesian gradient pulled back through the placement (whose
    Jacobian is taken by central FP64 differences);
  - a DOF optimisation lowers the energy and keeps every bond length of the input pose.
"""
import os

import numpy as np
import pytest

pytest.importorskip("torch")

import dof_ref as DR  # noqa: E402
import oracle as O  # noqa: E402
from pxdock_gb300 import abi, model, synth  # noqa: E402
from unroll_ref import quat_rot  # noqa: E402


@pytest.fixture(scope="module")
def system():
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=500, cube=18.0, cavity=6.0, n_rotors=3))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    assert rec.n_rotors == 3
    box = model.make_box((0.0, 0.0, 0.0), (12.0, 12.0, 12.0), 0.5)
    port = O.PortSystem(rec, lig)
    port.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)), nthreads=os.cpu_count() or 1)
    port.set_slope(1e6)
    return rec, lig, port


def starts(lig, port, n, seed):
    """Input poses: the ligand's pose turned, moved and twisted (bond geometry kept)."""
    rng = np.random.default_rng(seed)
    x0 = lig.poses[0]
    out = []
    for _ in range(n):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        rot = quat_rot(q)
        tors = rng.normal(scale=0.3, size=lig.n_torsions)
        c = x0.mean(axis=0) + rng.normal(scale=0.5, size=3)
        out.append(port.ligand_apply(x0, c, rot, tors))
    return out


@pytest.mark.parametrize("iters", [1, 3, 8])
def test_restated_lbfgs_reproduces_the_port(system, iters):
    rec, lig, port = system
    R = rec.n_rotors
    N = lig.n_atoms
    p = abi.lbfgs_params(max_iter=iters, history=10)

    def cart(v):
        e, tg, lg = port.score_grad(v[3 * N:], v[:3 * N].reshape(-1, 3))
        return e, np.concatenate([lg.reshape(-1), tg])

    for x in starts(lig, port, 4, 5):
        v0 = np.concatenate([x.reshape(-1), np.zeros(R)])
        v, e, nev, st = DR.lbfgs(cart, v0, DR.params_dict(p))
        ref = port.lbfgs(p, np.zeros(R), x)
        assert nev == ref["nevals"] and st == ref["status"], (nev, ref["nevals"], st, ref["status"])
        np.testing.assert_allclose(v[:3 * N].reshape(-1, 3), ref["xyz"], atol=1e-7)
        ef, _, _ = port.score_grad(v[3 * N:], v[:3 * N].reshape(-1, 3))
        assert abs(ef - ref["energy"]) <= 1e-7 * max(1.0, abs(ef))


def test_dof_gradient_is_the_pulled_back_cartesian_gradient(system):
    """dE/dq = J(q)^T dE/dx with J the Jacobian of the placement, here by central FP64
    differences of the placed coordinates. (The objective's gradient is the interpolated
    map gradient, not the derivative of the interpolated energy, so differences of the
    energy itself are not the reference for it.)"""
    rec, lig, port = system
    R = rec.n_rotors
    for x in starts(lig, port, 3, 7):
        s = DR.DofSystem(port, rec, lig, x)
        q = s.q0()
        rng = np.random.default_rng(1)
        q[:3] += rng.normal(scale=0.1, size=3)
        q[3:7] += rng.normal(scale=0.05, size=4)
        q[7:] += rng.normal(scale=0.1, size=len(q) - 7)
        _, g = s(q)
        _, tg, gx = port.score_grad(q[len(q) - R:], s.place(q))
        h = 1e-6
        n = len(q) - R
        J = np.zeros((3 * lig.n_atoms, n))
        for k in range(n):
            qp, qm = q.copy(), q.copy()
            qp[k] += h
            qm[k] -= h
            J[:, k] = (s.place(qp) - s.place(qm)).reshape(-1) / (2 * h)
        want = J.T @ gx.reshape(-1)
        scale = np.abs(J).T @ np.abs(gx.reshape(-1))
        assert np.all(np.abs(g[:n] - want) <= 1e-7 * np.maximum(1.0, scale)), np.c_[g[:n], want]
        np.testing.assert_array_equal(g[n:], tg)


def test_dof_optimisation_keeps_bonds(system):
    rec, lig, port = system
    p = abi.lbfgs_params(max_iter=60, history=10, dof_mode=abi.DOF_RIGID_TORSION)
    for x in starts(lig, port, 3, 9):
        e0, _, _ = port.score_grad(np.zeros(rec.n_rotors), x)
        xf, ef, nev, st = DR.optimize_dof(port, rec, lig, x, p)
        assert ef < e0 and nev > 1
        # rigid fragments turned about their bonds: every bond length is kept
        b = lig.ff.bonds
        assert len(b) >= lig.n_atoms - 1
        d0 = np.linalg.norm(x[b[:, 0]] - x[b[:, 1]], axis=-1)
        d1 = np.linalg.norm(xf[b[:, 0]] - xf[b[:, 1]], axis=-1)
        np.testing.assert_allclose(d1, d0, atol=1e-9)
