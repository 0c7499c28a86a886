"""Backward torsion-tree kinematics (pxd_ligand_backward) against FP64 central finite
differences through the port's forward kinematics (free_ligand::apply_parameters,
data.cpp:592-641): gradients with respect to the centre, a left rotation of the root
orientation and every torsion. The reference has no backward pass; finite differences
are the oracle. Tolerance: 1e-4 of the largest component (FP32 on the GPU)."""
import os

import numpy as np
import pytest

import oracle as O
from pxdock_gb300 import model, native, synth

pytestmark = pytest.mark.gpu

H = 1e-5


def rot(axis, ang):
    a = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K


@pytest.fixture(scope="module")
def kin():
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=1000, cube=26.0, cavity=8.5))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (16.0, 16.0, 16.0), 0.375)
    types = sorted(set(int(t) for t in lig.vdw_type))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, types)
    ctx.set_slope(1e6)
    lid = ctx.add_ligand(lig)
    port = O.PortSystem(rec, lig)
    port.build_grid(box, types, nthreads=os.cpu_count() or 1)
    port.set_slope(1e6)
    yield dict(ctx=ctx, lid=lid, port=port, lig=lig)
    ctx.close()


def params(k, T):
    rng = np.random.default_rng(40 + k)
    c = rng.uniform(-1.0, 1.0, 3)
    R = rot(rng.normal(size=3), rng.uniform(-np.pi, np.pi))
    t = rng.uniform(-np.pi, np.pi, T)
    return c, R, t


def fd(energy, c, R, t):
    """Central differences of energy(c, R, t) in centre, left rotation and torsions."""
    gc, gw, gt = np.zeros(3), np.zeros(3), np.zeros(len(t))
    for d in range(3):
        e = np.eye(3)[d]
        gc[d] = (energy(c + H * e, R, t) - energy(c - H * e, R, t)) / (2 * H)
        gw[d] = (energy(c, rot(e, H) @ R, t) - energy(c, rot(e, -H) @ R, t)) / (2 * H)
    for k in range(len(t)):
        e = np.eye(len(t))[k]
        gt[k] = (energy(c, R, t + H * e) - energy(c, R, t - H * e)) / (2 * H)
    return gc, gw, gt


def check(got, want):
    for a, b in zip(got, want):
        scale = max(1e-6, np.max(np.abs(np.concatenate([np.ravel(w) for w in want]))))
        assert np.max(np.abs(a - b)) <= 1e-4 * scale, (a, b)


def test_linear_energy_matches_finite_differences(kin):
    """E = sum_i w_i . x_i: the backward pass of a fixed dE/dx is exact."""
    lig, port = kin["lig"], kin["port"]
    x0 = lig.poses[0]
    T = lig.n_torsions
    for k in range(4):
        c, R, t = params(k, T)
        w = np.random.default_rng(k).normal(size=x0.shape)
        energy = lambda c_, R_, t_: float(np.sum(w * port.ligand_apply(x0, c_, R_, t_)))
        x = port.ligand_apply(x0, c, R, t)
        gc, gw, gt = kin["ctx"].ligand_backward(kin["lid"], x[None], c[None], w[None])
        check((gc[0], gw[0], gt[0]), fd(energy, c, R, t))


@pytest.fixture(scope="module")
def brute():
    """No maps: the objective's gradient is then the exact derivative of its energy (with
    maps it is the trilinear blend of stored gradients, as in the reference, which
    differs from the derivative of the blended energy by the interpolation error)."""
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=300, cube=18.0, cavity=6.5))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    lid = ctx.add_ligand(lig)
    yield dict(ctx=ctx, lid=lid, port=O.PortSystem(rec, lig), lig=lig)
    ctx.close()


def test_score_torsion_gradients_match_finite_differences(brute):
    """The torsional DOF mode: dE/dx of the objective on the GPU, mapped to rigid-body and
    torsion gradients, against FP64 differences of the objective through the tree."""
    kin = brute
    lig, port = kin["lig"], kin["port"]
    x0 = lig.poses[0]
    c0 = x0.mean(axis=0)
    T = lig.n_torsions
    for k in range(3):
        rng = np.random.default_rng(70 + k)
        c = c0 + rng.normal(scale=0.3, size=3)
        R = rot(rng.normal(size=3), rng.uniform(-0.3, 0.3))
        t = rng.uniform(-0.4, 0.4, T)
        energy = lambda c_, R_, t_: port.score_grad([], port.ligand_apply(x0, c_, R_, t_))[0]
        x = port.ligand_apply(x0, c, R, t)
        _, g, _ = kin["ctx"].score_grad(kin["lid"], x[None])
        gc, gw, gt = kin["ctx"].ligand_backward(kin["lid"], x[None], c[None], g)
        want = fd(energy, c, R, t)
        scale = max(np.max(np.abs(np.concatenate(want))), 1.0)
        for a, b in zip((gc[0], gw[0], gt[0]), want):
            assert np.max(np.abs(a - b)) <= 2e-4 * scale, (a, b)
