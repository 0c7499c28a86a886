"""Differentiating through unrolled L-BFGS (pxdock_gb300.unroll) on the GPU against the
same unroll on the FP64 CPU backend (oracle/unroll_ref.py, whose gradient is pinned to
central differences of the unrolled loss in test_oracle_unroll.py).

Tolerances: the DOF-space Hessian-vector products (kinematics JVP, adjoint on dual
numbers, derivative of the pose backward) within 1e-3 of the pose's largest component,
leaving out components whose FP64 difference quotient changes between steps 1e-6 and
2.5e-7 (a kink inside the step); the gradient of the unrolled loss with respect to the 36
weights and the 32 x 256 tables within 2e-2 of the largest entry (FP32 trajectories of 5
steps against FP64)."""
import os

import numpy as np
import pytest

import oracle as O
import unroll_ref as U
from pxdock_gb300 import abi, model, native, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def two(golden):
    from pxdock_gb300 import unroll as UN
    native.load(auto_build=True)
    sf, _ = model.load_scoring_function(os.path.join(golden, "scoring_function.json"))
    systems = [(model.Receptor.from_json(synth.make_receptor(seed=s, n_heavy=500, cube=18.0, cavity=6.0)),
                model.Ligand.from_json(synth.make_ligand(seed=l, n_heavy=h, n_rot=r)))
               for s, l, h, r in ((0, 1, 24, 5), (5, 7, 18, 3))]
    ctxs = []
    for rec, lig in systems:
        c = native.Context(0)
        c.set_receptor(rec)
        c.set_scoring_function(0, sf)
        c.add_ligand(lig)
        ctxs.append(c)
    P_each = 3
    order = np.repeat([0, 1], P_each)
    A = max(l.n_atoms for _, l in systems)
    D = 7 + max(l.n_torsions for _, l in systems)
    dev = torch.device("cuda", 0)
    ref = np.zeros((len(order), A, 3))
    for p, c in enumerate(order):
        x0 = systems[c][1].poses[0]
        ref[p, : len(x0)] = x0 - x0.mean(axis=0)
    rng = np.random.default_rng(3)
    nt = [systems[c][1].n_torsions for c in order]
    q0 = UN.random_dofs(rng, nt, D, centre_scale=0.6, tors_scale=0.4)
    qt = UN.random_dofs(rng, nt, D, centre_scale=0.6, tors_scale=0.4)
    gpu = UN.KernelBackend(ctxs, torch.tensor(order.astype(np.int32), device=dev),
                           torch.zeros(len(order), dtype=torch.int32, device=dev),
                           torch.tensor(ref, dtype=torch.float32, device=dev), D)
    cpu = U.PortBackend([U.Pose(systems[c][0], systems[c][1], sf, ref[p, : systems[c][1].n_atoms], D)
                         for p, c in enumerate(order)])
    yield dict(gpu=gpu, cpu=cpu, q0=q0, qt=qt, sf=sf, order=order, systems=systems, D=D, dev=dev,
               n_atoms=np.array([systems[c][1].n_atoms for c in order]))
    for c in ctxs:
        c.close()


def test_dof_hessian_vector_products(two):
    gpu, cpu, dev = two["gpu"], two["cpu"], two["dev"]
    w = abi.sf_weights(two["sf"])
    tab = abi.smooth_pair_tables(1)
    q = two["q0"]
    u = np.random.default_rng(9).normal(size=q.shape)
    for p, c in enumerate(two["order"]):
        u[p, 7 + two["systems"][c][1].n_torsions:] = 0.0
    qg = torch.tensor(q, dtype=torch.float32, device=dev)
    wg, tg = torch.tensor(w, device=dev), torch.tensor(tab, dtype=torch.float32, device=dev)
    g, x, gx = gpu.grad(qg, wg, tg)
    hu, dw, dt = gpu.hvp(qg, torch.tensor(u, dtype=torch.float32, device=dev), x, gx, wg, tg)
    hu = hu.cpu().numpy()
    ref = [cpu.poses[p].hvp(q[p], u[p], w, tab.reshape(-1), eps=1e-6) for p in range(len(q))]
    ref4 = [cpu.poses[p].hvp(q[p], u[p], w, tab.reshape(-1), eps=2.5e-7) for p in range(len(q))]
    checked = total = 0
    for p in range(len(q)):
        scale = max(np.max(np.abs(ref[p][0])), 1e-6)
        smooth = np.abs(ref[p][0] - ref4[p][0]) <= 1e-4 * scale
        total += smooth.size
        checked += smooth.sum()
        assert np.max(np.abs(hu[p] - ref[p][0])[smooth]) <= 1e-3 * scale, (p, hu[p], ref[p][0])
    assert checked >= 0.9 * total
    rw = np.sum([r[1] for r in ref], axis=0)
    np.testing.assert_allclose(dw.cpu().numpy(), rw, rtol=1e-2, atol=1e-3 * np.max(np.abs(rw)))


def test_unrolled_gradient_matches_fp64(two):
    from pxdock_gb300 import unroll as UN
    gpu, cpu, dev = two["gpu"], two["cpu"], two["dev"]
    K, hist, cap = 5, 4, 0.3
    out = {}
    for name, be, dt_ in (("gpu", gpu, torch.float64), ("cpu", cpu, torch.float64)):
        d = dev if name == "gpu" else torch.device("cpu")
        w = torch.tensor(abi.sf_weights(two["sf"]), dtype=torch.float64, device=d, requires_grad=True)
        t = torch.tensor(abi.smooth_pair_tables(1), dtype=torch.float64, device=d, requires_grad=True)
        q0 = torch.tensor(two["q0"], dtype=dt_, device=d)
        target = UN.place(be, torch.tensor(two["qt"], dtype=dt_, device=d)).detach()
        qK = UN.lbfgs_unroll(be, q0, w, t, steps=K, history=hist, cap=cap, every=2)
        loss = UN.rmsd_loss(UN.place(be, qK).to(dt_), target.to(dt_), torch.tensor(two["n_atoms"], device=d))
        loss.backward()
        out[name] = (loss.item(), w.grad.cpu().numpy(), t.grad.cpu().numpy().reshape(-1))
    (lg, wg, tg), (lc, wc, tc) = out["gpu"], out["cpu"]
    assert abs(lg - lc) <= 1e-3 * abs(lc)
    np.testing.assert_allclose(wg, wc, rtol=2e-2, atol=2e-2 * np.max(np.abs(wc)))
    np.testing.assert_allclose(tg, tc, rtol=2e-2, atol=2e-2 * np.max(np.abs(tc)))
