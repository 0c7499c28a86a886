"""The unrolled L-BFGS and its gradient (pxdock_gb300.unroll, shared by the GPU and the
FP64 host backend of oracle/unroll_ref.py): on the FP64 backend, the gradient of the
unrolled loss with respect to weights and table bins agrees with central FP64
differences of the loss itself, with and without an active step cap, over several steps.

The unrolled loss is piecewise smooth in the parameters: a parameter change moves the
trajectory, and so the pair distances, across pair-table bin edges and ramp ends.
Over several steps these kinks are dense (differences at h = 1e-5 .. 1e-7 straddle them),
so the differences use h = 1e-8, where the loss (~4) still has ~1e-8 relative FP64
resolution."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import unroll_ref as U  # noqa: E402
from pxdock_gb300 import abi, model, synth  # noqa: E402
from pxdock_gb300 import unroll as UN  # noqa: E402


@pytest.mark.parametrize("steps,cap", [(1, 0.3), (3, 0.3), (2, 1e9), (5, 0.3)])
def test_unrolled_gradient_matches_differences(golden, steps, cap):
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=500, cube=18.0, cavity=6.0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    sf, _ = model.load_scoring_function(os.path.join(golden, "scoring_function.json"))
    x0 = lig.poses[0] - lig.poses[0].mean(axis=0)
    T = lig.n_torsions
    D = 7 + T
    be = U.PortBackend([U.Pose(rec, lig, sf, x0, D)])
    rng = np.random.default_rng(3)
    q0 = torch.tensor(UN.random_dofs(rng, [T], D, centre_scale=0.6, tors_scale=0.4))
    target = UN.place(be, torch.tensor(UN.random_dofs(rng, [T], D, centre_scale=0.6, tors_scale=0.4))).detach()
    n = torch.full((1,), lig.n_atoms)

    def loss(w, t):
        qK = UN.lbfgs_unroll(be, q0, w, t, steps=steps, history=4, cap=cap, every=2)
        return UN.rmsd_loss(UN.place(be, qK), target, n)

    w = torch.tensor(abi.sf_weights(sf), requires_grad=True)
    t = torch.tensor(abi.smooth_pair_tables(1), requires_grad=True)
    loss(w, t).backward()
    h = 1e-8
    with torch.no_grad():
        for k in (0, 1, 7, 8, 11):
            wp, wm = w.detach().clone(), w.detach().clone()
            wp[k] += h
            wm[k] -= h
            fd = (loss(wp, t.detach()) - loss(wm, t.detach())).item() / (2 * h)
            assert abs(w.grad[k].item() - fd) <= 1e-4 * max(1.0, abs(fd)), (k, w.grad[k].item(), fd)
        nz = torch.nonzero(t.grad.reshape(-1)).reshape(-1)
        for k in nz[:: max(1, len(nz) // 4)][:4].tolist():
            tp, tm = t.detach().clone().reshape(-1), t.detach().clone().reshape(-1)
            tp[k] += h
            tm[k] -= h
            fd = (loss(w.detach(), tp.view(32, 256)) - loss(w.detach(), tm.view(32, 256))).item() / (2 * h)
            assert abs(t.grad.reshape(-1)[k].item() - fd) <= 1e-4 * max(1.0, abs(fd)), (k, fd)


def _setup(golden):
    rec = model.Receptor.from_json(synth.make_receptor(seed=0, n_heavy=500, cube=18.0, cavity=6.0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    sf, _ = model.load_scoring_function(os.path.join(golden, "scoring_function.json"))
    x0 = lig.poses[0] - lig.poses[0].mean(axis=0)
    T = lig.n_torsions
    D = 7 + T
    be = U.PortBackend([U.Pose(rec, lig, sf, x0, D)])
    rng = np.random.default_rng(3)
    q0 = torch.tensor(UN.random_dofs(rng, [T], D, centre_scale=0.6, tors_scale=0.4))
    target = UN.place(be, torch.tensor(UN.random_dofs(rng, [T], D, centre_scale=0.6, tors_scale=0.4))).detach()
    return be, sf, q0, target, torch.full((1,), lig.n_atoms)


def test_truncated_gradient_is_the_gradient_of_the_last_steps(golden):
    """truncate=T: the same loss, and the gradient of the last T steps from the state that
    the first steps reach, held fixed (central differences over the last T steps alone)."""
    be, sf, q0, target, n = _setup(golden)
    steps, T = 4, 2
    w = torch.tensor(abi.sf_weights(sf), requires_grad=True)
    t = torch.tensor(abi.smooth_pair_tables(1))
    full = UN.lbfgs_unroll(be, q0, w.detach(), t, steps=steps, history=4, cap=0.3, every=2)
    qK = UN.lbfgs_unroll(be, q0, w, t, steps=steps, history=4, cap=0.3, every=2, truncate=T)
    assert torch.equal(qK.detach(), full)
    UN.rmsd_loss(UN.place(be, qK), target, n).backward()
    # the state after steps - T as a constant, then the last T steps as a function of w
    import pxdock_gb300.unroll as mod
    with torch.no_grad():
        P, D = q0.shape
        z = torch.zeros((4, P, D), dtype=q0.dtype)
        st0 = (q0, torch.zeros_like(q0), torch.zeros_like(q0), z, z.clone(), torch.zeros((4, P), dtype=q0.dtype),
               torch.zeros((4, P), dtype=q0.dtype), torch.ones(P, dtype=q0.dtype))
        mid = mod._lbfgs_steps(0, steps - T, be, w.detach(), t, 0.3, *st0)

        def tail(wv):
            out = mod._lbfgs_steps(steps - T, steps, be, wv, t, 0.3, *mid)
            return UN.rmsd_loss(UN.place(be, out[0]), target, n)

        assert torch.equal(tail(w.detach()), UN.rmsd_loss(UN.place(be, full), target, n))
        h = 1e-8
        for k in (0, 1, 7, 8):
            wp, wm = w.detach().clone(), w.detach().clone()
            wp[k] += h
            wm[k] -= h
            fd = (tail(wp) - tail(wm)).item() / (2 * h)
            assert abs(w.grad[k].item() - fd) <= 1e-4 * max(1.0, abs(fd)), (k, w.grad[k].item(), fd)


def test_clipped_gradient_is_bounded(golden):
    """clip=c: the forward is unchanged and the gradient reaching q0 has rows of norm at
    most c times the largest single-segment gain (here: below the unclipped one)."""
    be, sf, q0, target, n = _setup(golden)
    w = torch.tensor(abi.sf_weights(sf))
    t = torch.tensor(abi.smooth_pair_tables(1))
    grads = []
    for clip in (None, 1e-3):
        q = q0.clone().requires_grad_(True)
        qK = UN.lbfgs_unroll(be, q, w, t, steps=4, history=4, cap=0.3, every=2, clip=clip)
        UN.rmsd_loss(UN.place(be, qK), target, n).backward()
        grads.append((qK.detach(), q.grad.clone()))
    assert torch.equal(grads[0][0], grads[1][0])
    assert grads[1][1].norm() < grads[0][1].norm()
