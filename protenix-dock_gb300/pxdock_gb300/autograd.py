"""torch.autograd bindings of the differentiable score and the pose kinematics.

Each Function calls the library's hand-written kernels on the current torch stream:

- ``empirical_score(ctx, lig_ids, xyz, weights, tables)``: per-pose empirical score
  S(x; w, T) (pxd_score_adjoint_multi_dev, over one context or several in one launch).
  Forward runs the adjoint kernel once (scores, features, dS/dx, sum_p dS_p/dT); the
  backward scales those by dL/dS, re-running the kernel only for the table gradient
  when the per-pose output weights differ.
- ``ligand_pose(ctx, lig, xyz_ref, centers, quats, torsions)``: torsion-tree forward
  kinematics (pxd_ligand_pose_dev) with its backward (pxd_ligand_pose_backward_dev):
  atom gradients become centre, quaternion and torsion gradients.
- ``ligand_pose_multi(ctxs, ctx_ids, lig_ids, xyz_ref, dofs)``: the same over poses of
  many contexts in one launch (pxd_ligand_pose_multi_dev).
- ``docking_energy(ctx, lig_ids, xyz)``: the docking objective (grid maps + intra-ligand
  force field, pxd_score_grad_dev, or pxd_score_grad_multi_dev over several contexts) with
  its analytic coordinate gradient; it has no parameters.

Torch is only the autograd and memory plumbing here; there is no torch fallback.
"""
import torch

from . import abi, native


def _ptr(t):
    return None if t is None else t.data_ptr()


def _stream():
    """The current torch stream as a CUDA stream handle. torch's default stream has the
    handle 0, which the library reads as "the context's own stream", so it is passed as
    cudaStreamLegacy (1), the same legacy default stream."""
    return torch.cuda.current_stream().cuda_stream or 1


class _EmpiricalScore(torch.autograd.Function):
    """Forward runs the adjoint kernel once with unit output weights: scores, the
    per-pose features, dS/dx and (when the tables need a gradient) sum_p dS_p/dT. The
    backward scales those: dx = g_p dS_p/dx, dw from sum_p g_p features_p, and dT = g_0
    sum_p dS_p/dT when every g_p is equal (the usual summed or averaged score); other g
    re-run the adjoint kernel for dT."""

    @staticmethod
    def forward(fctx, xyz, weights, tables, pctxs, which, ctx_ids, lig_ids, rec_tors):
        P, A, _ = xyz.shape
        dev = xyz.device
        x = xyz.detach().to(torch.float32).contiguous()
        w = weights.detach().to(torch.float64).contiguous()
        t = None if tables is None else tables.detach().to(torch.float32).contiguous()
        score = torch.empty(P, dtype=torch.float64, device=dev)
        need_x, need_w, need_t = fctx.needs_input_grad[0], fctx.needs_input_grad[1], \
            tables is not None and fctx.needs_input_grad[2]
        empty = torch.empty(0, device=dev)
        if need_x or need_w or need_t:
            ones = torch.ones(P, dtype=torch.float64, device=dev)
            feats = torch.empty((P, abi.NUM_SCORE_FEATURES), dtype=torch.float64, device=dev)
            dx = torch.empty_like(x)
            dt = torch.zeros(abi.PAIR_TYPES * abi.PAIR_BINS, dtype=torch.float64, device=dev) if need_t else None
            native.score_adjoint_multi_dev(pctxs, which, P, A, _ptr(ctx_ids), _ptr(lig_ids), _ptr(x), _ptr(rec_tors),
                                           _ptr(w), _ptr(t), _ptr(ones), _ptr(score), _ptr(feats), _ptr(dx), None,
                                           _ptr(dt), _stream())
        else:
            feats = dx = dt = None
            native.score_adjoint_multi_dev(pctxs, which, P, A, _ptr(ctx_ids), _ptr(lig_ids), _ptr(x), _ptr(rec_tors),
                                           _ptr(w), _ptr(t), None, _ptr(score), None, None, None, None, _stream())
        fctx.save_for_backward(x, w, t if t is not None else empty, lig_ids,
                               ctx_ids if ctx_ids is not None else empty, rec_tors if rec_tors is not None else empty,
                               feats if feats is not None else empty, dx if dx is not None else empty,
                               dt if dt is not None else empty)
        fctx.meta = (pctxs, which, tables is not None, xyz.dtype, weights.dtype,
                     None if tables is None else tables.dtype)
        return score

    @staticmethod
    def backward(fctx, grad_score):
        x, w, t, lig_ids, ctx_ids, rec_tors, feats, dx, dt = fctx.saved_tensors
        pctxs, which, has_tab, xdt, wdt, tdt = fctx.meta
        P, A, _ = x.shape
        g = grad_score.detach().to(torch.float64).contiguous()
        gx = gw = gt = None
        if fctx.needs_input_grad[0]:
            gx = (dx * g.to(torch.float32)[:, None, None]).to(xdt)
        if fctx.needs_input_grad[1]:
            gw = abi.weights_grad(w, (feats * g[:, None]).sum(0)).to(wdt)
        if has_tab and fctx.needs_input_grad[2]:
            if bool((g == g[0]).all()):
                gt = (dt * g[0]).view(abi.PAIR_TYPES, abi.PAIR_BINS).to(tdt)
            else:
                d2 = torch.zeros(abi.PAIR_TYPES * abi.PAIR_BINS, dtype=torch.float64, device=x.device)
                scratch = torch.empty_like(x)
                native.score_adjoint_multi_dev(pctxs, which, P, A, _ptr(ctx_ids if ctx_ids.numel() else None),
                                               _ptr(lig_ids), _ptr(x), _ptr(rec_tors if rec_tors.numel() else None),
                                               _ptr(w), _ptr(t), _ptr(g), None, None, _ptr(scratch), None, _ptr(d2),
                                               _stream())
                gt = d2.view(abi.PAIR_TYPES, abi.PAIR_BINS).to(tdt)
        return gx, gw, gt, None, None, None, None, None


def empirical_score(pctx, lig_ids, xyz, weights, tables=None, which=0, rec_tors=None, ctx_ids=None):
    """S per pose [P] (float64) for poses xyz [P][max_atoms][3] of the ligands lig_ids
    [P] (int32, device). pctx is one Context, or a list of Contexts with ctx_ids [P]
    (int32, device) naming each pose's context (one launch over all of them). weights
    [36]; tables [32][256] or None."""
    pctxs = list(pctx) if isinstance(pctx, (list, tuple)) else [pctx]
    if len(pctxs) > 1 and ctx_ids is None:
        raise ValueError("ctx_ids is required with several contexts")
    return _EmpiricalScore.apply(xyz, weights, tables, pctxs, which, ctx_ids if len(pctxs) > 1 else None, lig_ids,
                                 rec_tors)


class _LigandPose(torch.autograd.Function):
    @staticmethod
    def forward(fctx, centers, quats, torsions, pctx, lig, xyz_ref):
        P = centers.shape[0]
        N = xyz_ref.shape[0]
        c = centers.detach().to(torch.float32).contiguous()
        q = quats.detach().to(torch.float32).contiguous()
        tq = torsions.detach().to(torch.float32).contiguous()
        out = torch.empty((P, N, 3), dtype=torch.float32, device=centers.device)
        pctx.ligand_pose_dev(lig, P, _ptr(xyz_ref), _ptr(c), _ptr(q), _ptr(tq) if tq.numel() else None, _ptr(out),
                             _stream())
        fctx.save_for_backward(out, c, q)
        fctx.meta = (pctx, lig, centers.dtype, quats.dtype, torsions.dtype, torsions.shape[1])
        return out

    @staticmethod
    def backward(fctx, grad_xyz):
        out, c, q = fctx.saved_tensors
        pctx, lig, cdt, qdt, tdt, T = fctx.meta
        P = out.shape[0]
        g = grad_xyz.detach().to(torch.float32).contiguous()
        gc = torch.empty((P, 3), dtype=torch.float32, device=out.device)
        gq = torch.empty((P, 4), dtype=torch.float32, device=out.device)
        gt = torch.empty((P, max(T, 1)), dtype=torch.float32, device=out.device)
        pctx.ligand_pose_backward_dev(lig, P, _ptr(out), _ptr(c), _ptr(q), _ptr(g), _ptr(gc), _ptr(gq), _ptr(gt),
                                      _stream())
        return gc.to(cdt), gq.to(qdt), gt[:, :T].to(tdt), None, None, None


def ligand_pose(pctx, lig, xyz_ref, centers, quats, torsions):
    """Atom coordinates [P][N][3] (float32) of ligand lig for centres [P][3], quaternions
    [P][4] (w, x, y, z; normalised inside) and torsions [P][T]; xyz_ref [N][3] float32 on
    the device is the ligand's reference pose."""
    return _LigandPose.apply(centers, quats, torsions, pctx, lig, xyz_ref)


class _DockingEnergy(torch.autograd.Function):
    @staticmethod
    def forward(fctx, xyz, pctxs, ctx_ids, lig_ids, rec_tors):
        P, A, _ = xyz.shape
        x = xyz.detach().to(torch.float32).contiguous()
        e = torch.empty(P, dtype=torch.float64, device=xyz.device)
        g = torch.empty_like(x)
        R = max(c.n_rotors for c in pctxs)
        tg = torch.empty((P, max(R, 1)), dtype=torch.float32, device=xyz.device)
        if ctx_ids is None:
            pctxs[0].score_grad_dev(P, A, _ptr(lig_ids), _ptr(x), _ptr(rec_tors), _ptr(e), _ptr(g), _ptr(tg),
                                    _stream())
        else:
            native.score_grad_multi_dev(pctxs, P, A, _ptr(ctx_ids), _ptr(lig_ids), _ptr(x), _ptr(rec_tors), _ptr(e),
                                        _ptr(g), _ptr(tg), _stream())
        fctx.save_for_backward(g)
        fctx.xdt = xyz.dtype
        return e

    @staticmethod
    def backward(fctx, grad_e):
        (g,) = fctx.saved_tensors
        return (g * grad_e.to(torch.float32)[:, None, None]).to(fctx.xdt), None, None, None, None


def docking_energy(pctx, lig_ids, xyz, rec_tors=None, ctx_ids=None):
    """Docking objective per pose [P] (grid maps + intra-ligand terms) with its gradient;
    pctx is one Context, or a list of Contexts with ctx_ids [P] (one launch)."""
    pctxs = list(pctx) if isinstance(pctx, (list, tuple)) else [pctx]
    if len(pctxs) > 1 and ctx_ids is None:
        raise ValueError("ctx_ids is required with several contexts")
    return _DockingEnergy.apply(xyz, pctxs, ctx_ids if len(pctxs) > 1 else None, lig_ids, rec_tors)


class _LigandPoseMulti(torch.autograd.Function):
    @staticmethod
    def forward(fctx, dofs, pctxs, ctx_ids, lig_ids, xyz_ref):
        P, D = dofs.shape
        A = xyz_ref.shape[1]
        q = dofs.detach().to(torch.float32).contiguous()
        out = torch.empty((P, A, 3), dtype=torch.float32, device=dofs.device)
        native.ligand_pose_multi_dev(pctxs, P, A, D, _ptr(ctx_ids), _ptr(lig_ids), _ptr(xyz_ref), _ptr(q), _ptr(out),
                                     None, None, _stream())
        fctx.save_for_backward(out, q, ctx_ids, lig_ids)
        fctx.meta = (pctxs, dofs.dtype)
        return out

    @staticmethod
    def backward(fctx, grad_xyz):
        out, q, ctx_ids, lig_ids = fctx.saved_tensors
        pctxs, qdt = fctx.meta
        P, D = q.shape
        gq = torch.empty_like(q)
        native.ligand_pose_multi_dev(pctxs, P, out.shape[1], D, _ptr(ctx_ids), _ptr(lig_ids), None, _ptr(q),
                                     _ptr(out), _ptr(grad_xyz.detach().to(torch.float32).contiguous()), _ptr(gq),
                                     _stream())
        return gq.to(qdt), None, None, None, None


def ligand_pose_multi(pctxs, ctx_ids, lig_ids, xyz_ref, dofs):
    """Atom coordinates [P][A][3] of poses of several contexts in one launch: pose p is
    ligand lig_ids[p] of pctxs[ctx_ids[p]], xyz_ref [P][A][3] its reference coordinates,
    dofs [P][D] its centre, quaternion (normalised inside) and torsions (padded to D)."""
    return _LigandPoseMulti.apply(dofs, list(pctxs), ctx_ids, lig_ids, xyz_ref)
