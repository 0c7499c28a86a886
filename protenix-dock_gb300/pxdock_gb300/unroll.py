"""Differentiating through pose optimisation: an unrolled L-BFGS over pose DOFs on the
differentiable empirical score, with a loss on the final poses back-propagated to the
scoring parameters (36 weights, 32 x 256 pair tables).

    q_{k+1} = q_k - c_k H_k g_k,   g_k = dE/dq (q_k; w, T),
    q = (centre, quaternion, torsions), E = the empirical score of the pose that the
    torsion tree places from q, H_k the L-BFGS inverse Hessian (the reference's two-loop
    recursion over the last m steps, a pair kept when s.y > 1e-10, gamma = s.y / y.y of
    the newest kept pair; optimizer.cpp:455-500) and c_k = min(1, cap / max|H_k g_k|) in
    place of the strong-Wolfe line search, so that the unrolled map is differentiable.

g_k is a torch.autograd.Function (DofGradient) over the library's kernels: placement
(pxd_ligand_pose_multi_dev), the score adjoint (pxd_score_adjoint_multi_dev) and the pose
backward. Its vector-Jacobian product with an upstream u is second order:
    dL/dq += H_q u  and  dL/dtheta += d(u . g)/dtheta,
taken in forward mode over the adjoint: the kinematics JVP dx = J u
(pxd_ligand_pose_dir_multi_dev), the adjoint run on dual numbers along dx
(pxd_score_hvp_multi_dev: H_x dx and the mixed parameter derivatives), and the
derivative of the pose backward along u (pxd_ligand_pose_dir_multi_dev again), which adds
the kinematics' own curvature. Torch autograd differentiates the rest (two-loop
recursion, step cap, loss), so the gradient is that of the unrolled algorithm itself
(derivatives almost everywhere of the piecewise-smooth score). Segments of `every` steps
run under torch.utils.checkpoint and are recomputed in the backward pass.

The optimiser state (DOFs, history, two-loop dots, step cap) should be FP64: with FP32
state the two-loop products can overflow on steep LJ walls. The kernels take FP32 copies.
The same unroll runs on a CPU FP64 backend (the oracle's port) for the error check.
"""
import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import abi, native


def _p(t):
    return None if t is None else t.data_ptr()


class KernelBackend:
    """Poses of many receptor contexts on the GPU: ctx_ids, lig_ids [P] int32 device
    tensors; xyz_ref [P][A][3] float32 device tensor (each pose's ligand reference
    coordinates); dof = 7 + the largest torsion count."""

    dtype = torch.float32

    def __init__(self, contexts, ctx_ids, lig_ids, xyz_ref, dof, which=0):
        self.ctxs = list(contexts)
        self.ctx_ids, self.lig_ids, self.xyz_ref = ctx_ids, lig_ids, xyz_ref
        self.which, self.D = which, dof
        self.P, self.A = xyz_ref.shape[0], xyz_ref.shape[1]
        self.dev = xyz_ref.device
        self.ones = torch.ones(self.P, dtype=torch.float64, device=self.dev)
        self.evals = 0
        self.launches = 0

    @staticmethod
    def _stream():
        return torch.cuda.current_stream().cuda_stream or 1

    def place(self, q):
        x = torch.empty((self.P, self.A, 3), dtype=torch.float32, device=self.dev)
        native.ligand_pose_multi_dev(self.ctxs, self.P, self.A, self.D, _p(self.ctx_ids), _p(self.lig_ids),
                                     _p(self.xyz_ref), _p(q), _p(x), None, None, self._stream())
        self.launches += 1
        return x

    def place_backward(self, q, x, gx):
        gq = torch.empty_like(q)
        native.ligand_pose_multi_dev(self.ctxs, self.P, self.A, self.D, _p(self.ctx_ids), _p(self.lig_ids), None,
                                     _p(q), _p(x), _p(gx.contiguous()), _p(gq), self._stream())
        self.launches += 1
        return gq

    def grad(self, q, w, t):
        """(dE/dq, x, dE/dx) at q [P][D]."""
        q = q.to(torch.float32).contiguous()
        w, t = w.to(torch.float64).contiguous(), t.to(torch.float32).contiguous()
        x = self.place(q)
        gx = torch.empty_like(x)
        native.score_adjoint_multi_dev(self.ctxs, self.which, self.P, self.A, _p(self.ctx_ids), _p(self.lig_ids),
                                       _p(x), None, _p(w), _p(t), _p(self.ones), None, None, _p(gx), None, None,
                                       self._stream())
        self.launches += 1
        self.evals += self.P
        return self.place_backward(q, x, gx), x, gx

    def hvp(self, q, u, x, gx, w, t):
        """(H_q u, d(u.g)/dw [36], d(u.g)/dT [32*256]) at q. Every product is linear in u,
        so u is divided by its largest row norm N (FP64) before the FP32 kernels and the
        results are multiplied by N in FP64: adjoints that grow over many unrolled steps
        stay within FP32 range inside the kernels. N stays on the device (a 0-d tensor), so
        the backward pass queues its launches without waiting for the GPU."""
        q = q.to(torch.float32).contiguous()
        w, t = w.to(torch.float64).contiguous(), t.to(torch.float32).contiguous()
        N = u.detach().to(torch.float64).norm(dim=1).max()
        N = torch.where(torch.isfinite(N) & (N > 0), N, torch.ones_like(N))
        u = (u.to(torch.float64) / N).to(torch.float32).contiguous()
        xd = torch.empty_like(x)
        native.ligand_pose_dir_multi_dev(self.ctxs, self.P, self.A, self.D, _p(self.ctx_ids), _p(self.lig_ids),
                                         _p(x), _p(q), _p(u), None, None, None, _p(xd), self._stream())
        gxd = torch.empty_like(x)
        dw = torch.zeros(abi.NUM_SF_WEIGHTS, dtype=torch.float64, device=self.dev)
        dt = torch.zeros(abi.PAIR_TYPES * abi.PAIR_BINS, dtype=torch.float64, device=self.dev)
        native.score_hvp_multi_dev(self.ctxs, self.which, self.P, self.A, _p(self.ctx_ids), _p(self.lig_ids), _p(x),
                                   _p(xd), None, _p(w), _p(t), _p(self.ones), None, _p(gxd), _p(dw), _p(dt),
                                   self._stream())
        hu = torch.empty_like(q)
        native.ligand_pose_dir_multi_dev(self.ctxs, self.P, self.A, self.D, _p(self.ctx_ids), _p(self.lig_ids),
                                         _p(x), _p(q), _p(u), _p(xd), _p(gx), _p(gxd), _p(hu), self._stream())
        self.launches += 5
        self.evals += self.P
        return hu.to(torch.float64) * N, dw * N, dt * N


class _DofGradient(torch.autograd.Function):
    @staticmethod
    def forward(fctx, q, w, t, backend):
        g, x, gx = backend.grad(q.detach(), w.detach(), t.detach())
        fctx.save_for_backward(q, w, t, x, gx)
        fctx.backend = backend
        return g.to(q.dtype)

    @staticmethod
    def backward(fctx, u):
        q, w, t, x, gx = fctx.saved_tensors
        hu, dw, dt = fctx.backend.hvp(q.detach(), u.detach(), x, gx, w.detach(), t.detach())
        return hu.to(q.dtype), dw.to(w.dtype), dt.view(t.shape).to(t.dtype), None


class _Place(torch.autograd.Function):
    @staticmethod
    def forward(fctx, q, backend):
        qq = q.detach().to(backend.dtype).contiguous()
        x = backend.place(qq)
        fctx.save_for_backward(qq, x)
        fctx.backend, fctx.qdt = backend, q.dtype
        return x.to(q.dtype)

    @staticmethod
    def backward(fctx, gx):
        q, x = fctx.saved_tensors
        return fctx.backend.place_backward(q, x, gx.detach().to(x.dtype).contiguous()).to(fctx.qdt), None


def place(backend, q):
    """Atom coordinates [P][A][3] of the poses q, differentiable in q."""
    return _Place.apply(q, backend)


def _lbfgs_steps(k0, k1, backend, w, t, cap, q, qp, gp, S, Y, R, M, gamma):
    """Steps k0 .. k1-1 of the unrolled L-BFGS (history slots oldest .. newest)."""
    m = S.shape[0]
    for k in range(k0, k1):
        g = _DofGradient.apply(q, w, t, backend)
        if k > 0:
            s, y = q - qp, g - gp
            sy = (s * y).sum(1)
            keep = sy > 1e-10
            ok = keep.to(q.dtype)
            safe = torch.where(keep, sy, torch.ones_like(sy))
            S = torch.cat([S[1:], s[None]])
            Y = torch.cat([Y[1:], y[None]])
            R = torch.cat([R[1:], (ok / safe)[None]])
            M = torch.cat([M[1:], ok[None]])
            yy = (y * y).sum(1)
            gamma = torch.where(keep, sy / torch.where(yy > 0, yy, torch.ones_like(yy)), gamma)
        r = g
        alpha = [None] * m
        for j in range(m - 1, -1, -1):  # newest first
            alpha[j] = R[j] * (S[j] * r).sum(1)
            r = r - alpha[j][:, None] * Y[j]
        r = r * gamma[:, None]
        for j in range(m):  # oldest first
            beta = R[j] * (Y[j] * r).sum(1)
            r = r + (alpha[j] - beta)[:, None] * S[j]
        dmax = r.abs().max(1).values
        c = torch.clamp(cap / torch.where(dmax > 0, dmax, torch.full_like(dmax, cap)), max=1.0)
        qp, gp = q, g
        q = q - c[:, None] * r
    return q, qp, gp, S, Y, R, M, gamma


class _ClipRows(torch.autograd.Function):
    """Identity whose backward scales every row (last dimension) of the incoming gradient
    down to a Euclidean norm of at most max_norm."""

    @staticmethod
    def forward(fctx, x, max_norm):
        fctx.max_norm = max_norm
        return x.view_as(x)

    @staticmethod
    def backward(fctx, g):
        n = g.norm(dim=-1, keepdim=True)
        return g * torch.clamp(fctx.max_norm / torch.where(n > 0, n, torch.ones_like(n)), max=1.0), None


def lbfgs_unroll(backend, q0, w, t, steps, history=8, cap=0.3, every=10, truncate=None, clip=None):
    """q_K after `steps` unrolled L-BFGS steps from q0 [P][D], differentiable in w, t and
    q0; segments of `every` steps are checkpointed.

    The map q0 -> q_K is chaotic over many steps (the FP32 and FP64 trajectories part, and
    the exact derivative through 50 steps reaches ~1e50), so two bounded alternatives to the
    exact gradient are offered:
      truncate=T  backpropagates through the last T steps only: the optimiser state after
                  step steps - T enters as a constant (truncated backpropagation through
                  time); q0 then gets no gradient for T < steps;
      clip=c      at every segment boundary scales each pose's row of the state's incoming
                  gradient to a norm of at most c.
    Both leave the forward pass (q_K, the loss) unchanged; by default the gradient is exact."""
    P, D = q0.shape
    z = torch.zeros((history, P, D), dtype=q0.dtype, device=q0.device)
    state = (q0, torch.zeros_like(q0), torch.zeros_like(q0), z, z.clone(),
             torch.zeros((history, P), dtype=q0.dtype, device=q0.device),
             torch.zeros((history, P), dtype=q0.dtype, device=q0.device),
             torch.ones(P, dtype=q0.dtype, device=q0.device))
    cut = None if truncate is None else max(0, steps - int(truncate))
    bounds = sorted(set(list(range(0, steps, every)) + ([cut] if cut is not None and cut < steps else [])))
    for i, k0 in enumerate(bounds):
        k1 = bounds[i + 1] if i + 1 < len(bounds) else steps
        if k0 == cut:
            state = tuple(s.detach() for s in state)
        elif clip is not None and k0 > 0:
            state = tuple(_ClipRows.apply(s, clip) if s.requires_grad and s.dim() >= 2 else s for s in state)
        state = checkpoint(_lbfgs_steps, k0, k1, backend, w, t, cap, *state, use_reentrant=False)
    return state[0]


def rmsd_loss(x, target, n_atoms):
    """Mean over poses of the RMSD between x and target [P][A][3] over each pose's first
    n_atoms[p] atoms."""
    mask = (torch.arange(x.shape[1], device=x.device)[None, :] < n_atoms[:, None]).to(x.dtype)
    d2 = ((x - target) ** 2).sum(-1) * mask
    return torch.sqrt(d2.sum(1) / n_atoms.to(x.dtype)).mean()


def random_dofs(rng, n_tors, D, centre_scale=3.0, tors_scale=np.pi):
    """Seeded DOF rows [P][D]: centre in a cube, uniform quaternion, torsions uniform."""
    P = len(n_tors)
    q = np.zeros((P, D))
    q[:, :3] = rng.uniform(-centre_scale, centre_scale, size=(P, 3))
    qu = rng.normal(size=(P, 4))
    q[:, 3:7] = qu / np.linalg.norm(qu, axis=1, keepdims=True)
    for p in range(P):
        q[p, 7:7 + n_tors[p]] = rng.uniform(-tors_scale, tors_scale, size=n_tors[p])
    return q
