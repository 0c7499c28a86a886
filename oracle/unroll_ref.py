"""TEST INFRASTRUCTURE: FP64 host backend of the unrolled pose optimisation
(pxdock_gb300/unroll.py), on the port's FP64 kinematics (po_ligand_apply,
free_ligand::apply_parameters) and the port's differentiable score (po_score_diff). Only
tests/ and bench.py's CPU-baseline leg use it, as the checker.

The unrolled optimiser (pxdock_gb300.unroll.lbfgs_unroll) is shared with the GPU; this
module supplies its backend in FP64: pose placement and its backward (the formulas of the
GPU pose backward, restated in numpy), the score gradient, and the second-order products
as central differences of the FP64 adjoint along the unit direction (step 1e-8, small
enough that a kink inside the step -- a ramp end, the LJ clamp, a pair-table bin edge --
is rare: a pair crossing a bin edge inside the step would add a spike of its slope change
over 2e-8 to the mixed table derivative)."""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

import oracle as O


def quat_rot(q):
    q = np.asarray(q, float) / np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (a * c + b * d)],
                     [2 * (a * d + b * c), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (a * b + c * d), a * a - b * b - c * c + d * d]])


class Pose:
    """One pose's ligand: FP64 placement, its backward and the score gradient."""

    def __init__(self, rec, lig, sf, x_ref, dof):
        self.rec, self.lig, self.sf = rec, lig, sf
        self.port = O.PortSystem(rec, lig)
        self.x_ref = np.asarray(x_ref, float)
        self.dof = dof
        t = lig.tree
        self.T = lig.n_torsions
        self.perm = np.asarray(t.perm)
        self.frag_of = np.zeros(lig.n_atoms, int)
        for f in range(t.n_frags):
            self.frag_of[t.frag_start[f]:t.frag_end[f]] = f
        self.tors = [(int(t.tors_frag[k]), int(t.tors_parent[k]), int(t.tors_parent_atom[k]),
                      int(t.tors_mine_atom[k])) for k in range(self.T)]
        self.n_frags = t.n_frags

    def place(self, q):
        return self.port.ligand_apply(self.x_ref, q[:3], quat_rot(q[3:7]), q[7:7 + self.T])

    def backward(self, q, x, g):
        """dE/dq [dof] from dE/dx at x = place(q)."""
        c = q[:3]
        sf = np.zeros((self.n_frags, 3))
        st = np.zeros((self.n_frags, 3))
        for p in range(len(self.perm)):
            a = self.perm[p]
            sf[self.frag_of[p]] += g[a]
            st[self.frag_of[p]] += np.cross(x[a] - c, g[a])
        out = np.zeros(self.dof)  # torsions beyond the ligand's stay 0
        out[:3] = g.sum(axis=0)
        tt = np.cross(x - c, g).sum(axis=0)
        for k in range(self.T - 1, -1, -1):
            f, pf, pa, ma = self.tors[k]
            xp, xm = x[self.perm[pa]], x[self.perm[ma]]
            u = (xm - xp) / np.linalg.norm(xm - xp)
            out[7 + k] = u @ (st[f] - np.cross(xm - c, sf[f]))
            sf[pf] += sf[f]
            st[pf] += st[f]
        L = np.linalg.norm(q[3:7])
        w, v = q[3] / L, q[4:7] / L
        gq = np.concatenate([[-2 * tt @ v], 2 * (w * tt + np.cross(tt, v))])
        qn = np.concatenate([[w], v])
        out[3:7] = (gq - (gq @ qn) * qn) / L
        return out

    def grad(self, q, w, table):
        """(dE/dq, dE/dw, dE/dT) at q."""
        x = self.place(q)
        _, _, gx, gw, gt = O.port_score_diff(self.sf, self.rec, self.lig, self.rec.xyz, x, w, table)
        return self.backward(q, x, gx), gw, gt

    def hvp(self, q, u, w, table, eps=1e-8):
        n = np.linalg.norm(u)
        if n == 0:
            return np.zeros(self.dof), np.zeros(36), np.zeros(32 * 256)
        d = u / n
        gp, wp, tp = self.grad(q + eps * d, w, table)
        gm, wm, tm = self.grad(q - eps * d, w, table)
        s = n / (2 * eps)
        return s * (gp - gm), s * (wp - wm), s * (tp - tm)


class PortBackend:
    """The unrolled optimisation's backend in FP64 on the host: poses [P] (Pose
    objects), the same DOF rows as the GPU backend."""

    dtype = torch.float64

    def __init__(self, poses, threads=1):
        self.poses, self.P = poses, len(poses)
        self.A = max(p.lig.n_atoms for p in poses)
        self.threads = threads
        self.evals = 0

    def _map(self, fn):
        if self.threads > 1:
            with ThreadPoolExecutor(self.threads) as ex:
                return list(ex.map(fn, range(self.P)))
        return [fn(i) for i in range(self.P)]

    def place(self, q):
        qn = q.detach().cpu().numpy()
        out = np.zeros((self.P, self.A, 3))
        for i, pz in enumerate(self.poses):
            out[i, : pz.lig.n_atoms] = pz.place(qn[i])
        return torch.from_numpy(out)

    def place_backward(self, q, x, gx):
        qn, xn, gn = q.detach().cpu().numpy(), x.detach().cpu().numpy(), gx.detach().cpu().numpy()
        out = np.zeros_like(qn)
        for i, pz in enumerate(self.poses):
            n = pz.lig.n_atoms
            out[i] = pz.backward(qn[i], xn[i, :n], gn[i, :n])
        return torch.from_numpy(out)

    def grad(self, q, w, t):
        qn = q.detach().cpu().numpy()
        wn, tn = w.detach().cpu().numpy(), t.detach().cpu().numpy().reshape(-1)
        res = self._map(lambda i: self.poses[i].grad(qn[i], wn, tn))
        self.evals += self.P
        g = torch.from_numpy(np.array([r[0] for r in res]))
        return g, torch.zeros(1), torch.zeros(1)

    def hvp(self, q, u, x, gx, w, t):
        qn, un = q.detach().cpu().numpy(), u.detach().cpu().numpy()
        wn, tn = w.detach().cpu().numpy(), t.detach().cpu().numpy().reshape(-1)
        res = self._map(lambda i: self.poses[i].hvp(qn[i], un[i], wn, tn))
        self.evals += 2 * self.P
        hu = torch.from_numpy(np.array([r[0] for r in res]))
        return hu, torch.from_numpy(np.sum([r[1] for r in res], axis=0)), \
            torch.from_numpy(np.sum([r[2] for r in res], axis=0))
