"""TEST INFRASTRUCTURE: the rigid-body + torsion DOF mode of the batched optimiser in FP64.

lbfgs_step::apply and strong_wolfe (optimizer.cpp:205-560) restated in Python double over
any closure f(x) -> (energy, gradient), with the constants of pxd_lbfgs_params; and the
DOF closure of a pose: q = [centre (3), quaternion (4), ligand torsions (T), receptor
torsions (R)], placed from the pose's own input coordinates by the port's FP64 forward
kinematics (free_ligand::apply_parameters, data.cpp:522-641, via unroll_ref.Pose), scored
by the port's FP64 objective (binding_system_interactions::put_gradients), and mapped back
to q by the FP64 pose backward. Only tests/ use it, as the checker of the device mode.
"""
import math

import numpy as np

from unroll_ref import Pose

CONVERGED, NOT_CONVERGED, NAN = 0, 1, 2


def _cubic(x1, f1, g1, x2, f2, g2, lo, hi):
    d1 = g1 + g2 - 3.0 * (f1 - f2) / (x1 - x2)
    d2sq = d1 * d1 - g1 * g2
    if d2sq >= 0.0:
        d2 = math.sqrt(d2sq)
        if x1 <= x2:
            p = x2 - (x2 - x1) * ((g2 + d2 - d1) / (g2 - g1 + 2.0 * d2))
        else:
            p = x1 - (x1 - x2) * ((g1 + d2 - d1) / (g1 - g2 + 2.0 * d2))
        return min(max(p, lo), hi)
    return (lo + hi) / 2.0


def _strong_wolfe(obj, x, t, d, f, g, gtd, p, count):
    """strong_wolfe (optimizer.cpp:235-427): (f, g, t) accepted."""
    f_new, g_new = obj(x + t * d)
    count[0] += 1
    if math.isnan(f_new):
        return f_new, g, t
    gtd_new = float(g_new @ d)
    if abs(gtd_new) > p["ls_gtd_threshold"]:
        return f_new, g_new, t
    t_prev, f_prev, g_prev, gtd_prev = 0.0, f, g, gtd
    it = 0
    br = bf = bg = bgtd = None
    while it < p["ls_max"]:
        if f_new > f + p["ls_c1"] * t * gtd or (it > 1 and f_new >= f_prev):
            br, bf, bg, bgtd = [t_prev, t], [f_prev, f_new], [g_prev, g_new], [gtd_prev, gtd_new]
            break
        if abs(gtd_new) <= -p["ls_c2"] * gtd:
            return f_new, g_new, t
        if gtd_new >= 0.0:
            br, bf, bg, bgtd = [t_prev, t], [f_prev, f_new], [g_prev, g_new], [gtd_prev, gtd_new]
            break
        min_step, max_step, tmp = t + 0.01 * (t - t_prev), t * 10.0, t
        t = _cubic(t_prev, f_prev, gtd_prev, t, f_new, gtd_new, min_step, max_step)
        t_prev, f_prev, g_prev, gtd_prev = tmp, f_new, g_new, gtd_new
        f_new, g_new = obj(x + t * d)
        count[0] += 1
        gtd_new = float(g_new @ d)
        it += 1
    d_norm = 0.0
    if it == p["ls_max"]:
        br, bf, bg, bgtd = [0.0, t], [f, f_new], [g, g_new], [0.0, 0.0]
    else:
        d_norm = float(np.max(np.abs(d)))
    insuf, done = False, False
    lo, hi = (1, 0) if bf[0] > bf[1] else (0, 1)
    while not done and it < p["ls_max"]:
        min_step, max_step = (br[1], br[0]) if br[0] > br[1] else (br[0], br[1])
        eps = max_step - min_step
        if eps * d_norm < p["ls_tolerance_change"]:
            break
        t = _cubic(br[0], bf[0], bgtd[0], br[1], bf[1], bgtd[1], min_step, max_step)
        eps *= 0.1
        if min(max_step - t, t - min_step) < eps:
            if insuf or t >= max_step or t <= min_step:
                t = max_step - eps if abs(t - max_step) < abs(t - min_step) else min_step + eps
                insuf = False
            else:
                insuf = True
        else:
            insuf = False
        f_new, g_new = obj(x + t * d)
        count[0] += 1
        gtd_new = float(g_new @ d)
        it += 1
        if f_new > f + p["ls_c1"] * t * gtd or f_new >= bf[lo]:
            br[hi], bf[hi], bg[hi], bgtd[hi] = t, f_new, g_new, gtd_new
            lo, hi = (1, 0) if bf[0] > bf[1] else (0, 1)
        else:
            if abs(gtd_new) <= -p["ls_c2"] * gtd:
                done = True
            elif gtd_new * (br[hi] - br[lo]) >= 0.0:
                br[hi], bf[hi], bg[hi], bgtd[hi] = br[lo], bf[lo], bg[lo], bgtd[lo]
            br[lo], bf[lo], bg[lo], bgtd[lo] = t, f_new, g_new, gtd_new
    return bf[lo], bg[lo], br[lo]


def lbfgs(obj, x0, p):
    """lbfgs_step::apply (optimizer.cpp:429-560) on obj from x0: (x, loss, nevals, status);
    nevals counts the final evaluation of a run that moved, as the reference does."""
    x = np.array(x0, float)
    count = [1]
    loss, g = obj(x)
    if float(np.max(np.abs(g))) < p["tolerance_grad"]:
        return x, loss, count[0], CONVERGED
    m = p["history"]
    max_eval = p["max_eval"] if p["max_eval"] > 0 else p["max_iter"] * 5 // 4
    S, Y, RO = [], [], []
    H_diag, t, n_iter, status, updated = 1.0, 0.0, 0, NOT_CONVERGED, False
    g_prev, d = None, None
    while n_iter < p["max_iter"] and count[0] < max_eval:
        n_iter += 1
        reset = n_iter == 1
        if not reset:
            y, s = g - g_prev, d * t
            if float(np.max(np.abs(y))) > p["reset_threshold"]:
                reset = True
            else:
                ys = float(y @ s)
                if ys > 1e-10:
                    if len(S) == m:
                        S.pop(0), Y.pop(0), RO.pop(0)
                    S.append(s), Y.append(y), RO.append(1.0 / ys)
                    H_diag = ys / float(y @ y)
        if reset:
            S, Y, RO, H_diag = [], [], [], 1.0
            d = -g
            t = min(1.0, 1.0 / float(np.sum(np.abs(g)))) * p["lr"] * 0.1
        else:
            q = -g
            al = [0.0] * len(S)
            for k in range(len(S) - 1, -1, -1):
                al[k] = float(S[k] @ q) * RO[k]
                q = q - al[k] * Y[k]
            d = q * H_diag
            for k in range(len(S)):
                be = float(Y[k] @ d) * RO[k]
                d = d + (al[k] - be) * S[k]
            t = p["lr"]
        g_prev, prev_loss = g, loss
        gtd = float(g @ d)
        if gtd > -p["tolerance_change"]:
            status = CONVERGED
            break
        loss, g, t = _strong_wolfe(obj, x, t, d, loss, g, gtd, p, count)
        if math.isnan(loss):
            status = NAN
            break
        x = x + t * d
        updated = True
        if float(np.max(np.abs(g))) <= p["tolerance_grad"]:
            status = CONVERGED
            break
        if float(np.max(np.abs(d * t))) <= p["tolerance_change"]:
            status = CONVERGED
            break
        if abs(loss - prev_loss) < p["tolerance_change"]:
            status = CONVERGED
            break
    if updated:
        count[0] += 1
    return x, loss, count[0], status


class DofSystem:
    """The DOF objective of one pose: q -> (E, dE/dq) on a grid-built PortSystem `port`."""

    def __init__(self, port, rec, lig, x_ref):
        self.port, self.lig = port, lig
        self.T, self.R = lig.n_torsions, rec.n_rotors
        self.pose = Pose(rec, lig, None, np.asarray(x_ref, float), 7 + self.T)
        self.pose.port = port  # placement through the same port system

    def q0(self):
        q = np.zeros(7 + self.T + self.R)
        q[:3] = self.pose.x_ref.mean(axis=0)
        q[3] = 1.0
        return q

    def place(self, q):
        return self.pose.place(q[:7 + self.T])

    def __call__(self, q):
        x = self.place(q)
        e, tg, gx = self.port.score_grad(q[7 + self.T:], x)
        return e, np.concatenate([self.pose.backward(q[:7 + self.T], x, gx), tg])


def params_dict(p):
    """pxd_lbfgs_params (ctypes) as the dict lbfgs() takes."""
    return {k: getattr(p, k) for k, _ in type(p)._fields_}


def optimize_dof(port, rec, lig, x_in, params):
    """The DOF mode on one pose x_in: (placed final pose, FP64 energy there, nevals, status)."""
    sys_ = DofSystem(port, rec, lig, x_in)
    q, _, nevals, status = lbfgs(sys_, sys_.q0(), params_dict(params))
    x = sys_.place(q)
    e, _, _ = port.score_grad(q[7 + sys_.T:], x)
    return x, e, nevals, status
