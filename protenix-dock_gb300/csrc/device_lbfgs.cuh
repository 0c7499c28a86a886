// Batched L-BFGS + strong-Wolfe line search for one pose per warp (device code shared
// by the L-BFGS and Monte-Carlo kernels). Control flow restates lbfgs_step::apply and
// strong_wolfe (optimizer.cpp:205-560) with the caller's constants; pose vectors live in
// shared memory, the m-deep history in a per-warp scratch slab. The scalars that steer
// the iteration are FP64 and identical on all 32 lanes; every loop is bounded.
#pragma once

#include "device_eval.cuh"
#include "energy64.cuh"

namespace pxd {

struct LbfgsConsts {
    int max_iter, max_eval, m, ls_max;
    double lr, tol_grad, tol_change, c1, c2, ls_tol_change, gtd_threshold, reset;
};

struct Vecs {
    float *x, *g, *gp, *d, *q, *sv, *gnew, *gprev, *bg0, *bg1;
    float *S, *Y;
    double *ro, *al;
};

// D_pad-long vectors in a warp's optimiser slice: x, g, gp, d and the line search's g_new,
// g_prev and two bracket gradients. The history update's y / two-loop q and s share the
// space of g_prev and g_new: those are live only inside strong_wolfe and the final
// evaluation, q and s only between line searches. Eight vectors instead of ten keep four
// blocks' slices inside a smaller shared-memory carve-out, which leaves more L1 for the
// history slab, the map gathers and the topology records.
constexpr int kOptVecs = 8;

// Physical L-BFGS history slots of a warp: the m kept (s, y) pairs and one spare that
// receives the next pair before its curvature test decides whether it is kept, so the
// pair is written once, in the pass that forms it.
__host__ __device__ constexpr int hist_slots(int m) { return m + 1; }

// Floats of the FP64 two-loop scalars after the vectors: ro per physical slot (m + 1
// doubles) and al per kept pair (m doubles), rounded up to 16 bytes.
__host__ __device__ constexpr int opt_scalar_floats(int m) { return (2 * (2 * m + 1) + 3) / 4 * 4; }

// Carves the vectors from vb (kOptVecs * Dp floats) and the FP64 two-loop scalars ro, al
// (opt_scalar_floats(m) floats) after them.
__device__ __forceinline__ Vecs carve_vecs(float* vb, int Dp, int m) {
    Vecs v;
    v.x = vb;
    v.g = vb + Dp;
    v.gp = vb + 2 * Dp;
    v.d = vb + 3 * Dp;
    v.gnew = vb + 4 * Dp;
    v.gprev = vb + 5 * Dp;
    v.bg0 = vb + 6 * Dp;
    v.bg1 = vb + 7 * Dp;
    v.q = v.gprev;
    v.sv = v.gnew;
    v.ro = reinterpret_cast<double*>(vb + kOptVecs * Dp);
    v.al = v.ro + hist_slots(m);
    v.S = v.Y = nullptr;
    return v;
}

struct Closure {
    const EvalEnv* env;
    const DevLigand* L;
    const PoseBufs* b;
    const float* x0;
    int lane;
    int nevals;
};

__device__ __forceinline__ double closure_eval(Closure& c, double t, const float* d, float* g,
                                               double* gdot = nullptr) {
    ++c.nevals;
    return eval_pose(*c.env, *c.L, c.x0, d, static_cast<float>(t), g, *c.b, c.lane, gdot);
}

__device__ __forceinline__ double cubic_interpolate(double x1, double f1, double g1, double x2,
                                                    double f2, double g2, double lo, double hi) {
    double d1 = g1 + g2 - 3.0 * (f1 - f2) / (x1 - x2);
    const double d2sq = d1 * d1 - g1 * g2;
    if (d2sq >= 0.0) {
        const double d2 = sqrt(d2sq);
        if (x1 <= x2)
            d1 = x2 - (x2 - x1) * ((g2 + d2 - d1) / (g2 - g1 + 2.0 * d2));
        else
            d1 = x1 - (x1 - x2) * ((g1 + d2 - d1) / (g1 - g2 + 2.0 * d2));
        return fmin(fmax(d1, lo), hi);
    }
    return (lo + hi) / 2.0;
}

// The two ends of the line search's bracket (step, value, directional derivative,
// gradient) as named scalars selected by index 0 / 1: no dynamically indexed local arrays.
struct Bracket {
    double br0 = 0.0, br1 = 0.0, bf0 = 0.0, bf1 = 0.0, bgtd0 = 0.0, bgtd1 = 0.0;
    float *bg0, *bg1;
    __device__ double br(int i) const { return i ? br1 : br0; }
    __device__ double bf(int i) const { return i ? bf1 : bf0; }
    __device__ double bgtd(int i) const { return i ? bgtd1 : bgtd0; }
    __device__ float* bg(int i) const { return i ? bg1 : bg0; }
    __device__ void set_br(int i, double x) {
        if (i) br1 = x;
        else br0 = x;
    }
    __device__ void set_bf(int i, double x) {
        if (i) bf1 = x;
        else bf0 = x;
    }
    __device__ void set_bgtd(int i, double x) {
        if (i) bgtd1 = x;
        else bgtd0 = x;
    }
};

// strong_wolfe (optimizer.cpp:235-427); g holds the current gradient on entry and the
// accepted one on exit.
static __device__ void strong_wolfe(Closure& c, const LbfgsConsts& p, double& t_io, const float* d,
                             double& f_io, float* g, double gtd, const Vecs& v, int D,
                             int lane) {
    double t = t_io;
    const double f = f_io;
    float* g_new = v.gnew;
    float* g_prev = v.gprev;
    Bracket B;
    B.bg0 = v.bg0;
    B.bg1 = v.bg1;
    double gtd_new = 0.0;
    double f_new = closure_eval(c, t, d, g_new, &gtd_new);
    if (isnan(f_new)) {
        f_io = f_new;
        return;
    }
    if (fabs(gtd_new) > p.gtd_threshold) {
        f_io = f_new;
        vcopy(g, g_new, D, lane);
        return;
    }
    double t_prev = 0.0, f_prev = f, gtd_prev = gtd;
    // the previous trial's gradient: g itself until the first interpolation step
    const float* gpv = g;
    int ls_iter = 0;
    while (ls_iter < p.ls_max) {
        if ((f_new > f + p.c1 * t * gtd) || (ls_iter > 1 && f_new >= f_prev)) {
            B.br0 = t_prev; B.br1 = t; B.bf0 = f_prev; B.bf1 = f_new;
            vcopy(B.bg0, gpv, D, lane);
            vcopy(B.bg1, g_new, D, lane);
            B.bgtd0 = gtd_prev; B.bgtd1 = gtd_new;
            break;
        }
        if (fabs(gtd_new) <= -p.c2 * gtd) {
            // strong Wolfe holds at this trial: it is the accepted step
            t_io = t;
            f_io = f_new;
            vcopy(g, g_new, D, lane);
            return;
        }
        if (gtd_new >= 0.0) {
            B.br0 = t_prev; B.br1 = t; B.bf0 = f_prev; B.bf1 = f_new;
            vcopy(B.bg0, gpv, D, lane);
            vcopy(B.bg1, g_new, D, lane);
            B.bgtd0 = gtd_prev; B.bgtd1 = gtd_new;
            break;
        }
        const double min_step = t + 0.01 * (t - t_prev);
        const double max_step = t * 10.0;
        const double tmp = t;
        t = cubic_interpolate(t_prev, f_prev, gtd_prev, t, f_new, gtd_new, min_step, max_step);
        t_prev = tmp;
        f_prev = f_new;
        vcopy(g_prev, g_new, D, lane);
        gpv = g_prev;
        gtd_prev = gtd_new;
        f_new = closure_eval(c, t, d, g_new, &gtd_new);
        ++ls_iter;
    }
    double d_norm = 0.0;
    if (ls_iter == p.ls_max) {
        B.br0 = 0.0; B.br1 = t; B.bf0 = f; B.bf1 = f_new;
        vcopy(B.bg0, g, D, lane);
        vcopy(B.bg1, g_new, D, lane);
    } else {
        d_norm = vabsmax(d, D, lane);
    }
    bool insuf = false, done = false;
    int lo = 0, hi = 1;
    if (B.bf0 > B.bf1) {
        lo = 1;
        hi = 0;
    }
    while (!done && ls_iter < p.ls_max) {
        double min_step, max_step;
        if (B.br0 > B.br1) {
            min_step = B.br1;
            max_step = B.br0;
        } else {
            min_step = B.br0;
            max_step = B.br1;
        }
        double eps = max_step - min_step;
        if (eps * d_norm < p.ls_tol_change) break;
        t = cubic_interpolate(B.br0, B.bf0, B.bgtd0, B.br1, B.bf1, B.bgtd1, min_step, max_step);
        eps *= 0.1;
        if (fmin(max_step - t, t - min_step) < eps) {
            if (insuf || t >= max_step || t <= min_step) {
                if (fabs(t - max_step) < fabs(t - min_step))
                    t = max_step - eps;
                else
                    t = min_step + eps;
                insuf = false;
            } else {
                insuf = true;
            }
        } else {
            insuf = false;
        }
        f_new = closure_eval(c, t, d, g_new, &gtd_new);
        ++ls_iter;
        if (f_new > (f + p.c1 * t * gtd) || f_new >= B.bf(lo)) {
            B.set_br(hi, t);
            B.set_bf(hi, f_new);
            vcopy(B.bg(hi), g_new, D, lane);
            B.set_bgtd(hi, gtd_new);
            if (B.bf0 > B.bf1) {
                lo = 1;
                hi = 0;
            } else {
                lo = 0;
                hi = 1;
            }
        } else {
            if (fabs(gtd_new) <= -p.c2 * gtd) {
                done = true;
            } else if (gtd_new * (B.br(hi) - B.br(lo)) >= 0.0) {
                B.set_br(hi, B.br(lo));
                B.set_bf(hi, B.bf(lo));
                vcopy(B.bg(hi), B.bg(lo), D, lane);
                B.set_bgtd(hi, B.bgtd(lo));
            }
            B.set_br(lo, t);
            B.set_bf(lo, f_new);
            vcopy(B.bg(lo), g_new, D, lane);
            B.set_bgtd(lo, gtd_new);
        }
    }
    t_io = B.br(lo);
    f_io = B.bf(lo);
    vcopy(g, B.bg(lo), D, lane);
}


// lbfgs_step::apply (optimizer.cpp:429-560) on the pose held in v.x; returns status.
//
// The vector work of an iteration runs in fused passes over the warp's elements, each
// lane touching only its own elements (e = lane + 32 k), with the arithmetic of every
// element as in the textbook order, so the iterates are those of separate passes:
//   - the history update: y = g - g_prev and s = t d go straight into the spare history
//     slot, with max|y|, y.s and y.y in the same pass;
//   - the first loop: q -= al_k y_k fused with the next pair's s_{k-1} . q, then
//     d = H_diag q with y_0 . d;
//   - the second loop: d += (al_k - be_k) s_k fused with the next y_{k+1} . d, the last
//     step with g . d for the line search.
// Kept pairs sit in physical slots (base + j) % (m + 1), j = 0 .. count - 1 oldest first;
// the spare slot (base + count) % (m + 1) receives the next pair.
//
// energy receives the FP64 objective at the returned pose (energy64), or, with
// final_energy false (a caller that does not use it), the last FP32 loss.
static __device__ int lbfgs_pose(Closure& c, const LbfgsConsts& p, const Vecs& v, int D,
                          size_t Dp, int lane, double& energy, bool final_energy = true) {
    const int m = p.m;
    const int slots = hist_slots(m);
    const int max_eval = p.max_eval > 0 ? p.max_eval : p.max_iter * 5 / 4;
    c.x0 = v.x;
    c.nevals = 0;
    double loss = closure_eval(c, 0.0, nullptr, v.g);
    if (vabsmax(v.g, D, lane) < p.tol_grad) {
        energy = final_energy ? energy64(*c.env, *c.L, v.x, *c.b, lane) : loss;
        return PXD_POSE_CONVERGED;
    }
    int status = PXD_POSE_NOT_CONVERGED;
    int base = 0, count = 0;
    double H_diag = 1.0, t = 0.0, prev_loss;
    int n_iter = 0;
    bool updated = false;
    while (n_iter < p.max_iter && c.nevals < max_eval) {
        ++n_iter;
        bool reset = n_iter == 1;
        if (!reset) {
            const int spare = (base + count) % slots;
            float* ys_ = v.Y + spare * Dp;
            float* ss_ = v.S + spare * Dp;
            const float tf = static_cast<float>(t);
            float ymax = 0.f;
            DS a_ys{0.f, 0.f}, a_yy{0.f, 0.f};
            for (int e = lane; e < D; e += kWarp) {
                const float y = v.g[e] - v.gp[e];
                const float sv = v.d[e] * tf;
                ys_[e] = y;
                ss_[e] = sv;
                ymax = fmaxf(ymax, fabsf(y));
                ds_dot_acc(a_ys, y, sv);
                ds_dot_acc(a_yy, y, y);
            }
            reset = warp_max(ymax) > p.reset;
            if (!reset) {
                const double ys = ds_warp_sum(a_ys);
                const double yy = ds_warp_sum(a_yy);
                if (ys > 1e-10) {
                    if (count == m)
                        base = (base + 1) % slots;  // the oldest slot becomes the spare
                    else
                        ++count;
                    H_diag = ys / yy;
                    if (lane == 0) v.ro[spare] = 1.0 / ys;
                }
            }
            __syncwarp();
        }
        double gtd;
        if (reset || count == 0) {
            // d = -H_diag g (H_diag = 1 after a reset), g_prev = g, g . d and |g|_1
            if (reset) {
                base = count = 0;
                H_diag = 1.0;
            }
            const float hd = static_cast<float>(H_diag);
            DS acc{0.f, 0.f}, a_abs{0.f, 0.f};
            for (int e = lane; e < D; e += kWarp) {
                const float ge = v.g[e];
                const float de = reset ? -ge : (-ge) * hd;
                v.d[e] = de;
                v.gp[e] = ge;
                ds_dot_acc(acc, ge, de);
                ds_add(a_abs, fabsf(ge));
            }
            __syncwarp();
            gtd = ds_warp_sum(acc);
            if (reset) {
                const double inv = 1.0 / ds_warp_sum(a_abs);
                t = fmin(1.0, inv) * p.lr * 0.1;
            } else {
                t = p.lr;
            }
        } else {
            // first loop, newest to oldest: q = -g - sum al_k y_k
            DS acc{0.f, 0.f};
            {
                const float* sk = v.S + ((base + count - 1) % slots) * Dp;
                for (int e = lane; e < D; e += kWarp) {
                    const float ge = v.g[e];
                    v.q[e] = -ge;
                    v.gp[e] = ge;
                    ds_dot_acc(acc, sk[e], -ge);
                }
            }
            for (int k = count - 1; k >= 0; --k) {
                const int sl = (base + k) % slots;
                const double al = ds_warp_sum(acc) * v.ro[sl];
                if (lane == 0) v.al[k] = al;
                const float nal = static_cast<float>(-al);
                const float* yk = v.Y + sl * Dp;
                acc = DS{0.f, 0.f};
                if (k > 0) {
                    const float* sn = v.S + ((base + k - 1) % slots) * Dp;
                    for (int e = lane; e < D; e += kWarp) {
                        const float qe = fmaf(yk[e], nal, v.q[e]);
                        v.q[e] = qe;
                        ds_dot_acc(acc, sn[e], qe);
                    }
                } else {
                    // the last update, then d = H_diag q and the second loop's first dot
                    const float hd = static_cast<float>(H_diag);
                    for (int e = lane; e < D; e += kWarp) {
                        const float de = fmaf(yk[e], nal, v.q[e]) * hd;
                        v.d[e] = de;
                        ds_dot_acc(acc, yk[e], de);
                    }
                }
                __syncwarp();
            }
            // second loop, oldest to newest: d += (al_k - be_k) s_k
            for (int k = 0; k < count; ++k) {
                const int sl = (base + k) % slots;
                const double be = ds_warp_sum(acc) * v.ro[sl];
                const float w = static_cast<float>(v.al[k] - be);
                const float* sk = v.S + sl * Dp;
                const float* nx = k + 1 < count ? v.Y + ((base + k + 1) % slots) * Dp : v.g;
                acc = DS{0.f, 0.f};
                for (int e = lane; e < D; e += kWarp) {
                    const float de = fmaf(sk[e], w, v.d[e]);
                    v.d[e] = de;
                    ds_dot_acc(acc, nx[e], de);
                }
                __syncwarp();
            }
            gtd = ds_warp_sum(acc);  // g . d after the last step
            t = p.lr;
        }
        prev_loss = loss;
        if (gtd > -p.tol_change) {
            status = PXD_POSE_CONVERGED;
            break;
        }
        Vecs w = v;
        strong_wolfe(c, p, t, v.d, loss, v.g, gtd, w, D, lane);
        if (isnan(loss)) {
            status = PXD_POSE_NAN;
            break;
        }
        // x += t d, with max|g| and max|t d| for the convergence tests
        const float tf = static_cast<float>(t);
        float gmax = 0.f, smax = 0.f;
        for (int e = lane; e < D; e += kWarp) {
            const float de = v.d[e];
            v.x[e] = fmaf(de, tf, v.x[e]);
            gmax = fmaxf(gmax, fabsf(v.g[e]));
            smax = fmaxf(smax, fabsf(de * tf));
        }
        __syncwarp();
        updated = true;
        if (warp_max(gmax) <= p.tol_grad) {
            status = PXD_POSE_CONVERGED;
            break;
        }
        if (warp_max(smax) <= p.tol_change) {
            status = PXD_POSE_CONVERGED;
            break;
        }
        if (fabs(loss - prev_loss) < p.tol_change) {
            status = PXD_POSE_CONVERGED;
            break;
        }
    }
    // the reported energy: the FP64 objective at the returned pose; an optimisation that
    // moved counts it as its final evaluation, as the reference does (optimizer.cpp:552-556)
    if (updated) ++c.nevals;
    energy = final_energy ? energy64(*c.env, *c.L, v.x, *c.b, lane) : loss;
    return status;
}

}  // namespace pxd
