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

// Warp-uniform scalars of the line search and the iteration, one private copy per lane
// (lbfgs_pose's frame). They are read-modify-written throughout (counters, the bracket's
// swaps), which one shared copy cannot survive: after divergent code a warp may run as
// separate groups of lanes, and a group that has already stored a field's next value
// hands it to a group still reading the old one (an iteration counter advanced twice).
struct LsState {
    double t, f, fn, gtd, gn, tp, fp, gp, br0, br1, bf0, bf1, bgtd0, bgtd1, dn, loss, prev_loss, H_diag;
    int it, lo, hi, insuf, done, base, count, pad;
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

// Floats of the two-loop scalars after the vectors: ro = 1 / (y . s) per physical slot
// (m + 1 doubles) and the pairs' coefficients (m doubles, or FP32 in their first halves),
// rounded up to 16 bytes.
__host__ __device__ constexpr int opt_scalar_floats(int m) { return (2 * (2 * m + 1) + 3) / 4 * 4; }

// Carves the vectors from vb (kOptVecs * Dp floats) and the two-loop scalars ro, al
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

// FP64 objective at the optimiser's variables x (the reported energy).
__device__ __forceinline__ double closure_energy64(Closure& c, const float* x) {
    return energy64(*c.env, *c.L, x, *c.b, c.lane);
}

// The same closure evaluated by a team of warps (the single-walker search's team mode).
struct TeamClosure : Closure {
    const Team* team;
};

__device__ __forceinline__ double closure_eval(TeamClosure& c, double t, const float* d, float* g,
                                               double* gdot = nullptr) {
    ++c.nevals;
    return eval_pose<true>(*c.env, *c.L, c.x0, d, static_cast<float>(t), g, *c.b, c.lane, gdot, c.team);
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

// strong_wolfe (optimizer.cpp:235-427); g holds the current gradient on entry and the
// accepted one on exit. Its scalars live in S, the caller's lane-private state; the
// evaluation's directional derivative comes back through a local, so no field of S has
// its address taken and the compiler keeps S in registers. Cl is the closure over the
// variables: Closure (Cartesian) or DofClosure (rigid body + torsions).
template <class Cl>
static __device__ void strong_wolfe(Cl& c, const LbfgsConsts& p, const float* d, float* g,
                                    const Vecs& v, int D, int lane, LsState& S) {
    float* g_new = v.gnew;
    float* g_prev = v.gprev;
    S.f = S.loss;
    {
        double gn_new;
        S.fn = closure_eval(c, S.t, d, g_new, &gn_new);
        S.gn = gn_new;
    }
    if (isnan(S.fn)) {
        S.loss = S.fn;
        return;
    }
    if (fabs(S.gn) > p.gtd_threshold) {
        S.loss = S.fn;
        vcopy(g, g_new, D, lane);
        return;
    }
    S.tp = 0.0;
    S.fp = S.f;
    S.gp = S.gtd;
    // the previous trial's gradient: g itself until the first interpolation step
    const float* gpv = g;
    S.it = 0;
    while (S.it < p.ls_max) {
        if ((S.fn > S.f + p.c1 * S.t * S.gtd) || (S.it > 1 && S.fn >= S.fp)) {
            S.br0 = S.tp; S.br1 = S.t; S.bf0 = S.fp; S.bf1 = S.fn;
            vcopy(v.bg0, gpv, D, lane);
            vcopy(v.bg1, g_new, D, lane);
            S.bgtd0 = S.gp; S.bgtd1 = S.gn;
            break;
        }
        if (fabs(S.gn) <= -p.c2 * S.gtd) {
            // strong Wolfe holds at this trial: it is the accepted step
            S.loss = S.fn;
            vcopy(g, g_new, D, lane);
            return;
        }
        if (S.gn >= 0.0) {
            S.br0 = S.tp; S.br1 = S.t; S.bf0 = S.fp; S.bf1 = S.fn;
            vcopy(v.bg0, gpv, D, lane);
            vcopy(v.bg1, g_new, D, lane);
            S.bgtd0 = S.gp; S.bgtd1 = S.gn;
            break;
        }
        const double min_step = S.t + 0.01 * (S.t - S.tp);
        const double max_step = S.t * 10.0;
        const double tmp = S.t;
        S.t = cubic_interpolate(S.tp, S.fp, S.gp, S.t, S.fn, S.gn, min_step, max_step);
        S.tp = tmp;
        S.fp = S.fn;
        vcopy(g_prev, g_new, D, lane);
        gpv = g_prev;
        S.gp = S.gn;
        {
            double gn_new;
            S.fn = closure_eval(c, S.t, d, g_new, &gn_new);
            S.gn = gn_new;
        }
        ++S.it;
    }
    S.dn = 0.0;
    if (S.it == p.ls_max) {
        S.br0 = 0.0; S.br1 = S.t; S.bf0 = S.f; S.bf1 = S.fn;
        vcopy(v.bg0, g, D, lane);
        vcopy(v.bg1, g_new, D, lane);
    } else {
        S.dn = vabsmax(d, D, lane);
    }
    S.insuf = 0;
    S.done = 0;
    S.lo = S.bf0 > S.bf1 ? 1 : 0;
    S.hi = 1 - S.lo;
    while (!S.done && S.it < p.ls_max) {
        double min_step, max_step;
        if (S.br0 > S.br1) {
            min_step = S.br1;
            max_step = S.br0;
        } else {
            min_step = S.br0;
            max_step = S.br1;
        }
        double eps = max_step - min_step;
        if (eps * S.dn < p.ls_tol_change) break;
        double t = cubic_interpolate(S.br0, S.bf0, S.bgtd0, S.br1, S.bf1, S.bgtd1, min_step, max_step);
        eps *= 0.1;
        if (fmin(max_step - t, t - min_step) < eps) {
            if (S.insuf || t >= max_step || t <= min_step) {
                if (fabs(t - max_step) < fabs(t - min_step))
                    t = max_step - eps;
                else
                    t = min_step + eps;
                S.insuf = 0;
            } else {
                S.insuf = 1;
            }
        } else {
            S.insuf = 0;
        }
        S.t = t;
        {
            double gn_new;
            S.fn = closure_eval(c, S.t, d, g_new, &gn_new);
            S.gn = gn_new;
        }
        ++S.it;
        const int lo = S.lo, hi = S.hi;
        const double bf_lo = lo ? S.bf1 : S.bf0;
        if (S.fn > (S.f + p.c1 * S.t * S.gtd) || S.fn >= bf_lo) {
            if (hi) { S.br1 = S.t; S.bf1 = S.fn; S.bgtd1 = S.gn; } else { S.br0 = S.t; S.bf0 = S.fn; S.bgtd0 = S.gn; }
            vcopy(hi ? v.bg1 : v.bg0, g_new, D, lane);
            S.lo = S.bf0 > S.bf1 ? 1 : 0;
            S.hi = 1 - S.lo;
        } else {
            if (fabs(S.gn) <= -p.c2 * S.gtd) {
                S.done = 1;
            } else if (S.gn * ((hi ? S.br1 : S.br0) - (lo ? S.br1 : S.br0)) >= 0.0) {
                if (hi) { S.br1 = S.br0; S.bf1 = S.bf0; S.bgtd1 = S.bgtd0; } else { S.br0 = S.br1; S.bf0 = S.bf1; S.bgtd0 = S.bgtd1; }
                vcopy(hi ? v.bg1 : v.bg0, lo ? v.bg1 : v.bg0, D, lane);
            }
            if (lo) { S.br1 = S.t; S.bf1 = S.fn; S.bgtd1 = S.gn; } else { S.br0 = S.t; S.bf0 = S.fn; S.bgtd0 = S.gn; }
            vcopy(lo ? v.bg1 : v.bg0, g_new, D, lane);
        }
    }
    S.t = S.lo ? S.br1 : S.br0;
    S.loss = S.lo ? S.bf1 : S.bf0;
    vcopy(g, S.lo ? v.bg1 : v.bg0, D, lane);
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
// With kRegLoop and D <= 256 both loops keep the direction in registers (two_loop_regs)
// instead of the shared q and d, with the same arithmetic.
// Kept pairs sit in physical slots (base + j) % (m + 1), j = 0 .. count - 1 oldest first;
// the spare slot (base + count) % (m + 1) receives the next pair. The iteration's scalars
// (loss, step, H_diag, the history ring) live with the line search's in the lane-private
// LsState.
//
// energy receives the FP64 objective at the returned pose (energy64), or, with
// final_energy false (a caller that does not use it), the last FP32 loss.
// The two-loop recursion for D <= E * 32, the direction held in registers (E elements per
// lane) instead of the shared vectors q and d. Each pass's history elements are loaded
// before the reduction its coefficient waits on, and no pass stores or reloads the
// direction, so the only dependent chain left is the reduction itself: what a warp alone on
// its SM (the single-walker search) waits on. Lane-element order, products and accumulation
// are those of the shared-vector loops, so the result is the same bit for bit. kF32: the
// coefficients in FP32 (see lbfgs_pose). Writes g_prev = g and d; returns g . d.
// Dot product of a lane's E register elements (x[j] * y[j] where lane + 32 j < D) with
// the products' exact errors, summed as a pairwise two-sum tree (depth log2 E instead of E
// dependent compensated additions), rounded once to FP32, then summed over the warp by a
// plain FP32 butterfly: the same value on every lane. The single-walker search's two-loop
// dot products, whose dependent chain is what a warp alone on its SM waits on.
template <int E>
__device__ __forceinline__ float lane_tree_warp_dot(const float* x, const float* y, int lane, int D) {
    float p[E], pe = 0.f;
#pragma unroll
    for (int j = 0; j < E; ++j) {
        const bool ok = lane + j * kWarp < D;
        const float a = ok ? x[j] : 0.f, b = ok ? y[j] : 0.f;
        p[j] = a * b;
        pe += fmaf(a, b, -p[j]);
    }
#pragma unroll
    for (int w = 1; w < E; w *= 2) {
#pragma unroll
        for (int j = 0; j + w < E; j += 2 * w) {
            const float s = p[j] + p[j + w];
            const float bb = s - p[j];
            pe += (p[j] - (s - bb)) + (p[j + w] - bb);
            p[j] = s;
        }
    }
    float f = p[0] + pe;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) f += __shfl_xor_sync(kFull, f, off);
    return f;
}

// two_loop_regs with FP32 coefficients and the per-pass dot products of
// lane_tree_warp_dot (the single-walker search). Writes g_prev = g and d; returns g . d.
template <int E>
static __device__ __forceinline__ double two_loop_regs_tree(const Vecs& v, int base, int count, int slots,
                                                            size_t Dp, int D, int lane, float hd) {
    float r[E], xv[E];
    int sl = base + count - 1 >= slots ? base + count - 1 - slots : base + count - 1;
    {
        const float* sk = v.S + sl * Dp;
#pragma unroll
        for (int j = 0; j < E; ++j) {
            const int e = lane + j * kWarp;
            r[j] = 0.f;
            xv[j] = 0.f;
            if (e < D) {
                const float ge = v.g[e];
                r[j] = -ge;
                v.gp[e] = ge;
                xv[j] = sk[e];
            }
        }
    }
    float dot = lane_tree_warp_dot<E>(xv, r, lane, D);
    float* alf = reinterpret_cast<float*>(v.al);
    for (int k = count - 1; k >= 0; --k) {
        const float* yk = v.Y + sl * Dp;
        const int sn_slot = sl == 0 ? slots - 1 : sl - 1;
        const float* sn = v.S + sn_slot * Dp;
        float yv[E];
#pragma unroll
        for (int j = 0; j < E; ++j) {
            const int e = lane + j * kWarp;
            yv[j] = e < D ? yk[e] : 0.f;
            xv[j] = e < D && k > 0 ? sn[e] : 0.f;
        }
        const float a = dot * static_cast<float>(v.ro[sl]);
        alf[k] = a;  // every lane holds the same value
#pragma unroll
        for (int j = 0; j < E; ++j) r[j] = fmaf(yv[j], -a, r[j]);
        if (k > 0) {
            dot = lane_tree_warp_dot<E>(xv, r, lane, D);
        } else {
#pragma unroll
            for (int j = 0; j < E; ++j) r[j] *= hd;
            dot = lane_tree_warp_dot<E>(yv, r, lane, D);
        }
        sl = sn_slot;
    }
    __syncwarp();
    sl = base;
    for (int k = 0; k < count; ++k) {
        const float* sk = v.S + sl * Dp;
        const int nx_slot = sl + 1 == slots ? 0 : sl + 1;
        const float* nx = k + 1 < count ? v.Y + nx_slot * Dp : v.g;
        float sv[E];
#pragma unroll
        for (int j = 0; j < E; ++j) {
            const int e = lane + j * kWarp;
            sv[j] = e < D ? sk[e] : 0.f;
            xv[j] = e < D ? nx[e] : 0.f;
        }
        const float w = alf[k] - dot * static_cast<float>(v.ro[sl]);
#pragma unroll
        for (int j = 0; j < E; ++j) r[j] = fmaf(sv[j], w, r[j]);
        if (k + 1 < count) dot = lane_tree_warp_dot<E>(xv, r, lane, D);
        sl = nx_slot;
    }
    // g . d for the line search, compensated as elsewhere
    DS acc{0.f, 0.f};
#pragma unroll
    for (int j = 0; j < E; ++j) {
        const int e = lane + j * kWarp;
        if (e < D) {
            v.d[e] = r[j];
            ds_dot_acc(acc, v.g[e], r[j]);
        }
    }
    __syncwarp();
    return ds_warp_sum(acc);
}

template <int E, bool kF32>
static __device__ __forceinline__ double two_loop_regs(const Vecs& v, int base, int count, int slots,
                                                       size_t Dp, int D, int lane, float hd) {
    float r[E];
    int sl = base + count - 1 >= slots ? base + count - 1 - slots : base + count - 1;
    DS acc{0.f, 0.f};
    {
        const float* sk = v.S + sl * Dp;
#pragma unroll
        for (int j = 0; j < E; ++j) {
            const int e = lane + j * kWarp;
            r[j] = 0.f;
            if (e < D) {
                const float ge = v.g[e];
                r[j] = -ge;
                v.gp[e] = ge;
                ds_dot_acc(acc, sk[e], -ge);
            }
        }
    }
    float* alf = reinterpret_cast<float*>(v.al);
    for (int k = count - 1; k >= 0; --k) {
        const float* yk = v.Y + sl * Dp;
        const int sn_slot = sl == 0 ? slots - 1 : sl - 1;
        const float* sn = v.S + sn_slot * Dp;
        float yv[E], sv[E];
#pragma unroll
        for (int j = 0; j < E; ++j) {
            const int e = lane + j * kWarp;
            yv[j] = e < D ? yk[e] : 0.f;
            sv[j] = e < D && k > 0 ? sn[e] : 0.f;
        }
        float nal;
        if constexpr (kF32) {
            const float a = ds_warp_sum_f(acc) * static_cast<float>(v.ro[sl]);
            if (lane == 0) alf[k] = a;
            nal = -a;
        } else {
            const double al = ds_warp_sum(acc) * v.ro[sl];
            if (lane == 0) v.al[k] = al;
            nal = static_cast<float>(-al);
        }
        acc = DS{0.f, 0.f};
        if (k > 0) {
#pragma unroll
            for (int j = 0; j < E; ++j) {
                if (lane + j * kWarp < D) {
                    r[j] = fmaf(yv[j], nal, r[j]);
                    ds_dot_acc(acc, sv[j], r[j]);
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < E; ++j) {
                if (lane + j * kWarp < D) {
                    r[j] = fmaf(yv[j], nal, r[j]) * hd;
                    ds_dot_acc(acc, yv[j], r[j]);
                }
            }
        }
        sl = sn_slot;
    }
    __syncwarp();  // alf written by lane 0 above, read by every lane below
    sl = base;
    for (int k = 0; k < count; ++k) {
        const float* sk = v.S + sl * Dp;
        const int nx_slot = sl + 1 == slots ? 0 : sl + 1;
        const float* nx = k + 1 < count ? v.Y + nx_slot * Dp : v.g;
        float sv[E], nv[E];
#pragma unroll
        for (int j = 0; j < E; ++j) {
            const int e = lane + j * kWarp;
            sv[j] = e < D ? sk[e] : 0.f;
            nv[j] = e < D ? nx[e] : 0.f;
        }
        float w;
        if constexpr (kF32)
            w = alf[k] - ds_warp_sum_f(acc) * static_cast<float>(v.ro[sl]);
        else
            w = static_cast<float>(v.al[k] - ds_warp_sum(acc) * v.ro[sl]);
        acc = DS{0.f, 0.f};
#pragma unroll
        for (int j = 0; j < E; ++j) {
            if (lane + j * kWarp < D) {
                r[j] = fmaf(sv[j], w, r[j]);
                ds_dot_acc(acc, nv[j], r[j]);
            }
        }
        sl = nx_slot;
    }
#pragma unroll
    for (int j = 0; j < E; ++j) {
        const int e = lane + j * kWarp;
        if (e < D) v.d[e] = r[j];
    }
    __syncwarp();
    return ds_warp_sum(acc);  // g . d after the last step
}

template <bool kFast = false, bool kRegLoop = kFast, class Cl>
static __device__ int lbfgs_pose(Cl& c, const LbfgsConsts& p, const Vecs& v, int D,
                          size_t Dp, int lane, double& energy, bool final_energy = true) {
    const int m = p.m;
    const int slots = hist_slots(m);
    const int max_eval = p.max_eval > 0 ? p.max_eval : p.max_iter * 5 / 4;
    c.x0 = v.x;
    c.nevals = 0;
    LsState S;
    S.loss = closure_eval(c, 0.0, nullptr, v.g);
    if (vabsmax(v.g, D, lane) < p.tol_grad) {
        energy = final_energy ? closure_energy64(c, v.x) : S.loss;
        return PXD_POSE_CONVERGED;
    }
    int status = PXD_POSE_NOT_CONVERGED;
    S.base = 0;
    S.count = 0;
    S.H_diag = 1.0;
    S.t = 0.0;
    int n_iter = 0;
    bool updated = false;
    while (n_iter < p.max_iter && c.nevals < max_eval) {
        ++n_iter;
        bool reset = n_iter == 1;
        if (!reset) {
            const int spare = (S.base + S.count) % slots;
            float* ys_ = v.Y + spare * Dp;
            float* ss_ = v.S + spare * Dp;
            const float tf = static_cast<float>(S.t);
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
                    if (S.count == m)
                        S.base = (S.base + 1) % slots;  // the oldest slot becomes the spare
                    else
                        ++S.count;
                    S.H_diag = ys / yy;
                    if (lane == 0) v.ro[spare] = 1.0 / ys;
                }
            }
            __syncwarp();
        }
        double gtd;
        if (reset || S.count == 0) {
            // d = -H_diag g (H_diag = 1 after a reset), g_prev = g, g . d and |g|_1
            if (reset) {
                S.base = S.count = 0;
                S.H_diag = 1.0;
            }
            const float hd = static_cast<float>(S.H_diag);
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
                S.t = fmin(1.0, inv) * p.lr * 0.1;
            } else {
                S.t = p.lr;
            }
        } else if (kFast && D <= 4 * kWarp) {
            gtd = two_loop_regs_tree<4>(v, S.base, S.count, slots, Dp, D, lane, static_cast<float>(S.H_diag));
            S.t = p.lr;
        } else if (kFast && D <= 8 * kWarp) {
            gtd = two_loop_regs_tree<8>(v, S.base, S.count, slots, Dp, D, lane, static_cast<float>(S.H_diag));
            S.t = p.lr;
        } else if (kRegLoop && D <= 4 * kWarp) {
            gtd = two_loop_regs<4, kFast>(v, S.base, S.count, slots, Dp, D, lane, static_cast<float>(S.H_diag));
            S.t = p.lr;
        } else if (kRegLoop && D <= 8 * kWarp) {
            gtd = two_loop_regs<8, kFast>(v, S.base, S.count, slots, Dp, D, lane, static_cast<float>(S.H_diag));
            S.t = p.lr;
        } else {
            // first loop, newest to oldest: q = -g - sum al_k y_k. The ring's base and count
            // are read once into registers: the line-search state lives in the lane's frame,
            // and its fields would otherwise be reloaded from local memory at every pass.
            const int base = S.base, count = S.count;
            int sl = base + count - 1 >= slots ? base + count - 1 - slots : base + count - 1;
            DS acc{0.f, 0.f};
            {
                const float* sk = v.S + sl * Dp;
                for (int e = lane; e < D; e += kWarp) {
                    const float ge = v.g[e];
                    v.q[e] = -ge;
                    v.gp[e] = ge;
                    ds_dot_acc(acc, sk[e], -ge);
                }
            }
            // kFast: the coefficients alpha_k = rho_k s_k . q and alpha_k - beta_k are formed in
            // FP32 from the compensated dot products (each dot rounded once) instead of FP64:
            // they scale FP32 vectors, and off the FP64 pipe every pass's dependent chain is
            // shorter (the single-walker search's relaxations, 11 % faster).
            float* alf = reinterpret_cast<float*>(v.al);
            for (int k = count - 1; k >= 0; --k) {
                float nal;
                if constexpr (kFast) {
                    const float a = ds_warp_sum_f(acc) * static_cast<float>(v.ro[sl]);
                    if (lane == 0) alf[k] = a;
                    nal = -a;
                } else {
                    const double al = ds_warp_sum(acc) * v.ro[sl];
                    if (lane == 0) v.al[k] = al;
                    nal = static_cast<float>(-al);
                }
                const float* yk = v.Y + sl * Dp;
                const int sn_slot = sl == 0 ? slots - 1 : sl - 1;
                acc = DS{0.f, 0.f};
                if (k > 0) {
                    const float* sn = v.S + sn_slot * Dp;
                    for (int e = lane; e < D; e += kWarp) {
                        const float qe = fmaf(yk[e], nal, v.q[e]);
                        v.q[e] = qe;
                        ds_dot_acc(acc, sn[e], qe);
                    }
                } else {
                    // the last update, then d = H_diag q and the second loop's first dot
                    const float hd = static_cast<float>(S.H_diag);
                    for (int e = lane; e < D; e += kWarp) {
                        const float de = fmaf(yk[e], nal, v.q[e]) * hd;
                        v.d[e] = de;
                        ds_dot_acc(acc, yk[e], de);
                    }
                }
                __syncwarp();
                sl = sn_slot;
            }
            // second loop, oldest to newest: d += (al_k - be_k) s_k
            sl = base;
            for (int k = 0; k < count; ++k) {
                float w;
                if constexpr (kFast) {
                    w = alf[k] - ds_warp_sum_f(acc) * static_cast<float>(v.ro[sl]);
                } else {
                    const double be = ds_warp_sum(acc) * v.ro[sl];
                    w = static_cast<float>(v.al[k] - be);
                }
                const float* sk = v.S + sl * Dp;
                const int nx_slot = sl + 1 == slots ? 0 : sl + 1;
                const float* nx = k + 1 < count ? v.Y + nx_slot * Dp : v.g;
                acc = DS{0.f, 0.f};
                for (int e = lane; e < D; e += kWarp) {
                    const float de = fmaf(sk[e], w, v.d[e]);
                    v.d[e] = de;
                    ds_dot_acc(acc, nx[e], de);
                }
                __syncwarp();
                sl = nx_slot;
            }
            gtd = ds_warp_sum(acc);  // g . d after the last step
            S.t = p.lr;
        }
        S.prev_loss = S.loss;
        if (gtd > -p.tol_change) {
            status = PXD_POSE_CONVERGED;
            break;
        }
        S.gtd = gtd;
        strong_wolfe(c, p, v.d, v.g, v, D, lane, S);
        if (isnan(S.loss)) {
            status = PXD_POSE_NAN;
            break;
        }
        // x += t d, with max|g| and max|t d| for the convergence tests
        const float tf = static_cast<float>(S.t);
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
        if (fabs(S.loss - S.prev_loss) < p.tol_change) {
            status = PXD_POSE_CONVERGED;
            break;
        }
    }
    // the reported energy: the FP64 objective at the returned pose; an optimisation that
    // moved counts it as its final evaluation, as the reference does (optimizer.cpp:552-556)
    if (updated) ++c.nevals;
    energy = final_energy ? closure_energy64(c, v.x) : S.loss;
    return status;
}

}  // namespace pxd
