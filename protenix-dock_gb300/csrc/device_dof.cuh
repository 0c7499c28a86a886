// Rigid-body + torsion variables for the batched optimiser (PXD_DOF_RIGID_TORSION).
//
// The optimiser's vector is q = [centre (3) | quaternion (4) | ligand torsions (T) |
// receptor torsions (R)]. An evaluation places the ligand from the pose's own input
// coordinates with the torsion-tree forward map (free_ligand::apply_parameters,
// data.cpp:592-641): the input's geometric centre goes to the centre, the tree turns by
// the normalised quaternion, torsion k turns its subtree about its bond by q[7 + k]. The
// placed pose is scored by the same evaluation as the Cartesian closure, and its
// Cartesian gradient is pulled back to q:
//   dE/dcentre     = sum_i g_i
//   dE/dquaternion from the torque t = sum_i (x_i - centre) x g_i: a change dq of the
//                  unit quaternion (w, v) turns the pose by 2 (w dv - dw v + v x dv), so
//                  dE/dw = -2 t.v and dE/dv = 2 (w t + t x v), projected for the
//                  normalisation and divided by |q|;
//   dE/dtheta_k    = u_k . sum over the torsion's subtree of (x_i - x_bond) x g_i.
// One warp per pose; the per-fragment sums run one lane per fragment over its atoms in
// order and the subtree propagation on lane 0, so the gradient does not depend on the
// schedule.
#pragma once

#include "device_kin.cuh"
#include "device_lbfgs.cuh"

namespace pxd {

// Floats of a warp's forward-map frames (also the backward's per-fragment sums).
constexpr int kKinFloats = static_cast<int>(sizeof(KinShared) / sizeof(float));

struct DofClosure {
    const EvalEnv* env;
    const DevLigand* L;
    const PoseBufs* b;
    const float* x0;    // the optimiser's variables (base point of the line search)
    int lane;
    int nevals;
    float* q;           // [D] the evaluated variables
    float* xc;          // [3N + R] placed pose | receptor torsions (the Cartesian closure's x)
    float* gc;          // [3N + R] its Cartesian gradient
    KinShared* ks;
    float4* rel;        // [N] input coordinates relative to their tree anchors (permuted order)
    float4* axes;       // [32] unit input-frame torsion axes
};

// The input-frame half of the forward map, which does not depend on the variables, once
// per pose: the input's geometric centre (returned: the centre variable's start), every
// atom relative to its anchor (the centre for root atoms, the fragment's bond atom, or for
// a bond atom its parent's bond atom; data.cpp:540-559) and the torsion axes
// (data.cpp:530-537), with the arithmetic of ligand_forward.
static __device__ float3 dof_prepare(const DofClosure& c, const float* xref) {
    const DevLigand& L = *c.L;
    const int N = L.n_atoms;
    const int lane = c.lane;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int p = lane; p < N; p += kWarp) {
        const int a = __ldg(&L.perm[p]);
        sx += xref[3 * a];
        sy += xref[3 * a + 1];
        sz += xref[3 * a + 2];
    }
    const float3 center = mul3(make_float3(warp_sum_f(sx), warp_sum_f(sy), warp_sum_f(sz)), 1.f / N);
    auto at = [&](int p) {
        const int a = __ldg(&L.perm[p]);
        return make_float3(xref[3 * a], xref[3 * a + 1], xref[3 * a + 2]);
    };
    for (int p = lane; p < N; p += kWarp) {
        const int f = __ldg(&L.frag_of[p]);
        const int mine = __ldg(&L.frag_mine[f]);
        float3 anchor;
        if (mine < 0) {
            anchor = center;
        } else if (p != mine) {
            anchor = at(mine);
        } else {
            const int pm = __ldg(&L.frag_mine[__ldg(&L.frag_parent[f])]);
            anchor = pm < 0 ? center : at(pm);
        }
        const float3 r = sub3(at(p), anchor);
        c.rel[p] = make_float4(r.x, r.y, r.z, 0.f);
    }
    if (lane < L.n_tors) {
        const int4 tq = __ldg(&L.tors[lane]);
        float3 ax = sub3(at(tq.w), at(tq.z));
        ax = mul3(ax, 1.f / sqrtf(dot3(ax, ax)));
        c.axes[lane] = make_float4(ax.x, ax.y, ax.z, 0.f);
    }
    __syncwarp();
    return center;
}

// xc = [placed ligand (atom order) | receptor torsions] for the variables q: the frames of
// the tree in pre-order on lane 0 (rotation of the root, then each torsion's Rodrigues
// rotation about its world axis after its parent's frame), then every atom.
static __device__ void dof_place(const DofClosure& c, const float* q) {
    const DevLigand& L = *c.L;
    const int N = L.n_atoms, T = L.n_tors, R = c.env->rec.n_rotors;
    const int lane = c.lane;
    KinShared& ks = *c.ks;
    if (lane == 0) {
        const Mat3 rot = unit_quat_rotation(q + 3);
        const float3 center = make_float3(q[0], q[1], q[2]);
        for (int f = 0; f < L.n_frags; ++f) {
            if (__ldg(&L.frag_mine[f]) < 0) {
                ks.fused[f] = rot;
                ks.origin[f] = center;
            }
        }
        for (int k = 0; k < T; ++k) {
            const int4 tq = __ldg(&L.tors[k]);
            const Mat3 fp = ks.fused[tq.y];
            const float3 axis_w = mat_apply(fp, xyz(c.axes[k]));
            const float3 mine_w = add3(mat_apply(fp, xyz(c.rel[tq.w])), ks.origin[tq.y]);
            ks.fused[tq.x] = matmul(rodrigues(axis_w, q[7 + k]), fp);
            ks.origin[tq.x] = mine_w;
        }
    }
    __syncwarp();
    for (int p = lane; p < N; p += kWarp) {
        const int f = __ldg(&L.frag_of[p]);
        const int mine = __ldg(&L.frag_mine[f]);
        const float3 w = (mine >= 0 && p == mine) ? ks.origin[f]
                                                   : add3(mat_apply(ks.fused[f], xyz(c.rel[p])), ks.origin[f]);
        const int a = __ldg(&L.perm[p]);
        c.xc[3 * a] = w.x;
        c.xc[3 * a + 1] = w.y;
        c.xc[3 * a + 2] = w.z;
    }
    for (int r = lane; r < R; r += kWarp) c.xc[3 * N + r] = q[7 + T + r];
    __syncwarp();
}

// g = dE/dq from the Cartesian gradient c.gc at the placed pose c.xc.
static __device__ void dof_pullback(const DofClosure& c, const float* q, float* g) {
    const DevLigand& L = *c.L;
    const int N = L.n_atoms, T = L.n_tors, F = L.n_frags, R = c.env->rec.n_rotors;
    const int lane = c.lane;
    float3* sf = reinterpret_cast<float3*>(c.ks);  // [kMaxFrags] force of each subtree
    float3* st = sf + kMaxFrags;                   // [kMaxFrags] torque about the centre
    const float3 ctr = make_float3(q[0], q[1], q[2]);
    float3 ftot = make_float3(0.f, 0.f, 0.f), ttot = ftot;
    for (int f = lane; f < F; f += kWarp) {
        float3 fs = make_float3(0.f, 0.f, 0.f), ts = fs;
        for (int p = __ldg(&L.frag_range[2 * f]); p < __ldg(&L.frag_range[2 * f + 1]); ++p) {
            const int a = __ldg(&L.perm[p]);
            const float3 xi = make_float3(c.xc[3 * a], c.xc[3 * a + 1], c.xc[3 * a + 2]);
            const float3 gi = make_float3(c.gc[3 * a], c.gc[3 * a + 1], c.gc[3 * a + 2]);
            fs = add3(fs, gi);
            ts = add3(ts, cross3(sub3(xi, ctr), gi));
        }
        sf[f] = fs;
        st[f] = ts;
        ftot = add3(ftot, fs);
        ttot = add3(ttot, ts);
    }
    ftot = make_float3(warp_sum_f(ftot.x), warp_sum_f(ftot.y), warp_sum_f(ftot.z));
    ttot = make_float3(warp_sum_f(ttot.x), warp_sum_f(ttot.y), warp_sum_f(ttot.z));
    __syncwarp();
    if (lane == 0) {
        for (int k = T - 1; k >= 0; --k) {
            const int4 tq = __ldg(&L.tors[k]);  // fragment, parent fragment, parent atom, bond atom
            const int ap = __ldg(&L.perm[tq.z]), am = __ldg(&L.perm[tq.w]);
            const float3 xp = make_float3(c.xc[3 * ap], c.xc[3 * ap + 1], c.xc[3 * ap + 2]);
            const float3 xm = make_float3(c.xc[3 * am], c.xc[3 * am + 1], c.xc[3 * am + 2]);
            float3 u = sub3(xm, xp);
            u = mul3(u, 1.f / sqrtf(dot3(u, u)));
            const float3 fs = sf[tq.x], ts = st[tq.x];
            g[7 + k] = dot3(u, sub3(ts, cross3(sub3(xm, ctr), fs)));
            sf[tq.y] = add3(sf[tq.y], fs);
            st[tq.y] = add3(st[tq.y], ts);
        }
        g[0] = ftot.x;
        g[1] = ftot.y;
        g[2] = ftot.z;
        const float len = sqrtf(q[3] * q[3] + q[4] * q[4] + q[5] * q[5] + q[6] * q[6]);
        const float w = q[3] / len;
        const float3 v = make_float3(q[4] / len, q[5] / len, q[6] / len);
        const float gw = -2.f * dot3(ttot, v);
        const float3 gv = mul3(add3(mul3(ttot, w), cross3(ttot, v)), 2.f);
        const float radial = gw * w + dot3(gv, v);
        g[3] = (gw - radial * w) / len;
        g[4] = (gv.x - radial * v.x) / len;
        g[5] = (gv.y - radial * v.y) / len;
        g[6] = (gv.z - radial * v.z) / len;
    }
    for (int r = lane; r < R; r += kWarp) g[7 + T + r] = c.gc[3 * N + r];
    __syncwarp();
}

// Energy and dE/dq at q = x0 + t d (d may be null: at x0); with gdot, *gdot = g . d.
// Out of line for the same reason as eval_pose.
static __device__ __noinline__ double dof_eval(DofClosure& c, double t, const float* d, float* g, double* gdot) {
    const DevLigand& L = *c.L;
    const int D = 7 + L.n_tors + c.env->rec.n_rotors;
    const int lane = c.lane;
    const float tf = static_cast<float>(t);
    for (int e = lane; e < D; e += kWarp) c.q[e] = d ? fmaf(d[e], tf, c.x0[e]) : c.x0[e];
    __syncwarp();
    dof_place(c, c.q);
    const double energy = eval_pose_body(*c.env, L, c.xc, nullptr, 0.f, c.gc, *c.b, lane);
    dof_pullback(c, c.q, g);
    if (gdot) {
        DS acc{0.f, 0.f};
        for (int e = lane; e < D; e += kWarp) ds_dot_acc(acc, g[e], d[e]);
        *gdot = ds_warp_sum(acc);
    }
    return energy;
}

__device__ __forceinline__ double closure_eval(DofClosure& c, double t, const float* d, float* g,
                                               double* gdot = nullptr) {
    ++c.nevals;
    return dof_eval(c, t, d, g, gdot);
}

// FP64 objective at the pose the variables x place; leaves that pose in c.xc.
__device__ __forceinline__ double closure_energy64(DofClosure& c, const float* x) {
    dof_place(c, x);
    return energy64(*c.env, *c.L, c.xc, *c.b, c.lane);
}

}  // namespace pxd
