// Differentiable empirical score: value, features and adjoint of one pose per warp, and
// (run on Dual numbers) the derivative of the adjoint along a direction of the
// coordinates: Hessian-vector product and mixed parameter derivatives.
//
// The terms are those of score_pose (root_scorer's leaf scorers, scorer.cpp:207-613),
// evaluated whatever their weight, plus the tabulated heavy-atom pair potential. The
// score is linear in 28 unweighted sums ("features"); the weights combine them
// (combine_features). The adjoint differentiates every pair / ring / donor term in
// closed form:
//   ramps      d ramp_down(v, lo, hi)/dv = -1/(hi - lo) on [lo, hi], 0 elsewhere;
//   clamped LJ  0 where the clamp is active;
//   angles     d acos(c)/dc = -1/sqrt(1 - c^2), 0 where the cosine is clamped;
//   rings      centroid gradient shared equally by the ring atoms, normal gradient
//              through n = (p1 - p0) x (p1 - p2) and its normalisation;
//   dihedrals  the analytic dihedral gradient of the force field (math.cpp:130-167).
// Everything is written over the scalar type S: S = float gives the score, features and
// gradients; S = Dual (coordinates carrying a direction v) gives the derivatives of the
// features, of the coordinate gradient (H v) and of the pair-table hat weights along v.
// A lane owns one receptor-side partner at a time; gradients of a ligand atom, ring or
// donor are reduced over the warp and added to the warp's gradient slice in shared
// memory (shared atomics, since torsion-strain lanes write any atom).
#pragma once

#include "device_dual.cuh"
#include "device_score.cuh"

namespace pxd {

constexpr int kNumW = PXD_NUM_SF_WEIGHTS;
constexpr int kNumF = PXD_NUM_SCORE_FEATURES;
constexpr int kTabN = PXD_PAIR_TYPES * PXD_PAIR_BINS;
constexpr float kTabInvWidth = static_cast<float>(1.0 / PXD_PAIR_BIN_WIDTH);
constexpr float kDegF = 57.29577951308232f;  // 180 / pi

enum Feature {
    F_COUL = 0, F_VDW = 1, F_ION = 2, F_PICAT = 4, F_STACK = 8, F_HBOND = 16,
    F_HYD = 24, F_TSTRAIN = 25, F_ROT = 26, F_TABLE = 27
};

__device__ __forceinline__ float ramp_down_d(float v, float lo, float hi) {
    return (v >= lo && v <= hi) ? -1.f / (hi - lo) : 0.f;
}
// get_reversed_linear_percent (math.h:196-215) over S
template <class S>
__device__ __forceinline__ S ramp_g(S v, float lo, float hi) {
    if (val(v) < lo) return lift<S>(1.f);
    if (val(v) <= hi) return 1.f - (v - lo) / (hi - lo);
    return lift<S>(0.f);
}
// ramp_down_c and its derivative in v
template <class S>
__device__ __forceinline__ S ramp_c_vd(S v, float c, float lo, float hi, float& dv) {
    if (val(v) < c) {
        dv = -ramp_down_d(c - val(v), lo, hi);
        return ramp_g(c - v, lo, hi);
    }
    dv = ramp_down_d(val(v) - c, lo, hi);
    return ramp_g(v - c, lo, hi);
}

__device__ __forceinline__ double warp_sum_fd(float v) {
    DS d{v, 0.f};
    return ds_warp_sum(d);
}

__device__ __forceinline__ void gadd(float4* G, int i, float3 g) {
    atomicAdd(&G[i].x, g.x);
    atomicAdd(&G[i].y, g.y);
    atomicAdd(&G[i].z, g.z);
}

// centroid and unit normal of a ligand ring (to_ring_centroid / to_ring_normal, scorer.cpp:128-172)
template <class S>
__device__ __forceinline__ void lig_ring_g(const float4* X, const float4* XT, const int* r,
                                           typename Vec<S>::type& c, typename Vec<S>::type& n) {
    int sz = 0;
    c = zero3<S>();
    for (int k = 0; k < 6; ++k) {
        const int a = __ldg(&r[k]);
        if (a < 0) break;
        c = add3(c, atom3<S>(X, XT, a));
        ++sz;
    }
    c = mul3(c, 1.f / sz);
    const auto p0 = atom3<S>(X, XT, __ldg(&r[0])), p1 = atom3<S>(X, XT, __ldg(&r[1])),
               p2 = atom3<S>(X, XT, __ldg(&r[2]));
    n = cross3(sub3(p1, p0), sub3(p1, p2));
    n = mul3(n, 1.f / sqrt_(dot3(n, n)));
}

// Gradient on a ligand ring's centroid (gc) and unit normal (gn) onto its atoms.
template <class S>
__device__ void ring_backward(const float4* X, const float4* XT, const int* r, typename Vec<S>::type gc,
                              typename Vec<S>::type gn, float4* G) {
    int sz = 0;
    while (sz < 6 && __ldg(&r[sz]) >= 0) ++sz;
    const auto share = mul3(gc, 1.f / sz);
    for (int k = 0; k < sz; ++k) gadd(G, __ldg(&r[k]), part3(share));
    const int i0 = __ldg(&r[0]), i1 = __ldg(&r[1]), i2 = __ldg(&r[2]);
    const auto a = sub3(atom3<S>(X, XT, i1), atom3<S>(X, XT, i0));
    const auto b = sub3(atom3<S>(X, XT, i1), atom3<S>(X, XT, i2));
    const auto n = cross3(a, b);
    const S len = sqrt_(dot3(n, n));
    const auto u = mul3(n, 1.f / len);
    const auto gnn = mul3(sub3(gn, mul3(u, dot3(gn, u))), 1.f / len);
    const auto ga = cross3(b, gnn), gb = cross3(gnn, a);
    gadd(G, i0, part3(mul3(ga, -1.f)));
    gadd(G, i1, part3(add3(ga, gb)));
    gadd(G, i2, part3(mul3(gb, -1.f)));
}

// stack_pair with the gradient of s * value on the ligand ring centroid and normal.
template <bool kGrad, class S>
__device__ __forceinline__ S stack_pair_adj(float3 rcf, float3 rnf, typename Vec<S>::type lc,
                                            typename Vec<S>::type ln, const float* p, float center, float s,
                                            typename Vec<S>::type& glc, typename Vec<S>::type& gln) {
    const auto rc = lift3<S>(rcf), rn = lift3<S>(rnf);
    const auto t = sub3(lc, rc);
    const S dist = sqrt_(dot3(t, t));
    if (val(dist) > p[1]) return lift<S>(0.f);
    const S D = ramp_g(dist, p[0], p[1]);
    const S dp1 = dot3(rn, t);
    const S s1 = sqrt_(dot3(t, t) - dp1 * dp1);
    const auto t2 = sub3(rc, lc);
    const S dp2 = dot3(ln, t2);
    const S s2 = sqrt_(dot3(t2, t2) - dp2 * dp2);
    const bool first = val(s1) < val(s2);
    const S sg = first ? s1 : s2;
    if (val(sg) > p[5]) return lift<S>(0.f);
    const S SG = ramp_g(sg, p[4], p[5]);
    const S c = min_(max_(dot3(rn, ln), -1.f), 1.f);
    S th = acos_(c) * kDegF;
    float sign = 1.f;
    if (180.f - val(th) < val(th)) {
        th = 180.f - th;
        sign = -1.f;
    }
    float dTH;
    const S TH = ramp_c_vd(th, center, p[2], p[3], dTH);
    if (kGrad && s != 0.f) {
        const float dD = ramp_down_d(val(dist), p[0], p[1]);
        const float dSG = ramp_down_d(val(sg), p[4], p[5]);
        auto g_lc = zero3<S>(), g_ln = zero3<S>();
        if (dD != 0.f && val(dist) > 0.f) g_lc = mul3(t, dD * SG * TH / dist);
        if (dSG != 0.f && val(sg) > 0.f) {
            const S k = D * dSG * TH / sg;
            if (first) {
                g_lc = add3(g_lc, mul3(sub3(t, mul3(rn, dp1)), k));
            } else {
                g_lc = sub3(g_lc, mul3(sub3(t2, mul3(ln, dp2)), k));
                g_ln = sub3(g_ln, mul3(t2, dp2 * k));
            }
        }
        const float dot = val(dot3(rn, ln));
        if (dTH != 0.f && dot > -1.f && dot < 1.f) {
            const S dth_dc = -kDegF / sqrt_(1.f - c * c);
            g_ln = add3(g_ln, mul3(rn, D * SG * dTH * sign * dth_dc));
        }
        glc = sub3(glc, mul3(g_lc, s));  // value = -D * SG * TH
        gln = sub3(gln, mul3(g_ln, s));
    }
    return -(D * SG * TH);
}

// hbond_pair with the gradient of s * value on the donor, hydrogen and acceptor.
template <bool kGrad, class S>
__device__ __forceinline__ S hbond_pair_adj(typename Vec<S>::type dpos, typename Vec<S>::type hpos,
                                            typename Vec<S>::type apos, const float* p, float s,
                                            typename Vec<S>::type& gd, typename Vec<S>::type& gh,
                                            typename Vec<S>::type& ga) {
    const auto ha = sub3(hpos, apos);
    const S D = sqrt_(dot3(ha, ha));
    float ddd;
    const S dd = ramp_c_vd(D, p[4], p[0], p[1], ddd);
    if (val(dd) < kEpsF) return lift<S>(0.f);
    const auto u = sub3(dpos, hpos), v = sub3(apos, hpos);
    const S lu = sqrt_(dot3(u, u)), lv = sqrt_(dot3(v, v));
    const S L = lu * lv + kEpsF;
    const S uv = dot3(u, v);
    const S cr = uv / L;
    const S c = min_(max_(cr, -1.f), 1.f);
    const S ang = acos_(c) * kDegF;
    float dAR;
    const S AR = ramp_c_vd(ang, p[5], p[2], p[3], dAR);
    if (kGrad && s != 0.f) {
        if (ddd != 0.f && val(D) > 0.f) {
            const auto g = mul3(ha, -s * ddd * AR / D);  // d(-dd * AR)/dh
            gh = add3(gh, g);
            ga = sub3(ga, g);
        }
        if (dAR != 0.f && val(cr) > -1.f && val(cr) < 1.f && val(lu) > 0.f && val(lv) > 0.f) {
            const S k = -s * dd * dAR * (-kDegF / sqrt_(1.f - c * c));
            const auto dcu = sub3(mul3(v, 1.f / L), mul3(u, uv * lv / (lu * L * L)));
            const auto dcv = sub3(mul3(u, 1.f / L), mul3(v, uv * lu / (lv * L * L)));
            gd = add3(gd, mul3(dcu, k));
            ga = add3(ga, mul3(dcv, k));
            gh = sub3(gh, mul3(add3(dcu, dcv), k));
        }
    }
    return -(dd * AR);
}

// Warp sum of a vector of S (both parts for Dual).
__device__ __forceinline__ float3 warp_sum_v(float3 v) { return warp_sum3(v); }
__device__ __forceinline__ D3 warp_sum_v(D3 v) {
    const float3 a = warp_sum3(val3(v)), b = warp_sum3(part3(v));
    return {Dual{a.x, b.x}, Dual{a.y, b.y}, Dual{a.z, b.z}};
}

// S = sum of weights x features (the weights take the places of root_scorer's
// coefficients and of the per-term scales and sub-coefficients).
__device__ __forceinline__ double combine_features(const double* w, const double* f) {
    double s = w[PXD_W_COEF + PXD_TERM_COULOMB] * f[F_COUL];
    s += w[PXD_W_COEF + PXD_TERM_VDW] * w[PXD_W_VDW_SCALE] * f[F_VDW];
    s += w[PXD_W_COEF + PXD_TERM_IONIC] * (w[PXD_W_IONIC] * f[F_ION] + w[PXD_W_IONIC + 1] * f[F_ION + 1]);
    double t = 0.0;
    for (int k = 0; k < 4; ++k) t += w[PXD_W_PICAT + k] * f[F_PICAT + k];
    s += w[PXD_W_COEF + PXD_TERM_PI_CATION] * t;
    for (int q = 0; q < 2; ++q) {
        t = 0.0;
        for (int k = 0; k < 4; ++k) t += w[PXD_W_STACK + 4 * q + k] * f[F_STACK + 4 * q + k];
        s += w[PXD_W_COEF + PXD_TERM_F2F + q] * t;
    }
    t = 0.0;
    for (int k = 0; k < 8; ++k) t += w[PXD_W_HBOND + k] * f[F_HBOND + k];
    s += w[PXD_W_COEF + PXD_TERM_HBOND] * w[PXD_W_HBOND_SCALE] * t;
    s += w[PXD_W_COEF + PXD_TERM_HYDROPHOBIC] * w[PXD_W_HYDRO_SCALE] * f[F_HYD];
    s += w[PXD_W_COEF + PXD_TERM_TSTRAIN] * f[F_TSTRAIN];
    s += w[PXD_W_COEF + PXD_TERM_ROTATABLE] * f[F_ROT];
    return s + f[F_TABLE];
}

// g * dS/dw, added into dw[36].
__device__ __forceinline__ void combine_grad(const double* w, const double* f, double g, double* dw) {
    double hb = 0.0;
    for (int k = 0; k < 8; ++k) hb += w[PXD_W_HBOND + k] * f[F_HBOND + k];
    double pc = 0.0;
    for (int k = 0; k < 4; ++k) pc += w[PXD_W_PICAT + k] * f[F_PICAT + k];
    double st[2] = {0.0, 0.0};
    for (int q = 0; q < 2; ++q)
        for (int k = 0; k < 4; ++k) st[q] += w[PXD_W_STACK + 4 * q + k] * f[F_STACK + 4 * q + k];
    double d[kNumW];
    d[PXD_W_COEF + PXD_TERM_COULOMB] = f[F_COUL];
    d[PXD_W_COEF + PXD_TERM_VDW] = w[PXD_W_VDW_SCALE] * f[F_VDW];
    d[PXD_W_COEF + PXD_TERM_IONIC] = w[PXD_W_IONIC] * f[F_ION] + w[PXD_W_IONIC + 1] * f[F_ION + 1];
    d[PXD_W_COEF + PXD_TERM_PI_CATION] = pc;
    d[PXD_W_COEF + PXD_TERM_F2F] = st[0];
    d[PXD_W_COEF + PXD_TERM_E2F] = st[1];
    d[PXD_W_COEF + PXD_TERM_HBOND] = w[PXD_W_HBOND_SCALE] * hb;
    d[PXD_W_COEF + PXD_TERM_HYDROPHOBIC] = w[PXD_W_HYDRO_SCALE] * f[F_HYD];
    d[PXD_W_COEF + PXD_TERM_TSTRAIN] = f[F_TSTRAIN];
    d[PXD_W_COEF + PXD_TERM_ROTATABLE] = f[F_ROT];
    d[PXD_W_COEF + PXD_TERM_GBSA] = 0.0;
    d[PXD_W_VDW_SCALE] = w[PXD_W_COEF + PXD_TERM_VDW] * f[F_VDW];
    d[PXD_W_HYDRO_SCALE] = w[PXD_W_COEF + PXD_TERM_HYDROPHOBIC] * f[F_HYD];
    d[PXD_W_HBOND_SCALE] = w[PXD_W_COEF + PXD_TERM_HBOND] * hb;
    for (int k = 0; k < 2; ++k) d[PXD_W_IONIC + k] = w[PXD_W_COEF + PXD_TERM_IONIC] * f[F_ION + k];
    for (int k = 0; k < 4; ++k) d[PXD_W_PICAT + k] = w[PXD_W_COEF + PXD_TERM_PI_CATION] * f[F_PICAT + k];
    for (int q = 0; q < 2; ++q)
        for (int k = 0; k < 4; ++k)
            d[PXD_W_STACK + 4 * q + k] = w[PXD_W_COEF + PXD_TERM_F2F + q] * f[F_STACK + 4 * q + k];
    for (int k = 0; k < 8; ++k)
        d[PXD_W_HBOND + k] = w[PXD_W_COEF + PXD_TERM_HBOND] * w[PXD_W_HBOND_SCALE] * f[F_HBOND + k];
    for (int k = 0; k < kNumW; ++k) dw[k] += g * d[k];
}

struct AdjPose {
    const float* wf;          // [36] weights (FP32 copies, shared)
    const float* tab;         // [32 * 256] pair table or NULL
    float* tgrad;             // [32 * 256] shared per-block table gradient or NULL
    float g;                  // dL/dS of this pose
};

template <class S>
__device__ __forceinline__ typename Vec<S>::type rec_pos_g(const DevRecScore& rs, const float4* loc_xyz, int j) {
    return lift3<S>(rec_pos(rs, loc_xyz, j));
}

// Features of the pose in X (every lane returns the same f[28]); with kGrad, adds
// g * dS/dx into G and g * dS/dT into the table gradient. With S = Dual (X carrying the
// direction XT), the same quantities' derivatives along XT instead.
template <bool kGrad, class S>
__device__ void score_adjoint_pose(const ScoreEnv& env, const DevLigand& L, const float4* X, const float4* XT,
                                   const float4* loc_xyz, const AdjPose& ap, float4* G, int lane, double* f) {
    using V = typename Vec<S>::type;
    const DevRecScore& rs = env.rs;
    const DevLigScore& ls = L.score;
    const DevSf& sf = *env.sf;
    const float* W = ap.wf;
    const float g = ap.g;
    const int N = L.n_atoms;
    const float s_coul = g * W[PXD_W_COEF + PXD_TERM_COULOMB] * kCoulombF;
    const float s_vdw = g * W[PXD_W_COEF + PXD_TERM_VDW] * W[PXD_W_VDW_SCALE];
    const bool table = ap.tab && ls.pclass;  // receptor atoms without a class carry -1
    // Coulomb, clamped LJ and the pair table over every ligand x receptor pair
    DS a_coul{0.f, 0.f}, a_vdw{0.f, 0.f}, a_tab{0.f, 0.f};
    for (int i = 0; i < N; ++i) {
        const V xi = atom3<S>(X, XT, i);
        const float qi = __ldg(&L.charge[i]);
        const float2 ti = sf.vdw_type[__ldg(&L.type[i])];
        const float sei4 = sqrtf(ti.y) * 4.f;
        const int ci = table ? __ldg(&ls.pclass[i]) : -1;
        S ec = lift<S>(0.f), ev = lift<S>(0.f), et = lift<S>(0.f);
        V gi = zero3<S>();
#pragma unroll 2
        for (int j = lane; j < rs.n_all; j += kWarp) {
            const float4 rj = __ldg(&rs.all_xyzq[j]);
            const float4 pr = __ldg(&rs.pair_rec[j]);  // sigma, sqrt(eps), class, local
            const int l = __float_as_int(pr.w);
            const V dv = sub3(xi, lift3<S>(l >= 0 ? xyz(loc_xyz[l]) : xyz(rj)));
            const S r2 = dot3(dv, dv);
            // 1 / (d + 1e-20) of the reference is 1 / d away from d = 0
            const S rinv = val(r2) > 0.f ? rsqrt_(r2) : lift<S>(1.f / kEpsF);
            const S d = r2 * rinv;
            ec = fma_(rinv, qi * rj.w, ec);
            const S sr = (ti.x + pr.x) * 0.5f * rinv;
            const S s2 = sr * sr;
            const S u6 = s2 * s2 * s2;
            const float fused = sei4 * pr.y;
            const S v = (u6 * u6 - u6) * fused;
            ev = ev + min_(max_(v, -sf.vdw_cutoff), sf.vdw_cutoff);
            S de_dd = lift<S>(0.f);
            if (kGrad) {
                de_dd = (-s_coul * qi * rj.w) * (rinv * rinv);
                if (val(v) <= sf.vdw_cutoff && val(v) >= -sf.vdw_cutoff)
                    de_dd = de_dd - (s_vdw * fused) * rinv * (12.f * u6 * u6 - 6.f * u6);
            }
            if (ci >= 0) {
                const int cj = __float_as_int(pr.z);
                const S tt = d * kTabInvWidth;
                if (cj >= 0 && val(tt) < static_cast<float>(PXD_PAIR_BINS - 1)) {
                    const int b = static_cast<int>(val(tt));
                    const S fr = tt - static_cast<float>(b);
                    const int p = (ci + cj) * PXD_PAIR_BINS + b;
                    const float t0 = __ldg(&ap.tab[p]), t1 = __ldg(&ap.tab[p + 1]);
                    et = et + fma_(fr, t1 - t0, lift<S>(t0));
                    if (kGrad) {
                        de_dd = de_dd + g * (t1 - t0) * kTabInvWidth;
                        if (ap.tgrad) {
                            atomicAdd(&ap.tgrad[p], part(g * (1.f - fr)));
                            atomicAdd(&ap.tgrad[p + 1], part(g * fr));
                        }
                    }
                }
            }
            if (kGrad) gi = add3(gi, mul3(dv, de_dd * rinv));
        }
        ds_add(a_coul, part(ec) * kCoulombF);
        ds_add(a_vdw, part(ev));
        ds_add(a_tab, part(et));
        if (kGrad) {
            const float3 gs = warp_sum3(part3(gi));
            if (lane == 0) gadd(G, i, gs);
        }
    }
    // hydrophobic contacts (scorer.cpp:278-311)
    DS a_hyd{0.f, 0.f};
    {
        const float sg = g * W[PXD_W_COEF + PXD_TERM_HYDROPHOBIC] * W[PXD_W_HYDRO_SCALE];
        for (int a = 0; a < ls.n_hyd; ++a) {
            const int i = __ldg(&ls.hyd[a]);
            const V xi = atom3<S>(X, XT, i);
            const float s1 = sf.vdw_sigma_raw[__ldg(&L.type[i])];
            S e = lift<S>(0.f);
            V gi = zero3<S>();
            for (int b = lane; b < rs.n_hyd; b += kWarp) {
                const int j = __ldg(&rs.hyd[b]);
                const float r1 = (s1 + __ldg(&rs.all_se[j]).x) * sf.hydro_factor + sf.hydro_min;
                const V dv = sub3(xi, rec_pos_g<S>(rs, loc_xyz, j));
                const S d = sqrt_(dot3(dv, dv));
                e = e - ramp_g(d, r1, r1 + sf.hydro_max);
                if (kGrad && val(d) > 0.f)
                    gi = add3(gi, mul3(dv, (-sg * ramp_down_d(val(d), r1, r1 + sf.hydro_max)) / d));
            }
            ds_add(a_hyd, part(e));
            if (kGrad) {
                const float3 gs = warp_sum3(part3(gi));
                if (lane == 0) gadd(G, i, gs);
            }
        }
    }
    // ionic (scorer.cpp:313-368): ligand cations x receptor anions, ligand anions x receptor cations
    float f_ion[2] = {0.f, 0.f};
    for (int k = 0; k < 2; ++k) {
        const float sk = g * W[PXD_W_COEF + PXD_TERM_IONIC] * W[PXD_W_IONIC + k];
        const int na = k == 0 ? ls.n_cat : ls.n_an;
        const int* la = k == 0 ? ls.cat : ls.an;
        const int nb = k == 0 ? rs.n_an : rs.n_cat;
        const int* rb = k == 0 ? rs.an : rs.cat;
        for (int a = 0; a < na; ++a) {
            const int i = __ldg(&la[a]);
            const V xi = atom3<S>(X, XT, i);
            V gi = zero3<S>();
            for (int b = lane; b < nb; b += kWarp) {
                const V dv = sub3(xi, rec_pos_g<S>(rs, loc_xyz, __ldg(&rb[b])));
                const S d = sqrt_(dot3(dv, dv));
                f_ion[k] -= part(ramp_g(d, sf.ionic[k][0], sf.ionic[k][1]));
                if (kGrad && val(d) > 0.f)
                    gi = add3(gi, mul3(dv, (-sk * ramp_down_d(val(d), sf.ionic[k][0], sf.ionic[k][1])) / d));
            }
            if (kGrad) {
                const float3 gs = warp_sum3(part3(gi));
                if (lane == 0) gadd(G, i, gs);
            }
        }
    }
    // cation-pi (scorer.cpp:370-462)
    float f_pc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < 2; ++k) {  // ligand cations x receptor ring5 / ring6 centroids
        const float sk = g * W[PXD_W_COEF + PXD_TERM_PI_CATION] * W[PXD_W_PICAT + k];
        const int nr = k == 0 ? rs.n_r5 : rs.n_r6;
        const float4* rc = k == 0 ? rs.r5c : rs.r6c;
        for (int a = 0; a < ls.n_cat; ++a) {
            const int i = __ldg(&ls.cat[a]);
            const V xi = atom3<S>(X, XT, i);
            V gi = zero3<S>();
            for (int b = lane; b < nr; b += kWarp) {
                const V dv = sub3(xi, lift3<S>(xyz(__ldg(&rc[b]))));
                const S d = sqrt_(dot3(dv, dv));
                f_pc[k] -= part(ramp_g(d, sf.picat[k][0], sf.picat[k][1]));
                if (kGrad && val(d) > 0.f)
                    gi = add3(gi, mul3(dv, (-sk * ramp_down_d(val(d), sf.picat[k][0], sf.picat[k][1])) / d));
            }
            if (kGrad) {
                const float3 gs = warp_sum3(part3(gi));
                if (lane == 0) gadd(G, i, gs);
            }
        }
    }
    for (int r = 0; r < ls.n_r5 + ls.n_r6; ++r) {  // ligand ring centroids x receptor cations
        const bool five = r < ls.n_r5;
        const int* ring = five ? ls.r5 + 6 * r : ls.r6 + 6 * (r - ls.n_r5);
        const int k = five ? 2 : 3;
        const float sk = g * W[PXD_W_COEF + PXD_TERM_PI_CATION] * W[PXD_W_PICAT + k];
        V c, n;
        lig_ring_g<S>(X, XT, ring, c, n);
        V gc = zero3<S>();
        for (int b = lane; b < rs.n_cat; b += kWarp) {
            const V dv = sub3(c, rec_pos_g<S>(rs, loc_xyz, __ldg(&rs.cat[b])));
            const S d = sqrt_(dot3(dv, dv));
            f_pc[k] -= part(ramp_g(d, sf.picat[k][0], sf.picat[k][1]));
            if (kGrad && val(d) > 0.f)
                gc = add3(gc, mul3(dv, (-sk * ramp_down_d(val(d), sf.picat[k][0], sf.picat[k][1])) / d));
        }
        if (kGrad) {
            // the ring backward is linear in gc: reduce both parts of gc, then map
            gc = warp_sum_v(gc);
            if (lane == 0) ring_backward<S>(X, XT, ring, gc, zero3<S>(), G);
        }
    }
    // pi stacking, face-to-face (centre 0) and edge-to-face (centre 90) (scorer.cpp:638-724)
    float f_st[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int w = 0; w < 2; ++w) {
        const float center = w == 0 ? 0.f : 90.f;
        for (int r = 0; r < ls.n_r5 + ls.n_r6; ++r) {
            const bool five = r < ls.n_r5;
            const int* ring = five ? ls.r5 + 6 * r : ls.r6 + 6 * (r - ls.n_r5);
            V lc, ln;
            lig_ring_g<S>(X, XT, ring, lc, ln);
            const int k5 = five ? 0 : 2, k6 = five ? 1 : 3;
            const float s5 = g * W[PXD_W_COEF + PXD_TERM_F2F + w] * W[PXD_W_STACK + 4 * w + k5];
            const float s6 = g * W[PXD_W_COEF + PXD_TERM_F2F + w] * W[PXD_W_STACK + 4 * w + k6];
            V glc = zero3<S>(), gln = zero3<S>();
            for (int b = lane; b < rs.n_r5; b += kWarp)
                f_st[4 * w + k5] += part(stack_pair_adj<kGrad, S>(xyz(__ldg(&rs.r5c[b])), xyz(__ldg(&rs.r5n[b])), lc,
                                                                  ln, sf.stack[w][k5], center, s5, glc, gln));
            for (int b = lane; b < rs.n_r6; b += kWarp)
                f_st[4 * w + k6] += part(stack_pair_adj<kGrad, S>(xyz(__ldg(&rs.r6c[b])), xyz(__ldg(&rs.r6n[b])), lc,
                                                                  ln, sf.stack[w][k6], center, s6, glc, gln));
            if (kGrad) {
                glc = warp_sum_v(glc);
                gln = warp_sum_v(gln);
                if (lane == 0) ring_backward<S>(X, XT, ring, glc, gln, G);
            }
        }
    }
    // hydrogen bonds, 8 donor/acceptor classes (scorer.cpp:464-577)
    float f_hb[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const float s_hb = g * W[PXD_W_COEF + PXD_TERM_HBOND] * W[PXD_W_HBOND_SCALE];
    for (int c = 0; c < 2; ++c) {  // ligand donors (charged, neutral) x receptor acceptors
        const int nd = c == 0 ? ls.n_donc : ls.n_donn;
        const int2* dl = c == 0 ? ls.donc : ls.donn;
        for (int a = 0; a < nd; ++a) {
            const int2 dh = __ldg(&dl[a]);
            const V dp = atom3<S>(X, XT, dh.x), hp = atom3<S>(X, XT, dh.y);
            V gd = zero3<S>(), gh = zero3<S>(), gdummy = zero3<S>();
            for (int u = 0; u < 2; ++u) {
                const int na = u == 0 ? rs.n_accc : rs.n_accn;
                const int* al = u == 0 ? rs.accc : rs.accn;
                const int k = 2 * c + u;
                const float sk = s_hb * W[PXD_W_HBOND + k];
                for (int b = lane; b < na; b += kWarp)
                    f_hb[k] += part(hbond_pair_adj<kGrad, S>(dp, hp, rec_pos_g<S>(rs, loc_xyz, __ldg(&al[b])),
                                                             sf.hbond[k], sk, gd, gh, gdummy));
            }
            if (kGrad) {
                const float3 sd = warp_sum3(part3(gd)), sh = warp_sum3(part3(gh));
                if (lane == 0) {
                    gadd(G, dh.x, sd);
                    gadd(G, dh.y, sh);
                }
            }
        }
    }
    for (int u = 0; u < 2; ++u) {  // ligand acceptors (charged, neutral) x receptor donors
        const int na = u == 0 ? ls.n_accc : ls.n_accn;
        const int* al = u == 0 ? ls.accc : ls.accn;
        for (int a = 0; a < na; ++a) {
            const int i = __ldg(&al[a]);
            const V apos = atom3<S>(X, XT, i);
            V ga = zero3<S>(), gd = zero3<S>(), gh = zero3<S>();
            for (int c = 0; c < 2; ++c) {
                const int nd = c == 0 ? rs.n_donc : rs.n_donn;
                const int2* dl = c == 0 ? rs.donc : rs.donn;
                const int k = 4 + 2 * c + u;
                const float sk = s_hb * W[PXD_W_HBOND + k];
                for (int b = lane; b < nd; b += kWarp) {
                    const int2 dh = __ldg(&dl[b]);
                    f_hb[k] += part(hbond_pair_adj<kGrad, S>(rec_pos_g<S>(rs, loc_xyz, dh.x),
                                                             rec_pos_g<S>(rs, loc_xyz, dh.y), apos, sf.hbond[k], sk,
                                                             gd, gh, ga));
                }
            }
            if (kGrad) {
                const float3 sa = warp_sum3(part3(ga));
                if (lane == 0) gadd(G, i, sa);
            }
        }
    }
    // torsion strain (scorer.cpp:579-613): one entry per lane
    DS a_ts{0.f, 0.f};
    {
        const float s_ts = g * W[PXD_W_COEF + PXD_TERM_TSTRAIN];
        const float kPi = 3.14159265358979f;
        for (int t = lane; t < ls.n_ts; t += kWarp) {
            const float4 co = __ldg(&ls.ts_coef[t]);
            const int2 rg = __ldg(&ls.ts_range[t]);
            int cnt = 0;
            while (cnt < rg.y) {
                const int4 q = __ldg(&ls.ts_quad[rg.x + cnt]);
                if (q.x == q.y) break;
                ++cnt;
            }
            if (cnt == 0) continue;
            S tmp = lift<S>(0.f);
            const float inv = 1.f / cnt;
            for (int j = 0; j < cnt; ++j) {
                const int4 q = __ldg(&ls.ts_quad[rg.x + j]);
                const V pi = atom3<S>(X, XT, q.x), pj = atom3<S>(X, XT, q.y), pk = atom3<S>(X, XT, q.z),
                        pl = atom3<S>(X, XT, q.w);
                // signed dihedral (math.cpp:112-128) and its gradient (math.cpp:130-167)
                const V rij = sub3(pj, pi), rkj = sub3(pj, pk), rkl = sub3(pl, pk);
                const V m = cross3(rij, rkj), n = cross3(rkj, rkl);
                const V wv = cross3(m, n);
                const S phi = atan2_(sqrt_(dot3(wv, wv)), dot3(m, n) + kEpsF);
                const S th = val(dot3(rij, n)) < 0.f ? phi : -phi;
                tmp = tmp + (1.f + cos_(th)) * co.x + (1.f + cos_(2.f * th - kPi)) * co.y +
                      (1.f + cos_(3.f * th)) * co.z + (1.f + cos_(4.f * th - kPi)) * co.w;
                if (kGrad && s_ts != 0.f) {
                    const S df = -(sin_(th) * co.x + 2.f * sin_(2.f * th - kPi) * co.y + 3.f * sin_(3.f * th) * co.z +
                                   4.f * sin_(4.f * th - kPi) * co.w);
                    const S mm = dot3(m, m), nn = dot3(n, n), nrkj2 = dot3(rkj, rkj);
                    if (val(mm) > 0.f && val(nn) > 0.f && val(nrkj2) > 0.f) {
                        const S nrkj = sqrt_(nrkj2);
                        const V gi = mul3(m, nrkj / mm), gl = mul3(n, -nrkj / nn);
                        const S pp = dot3(rij, rkj) / nrkj2, qq = dot3(rkj, rkl) / nrkj2;
                        const V sv = sub3(mul3(gi, pp), mul3(gl, qq));
                        const V gj = mul3(sub3(gi, sv), -1.f), gk = mul3(add3(gl, sv), -1.f);
                        const S k = df * (s_ts * inv);
                        gadd(G, q.x, part3(mul3(gi, k)));
                        gadd(G, q.y, part3(mul3(gj, k)));
                        gadd(G, q.z, part3(mul3(gk, k)));
                        gadd(G, q.w, part3(mul3(gl, k)));
                    }
                }
            }
            ds_add(a_ts, part(tmp) * inv);
        }
    }
    f[F_COUL] = ds_warp_sum(a_coul);
    f[F_VDW] = ds_warp_sum(a_vdw);
    for (int k = 0; k < 2; ++k) f[F_ION + k] = warp_sum_fd(f_ion[k]);
    for (int k = 0; k < 4; ++k) f[F_PICAT + k] = warp_sum_fd(f_pc[k]);
    for (int k = 0; k < 8; ++k) f[F_STACK + k] = warp_sum_fd(f_st[k]);
    for (int k = 0; k < 8; ++k) f[F_HBOND + k] = warp_sum_fd(f_hb[k]);
    f[F_HYD] = ds_warp_sum(a_hyd);
    f[F_TSTRAIN] = ds_warp_sum(a_ts);
    f[F_ROT] = IsDual<S>::value ? 0.0 : -1.0 / (2.620643 + ls.n_rot);  // constant: no tangent
    f[F_TABLE] = ds_warp_sum(a_tab);
}

}  // namespace pxd
