// Warp-cooperative energy + gradient of one pose (device code shared by the score,
// L-BFGS and Monte-Carlo kernels).
//
// One warp owns one pose. Ligand and receptor-local coordinates and gradient
// accumulators live in the warp's shared-memory slice; term lists are walked 32 at a
// time (one term per lane; the host ordered them so that no atom repeats within a
// 32-term round) and gradients are added with shared-memory atomics. Energies are
// summed per lane in a compensated FP32 pair (two-sum) and reduced across the warp,
// then returned as double.
//
// Each block restates one reference routine in FP32:
//   bonds / angles / dihedrals / pairs   interaction.cpp:27-168, pair.h:25-60, math.cpp:96-167
//   grid lookup with out-of-box penalty  grid.cpp:197-303
//   explicit inter pairs                 interaction.cpp:202-257
//   receptor rotors and chain rule       interaction.cpp:316-350, math.cpp:62-94
#pragma once

#include "pxd_internal.h"

namespace pxd {

constexpr float kCoulombF = 332.0637141491396f;
constexpr float kEpsF = 1e-20f;  // kParamEpsilon, math.h:128
constexpr unsigned kFull = 0xffffffffu;

// ----------------------------------------------------------- compensated sums
struct DS {
    float hi, lo;
};

__device__ __forceinline__ void ds_add(DS& a, float b) {
    // Knuth two-sum: s + err == a.hi + b exactly
    const float s = a.hi + b;
    const float bb = s - a.hi;
    const float err = (a.hi - (s - bb)) + (b - bb);
    a.hi = s;
    a.lo += err;
}

__device__ __forceinline__ void ds_add_ds(DS& a, const DS& b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    const float err = (a.hi - (s - bb)) + (b.hi - bb);
    a.hi = s;
    a.lo = a.lo + b.lo + err;
}

// Sum over the warp, the same on every lane: at each butterfly level both partners add the
// same two pairs, and the result does not depend on their order (two-sum's error term is
// the exact rounding error of hi + hi, and lo + lo commutes), so no final broadcast is
// needed.
__device__ __forceinline__ double ds_warp_sum(DS v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        DS o;
        o.hi = __shfl_xor_sync(kFull, v.hi, off);
        o.lo = __shfl_xor_sync(kFull, v.lo, off);
        ds_add_ds(v, o);
    }
    return static_cast<double>(v.hi) + static_cast<double>(v.lo);
}

// The same butterfly, the compensated pair kept (identical on every lane).
__device__ __forceinline__ DS ds_warp_reduce(DS v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        DS o;
        o.hi = __shfl_xor_sync(kFull, v.hi, off);
        o.lo = __shfl_xor_sync(kFull, v.lo, off);
        ds_add_ds(v, o);
    }
    return v;
}

// Butterfly reductions leave every lane with the same value (max and a two-operand sum
// commute), so they need no final broadcast.
// The warp sum rounded once to FP32 (hi + lo), without leaving the FP32 pipe.
__device__ __forceinline__ float ds_warp_sum_f(DS v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        DS o;
        o.hi = __shfl_xor_sync(kFull, v.hi, off);
        o.lo = __shfl_xor_sync(kFull, v.lo, off);
        ds_add_ds(v, o);
    }
    return v.hi + v.lo;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, off));
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    return v;
}

// One step of a dot product with the exact FP32 product (fma) accumulated as a
// compensated pair: ~44 significant bits, on the FP32 pipe.
__device__ __forceinline__ void ds_dot_acc(DS& acc, float x, float y) {
    const float p = x * y;
    const float pe = fmaf(x, y, -p);
    ds_add(acc, p);
    acc.lo += pe;
}

__device__ __forceinline__ double vabssum(const float* a, int D, int lane) {
    DS acc{0.f, 0.f};
    for (int e = lane; e < D; e += kWarp) ds_add(acc, fabsf(a[e]));
    return ds_warp_sum(acc);
}

__device__ __forceinline__ float vabsmax(const float* a, int D, int lane) {
    float m = 0.f;
    for (int e = lane; e < D; e += kWarp) m = fmaxf(m, fabsf(a[e]));
    return warp_max(m);
}

__device__ __forceinline__ void vcopy(float* dst, const float* src, int D, int lane) {
    for (int e = lane; e < D; e += kWarp) dst[e] = src[e];
    __syncwarp();
}

// ------------------------------------------------------------------ vectors
__device__ __forceinline__ float3 sub3(float3 a, float3 b) {
    return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float3 add3(float3 a, float3 b) {
    return make_float3(a.x + b.x, a.y + b.y, a.z + b.z);
}
__device__ __forceinline__ float3 mul3(float3 a, float s) {
    return make_float3(a.x * s, a.y * s, a.z * s);
}
__device__ __forceinline__ float dot3(float3 a, float3 b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }

__device__ __forceinline__ void atomic_add3(float4* p, float3 g) {
    atomicAdd(&p->x, g.x);
    atomicAdd(&p->y, g.y);
    atomicAdd(&p->z, g.z);
}
__device__ __forceinline__ void atomic_sub3(float4* p, float3 g) {
    atomicAdd(&p->x, -g.x);
    atomicAdd(&p->y, -g.y);
    atomicAdd(&p->z, -g.z);
}

// Rodrigues rotation and its theta-derivative (math.cpp:62-94), rows of 3.
struct Mat3 {
    float3 r0, r1, r2;
};
__device__ __forceinline__ float3 mat_apply(const Mat3& m, float3 v) {
    return make_float3(dot3(m.r0, v), dot3(m.r1, v), dot3(m.r2, v));
}
__device__ __forceinline__ void rotation_and_jacobian(float3 k, float theta, Mat3& R, Mat3& J) {
    float st, ct;
    sincosf(theta, &st, &ct);
    const float omc = 1.f - ct;
    const float kxo = k.x * omc, kyo = k.y * omc, kzo = k.z * omc;
    const float kxs = k.x * st, kys = k.y * st, kzs = k.z * st;
    R.r0 = make_float3(ct + k.x * kxo, k.y * kxo - kzs, kys + k.z * kxo);
    R.r1 = make_float3(kzs + k.x * kyo, ct + k.y * kyo, k.z * kyo - kxs);
    R.r2 = make_float3(k.x * kzo - kys, kxs + k.y * kzo, ct + k.z * kzo);
    J.r0 = make_float3(-st + k.x * kxs, -k.z * ct + k.x * kys, k.y * ct + k.x * kzs);
    J.r1 = make_float3(k.z * ct + k.y * kxs, -st + k.y * kys, -k.x * ct + k.y * kzs);
    J.r2 = make_float3(-k.y * ct + k.z * kxs, k.x * ct + k.z * kys, -st + k.z * kzs);
}

// ------------------------------------------------------------- term kernels
// Adds `g` to the gradient record p (shared memory): one 16-byte load and store.
__device__ __forceinline__ void add_rec(float4* p, float3 g) {
    float4 v = *p;
    v.x += g.x;
    v.y += g.y;
    v.z += g.z;
    *p = v;
}
__device__ __forceinline__ void sub_rec(float4* p, float3 g) {
    float4 v = *p;
    v.x -= g.x;
    v.y -= g.y;
    v.z -= g.z;
    *p = v;
}

// Squared pair distances are floored at 1e-4 A^2 (r = 0.01 A) in the FP32 pair terms: below
// r ~ 3e-3 A the 12th power overflows FP32 (the FP64 reference stays finite down to 1e-25 A),
// and the inf energy / NaN gradient would end the optimisation as a NaN. Only such near-
// coincident atoms see the floor; the reported FP64 energy (energy64.cuh) has none.
constexpr float kPairR2Floor = 1e-4f;

// One pre-combined pair (p = A, C, S2): energy into `en`, returns dE/dr_ij * r_ij / r
// (the gradient of atom j; atom i takes its negative).
__device__ __forceinline__ float3 pair_grad(float4 p, float4 xi, float4 xj, float& en) {
    const float3 rij = sub3(xyz(xj), xyz(xi));
    const float r2 = fmaxf(dot3(rij, rij), kPairR2Floor);
    const float rinv = rsqrtf(r2);
    const float rinv2 = rinv * rinv;
    const float x = p.z * rinv2;
    const float u6 = x * x * x;
    const float u12 = u6 * u6;
    const float ec = p.x * rinv;
    en = fmaf(p.y, u12 - u6, ec);
    const float de_dr_r = (p.y * (6.f * u6 - 12.f * u12) - ec) * rinv2;
    return mul3(rij, de_dr_r);
}

// Adds the bonded and non-bonded terms of `t` over coordinates `X`. The gradient of
// the atom in position k of a term goes to array k: G[k * gs + atom] (shared memory).
// Within a round the atoms of each position are distinct (host scheduling), so the
// lanes of a round update distinct records with plain loads and stores; a warp
// barrier between rounds orders a record's updates from different rounds. Padded
// slots (-1) compute nothing. Every loop runs a multiple of 32 slots, so all lanes
// meet every barrier. The caller sums the arrays. Matches
// intra_molecular_interactions::put_gradients.
__device__ __forceinline__ void topo_terms(const DevTopo& t, const float4* X, float4* G, int gs, DS& e,
                                           int lane) {
    float4* G0 = G;
    float4* G1 = G + gs;
    float4* G2 = G + 2 * gs;
    float4* G3 = G + 3 * gs;
    __syncwarp();
    // harmonic bonds (interaction.cpp:27-47)
    for (int s = lane; s < t.n_bond_slots; s += kWarp) {
        const int2 ij = __ldg(&t.bond_ij[s]);
        if (ij.x >= 0) {
            const float2 p = __ldg(&t.bond_p[s]);
            const float3 d = sub3(xyz(X[ij.y]), xyz(X[ij.x]));
            const float r = sqrtf(dot3(d, d));
            const float dr = r - p.y;
            ds_add(e, 0.5f * p.x * (dr * dr));
            const float de_dr = p.x * (1.f - __fdividef(p.y, r + kEpsF));
            const float3 g = mul3(d, de_dr);
            sub_rec(&G0[ij.x], g);
            add_rec(&G1[ij.y], g);
        }
        __syncwarp();
    }
    // harmonic angles (interaction.cpp:49-74, math.cpp:96-110)
    for (int s = lane; s < t.n_angle_slots; s += kWarp) {
        const int4 ijk = __ldg(&t.angle_ijk[s]);
        if (ijk.x >= 0) {
            const float2 p = __ldg(&t.angle_p[s]);
            const float3 xi = xyz(X[ijk.x]), xj = xyz(X[ijk.y]), xk = xyz(X[ijk.z]);
            const float3 v0 = sub3(xj, xi), v1 = sub3(xj, xk);
            const float3 c = cross3(v0, v1);
            const float rp = sqrtf(dot3(c, c));
            float3 gi = cross3(v0, c), gk = cross3(c, v1);
            gi = mul3(gi, -__fdividef(1.f, dot3(v0, v0) * rp + kEpsF));
            gk = mul3(gk, -__fdividef(1.f, dot3(v1, v1) * rp + kEpsF));
            const float theta = atan2f(rp, dot3(v0, v1) + kEpsF);
            const float delta = theta - p.y;
            ds_add(e, 0.5f * p.x * (delta * delta));
            const float de = p.x * delta;
            const float3 fi = mul3(gi, de), fk = mul3(gk, de);
            add_rec(&G0[ijk.x], fi);
            sub_rec(&G1[ijk.y], add3(fi, fk));
            add_rec(&G2[ijk.z], fk);
        }
        __syncwarp();
    }
    // Fourier dihedrals, impropers then propers (interaction.cpp:76-117, math.cpp:130-167)
    for (int s = lane; s < t.n_dih_slots; s += kWarp) {
        const int4 q = __ldg(&t.dih_ijkl[s]);
        if (q.x >= 0) {
            const float3 pi = xyz(X[q.x]), pj = xyz(X[q.y]), pk = xyz(X[q.z]), pl = xyz(X[q.w]);
            const float3 rij = sub3(pj, pi), rkj = sub3(pj, pk), rkl = sub3(pl, pk);
            const float3 m = cross3(rij, rkj), n = cross3(rkj, rkl);
            const float3 w = cross3(m, n);
            const float wlen = sqrtf(dot3(w, w));
            const float phi = atan2f(wlen, dot3(m, n) + kEpsF);
            const float theta = dot3(rij, n) < 0.f ? phi : -phi;
            const float nrkj2 = dot3(rkj, rkj);
            const float nrkj_1 = __fdividef(1.f, sqrtf(nrkj2) + kEpsF);
            const float nrkj_2 = nrkj_1 * nrkj_1;
            const float nrkj = nrkj2 * nrkj_1;
            // + kEpsF: a collapsed dihedral (m or n = 0, possible in FP32 only for a pose
            // flung ~1e11 A out of the box, where coordinates resolve to ~1e4 A) gives a zero
            // gradient instead of 0 * inf = NaN; resolvable geometries are unaffected
            const float a = -__fdividef(nrkj, dot3(m, m) + kEpsF);
            const float b = __fdividef(nrkj, dot3(n, n) + kEpsF);
            const float3 gi = mul3(m, -a), gl = mul3(n, -b);
            const float pp = dot3(rij, rkj) * nrkj_2, qq = dot3(rkj, rkl) * nrkj_2;
            const float3 sv = sub3(mul3(gi, pp), mul3(gl, qq));
            const float3 gj = mul3(sub3(gi, sv), -1.f), gk = mul3(add3(gl, sv), -1.f);
            const int2 tr = __ldg(&t.dih_terms[s]);
            float de = 0.f, et = 0.f;
            for (int u = 0; u < tr.y; ++u) {
                const float4 term = __ldg(&t.dih_term[tr.x + u]);  // k, periodicity, phase
                const float delta = theta * term.y - term.z;
                float sd, cd;
                __sincosf(delta, &sd, &cd);  // |delta| <= 7 pi: fast path within FP32 parity
                et += term.x * (1.f + cd);
                de += term.x * term.y * sd;
            }
            ds_add(e, et);
            add_rec(&G0[q.x], mul3(gi, -de));
            add_rec(&G1[q.y], mul3(gj, -de));
            add_rec(&G2[q.z], mul3(gk, -de));
            add_rec(&G3[q.w], mul3(gl, -de));
        }
        __syncwarp();
    }
    // 1-4 and all other pairs: Coulomb + LJ 12-6 (interaction.cpp:127-168, pair.h:25-60).
    // The next round's record is loaded while this round computes, so its L1/L2 latency
    // is not exposed at the round's barrier (the pair rounds are the most numerous).
    int2 ij_n = lane < t.n_pair_slots ? __ldg(&t.pair_ij[lane]) : make_int2(-1, -1);
    float4 p_n = lane < t.n_pair_slots ? __ldg(&t.pair_p[lane]) : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int s = lane; s < t.n_pair_slots; s += kWarp) {
        const int2 ij = ij_n;
        const float4 pp = p_n;
        if (s + kWarp < t.n_pair_slots) {
            ij_n = __ldg(&t.pair_ij[s + kWarp]);
            p_n = __ldg(&t.pair_p[s + kWarp]);
        }
        if (ij.x >= 0) {
            float en;
            const float3 g = pair_grad(pp, X[ij.x], X[ij.y], en);
            ds_add(e, en);
            sub_rec(&G0[ij.x], g);
            add_rec(&G1[ij.y], g);
        }
        __syncwarp();
    }
}

// topo_terms for a team of nw warps (warp w of them), which split the rounds: warp w takes
// rounds w, w + nw, ... into its own arrays G. Kept apart from topo_terms so that the
// one-warp kernels compile exactly as before.
//
// Adds the bonded and non-bonded terms of `t` over coordinates `X`. The gradient of
// the atom in position k of a term goes to array k: G[k * gs + atom] (shared memory).
// Within a round the atoms of each position are distinct (host scheduling), so the
// lanes of a round update distinct records with plain loads and stores; a warp
// barrier between rounds orders a record's updates from different rounds. Padded
// slots (-1) compute nothing. Every loop runs a multiple of 32 slots, so all lanes
// meet every barrier. The caller sums the arrays. Matches
// intra_molecular_interactions::put_gradients.
//
// A team of nw warps (warp w of them) splits the rounds: warp w takes rounds w, w + nw, ...
// into its own arrays G (nw = 1: every round).
__device__ __forceinline__ void topo_terms_split(const DevTopo& t, const float4* X, float4* G, int gs, DS& e,
                                           int lane, int w, int nw) {
    float4* G0 = G;
    float4* G1 = G + gs;
    float4* G2 = G + 2 * gs;
    float4* G3 = G + 3 * gs;
    const int first = lane + w * kWarp, step = nw * kWarp;
    __syncwarp();
    // harmonic bonds (interaction.cpp:27-47)
    for (int s = first; s < t.n_bond_slots; s += step) {
        const int2 ij = __ldg(&t.bond_ij[s]);
        if (ij.x >= 0) {
            const float2 p = __ldg(&t.bond_p[s]);
            const float3 d = sub3(xyz(X[ij.y]), xyz(X[ij.x]));
            const float r = sqrtf(dot3(d, d));
            const float dr = r - p.y;
            ds_add(e, 0.5f * p.x * (dr * dr));
            const float de_dr = p.x * (1.f - __fdividef(p.y, r + kEpsF));
            const float3 g = mul3(d, de_dr);
            sub_rec(&G0[ij.x], g);
            add_rec(&G1[ij.y], g);
        }
        __syncwarp();
    }
    // harmonic angles (interaction.cpp:49-74, math.cpp:96-110)
    for (int s = first; s < t.n_angle_slots; s += step) {
        const int4 ijk = __ldg(&t.angle_ijk[s]);
        if (ijk.x >= 0) {
            const float2 p = __ldg(&t.angle_p[s]);
            const float3 xi = xyz(X[ijk.x]), xj = xyz(X[ijk.y]), xk = xyz(X[ijk.z]);
            const float3 v0 = sub3(xj, xi), v1 = sub3(xj, xk);
            const float3 c = cross3(v0, v1);
            const float rp = sqrtf(dot3(c, c));
            float3 gi = cross3(v0, c), gk = cross3(c, v1);
            gi = mul3(gi, -__fdividef(1.f, dot3(v0, v0) * rp + kEpsF));
            gk = mul3(gk, -__fdividef(1.f, dot3(v1, v1) * rp + kEpsF));
            const float theta = atan2f(rp, dot3(v0, v1) + kEpsF);
            const float delta = theta - p.y;
            ds_add(e, 0.5f * p.x * (delta * delta));
            const float de = p.x * delta;
            const float3 fi = mul3(gi, de), fk = mul3(gk, de);
            add_rec(&G0[ijk.x], fi);
            sub_rec(&G1[ijk.y], add3(fi, fk));
            add_rec(&G2[ijk.z], fk);
        }
        __syncwarp();
    }
    // Fourier dihedrals, impropers then propers (interaction.cpp:76-117, math.cpp:130-167)
    for (int s = first; s < t.n_dih_slots; s += step) {
        const int4 q = __ldg(&t.dih_ijkl[s]);
        if (q.x >= 0) {
            const float3 pi = xyz(X[q.x]), pj = xyz(X[q.y]), pk = xyz(X[q.z]), pl = xyz(X[q.w]);
            const float3 rij = sub3(pj, pi), rkj = sub3(pj, pk), rkl = sub3(pl, pk);
            const float3 m = cross3(rij, rkj), n = cross3(rkj, rkl);
            const float3 w = cross3(m, n);
            const float wlen = sqrtf(dot3(w, w));
            const float phi = atan2f(wlen, dot3(m, n) + kEpsF);
            const float theta = dot3(rij, n) < 0.f ? phi : -phi;
            const float nrkj2 = dot3(rkj, rkj);
            const float nrkj_1 = __fdividef(1.f, sqrtf(nrkj2) + kEpsF);
            const float nrkj_2 = nrkj_1 * nrkj_1;
            const float nrkj = nrkj2 * nrkj_1;
            // + kEpsF: a collapsed dihedral (m or n = 0, possible in FP32 only for a pose
            // flung ~1e11 A out of the box, where coordinates resolve to ~1e4 A) gives a zero
            // gradient instead of 0 * inf = NaN; resolvable geometries are unaffected
            const float a = -__fdividef(nrkj, dot3(m, m) + kEpsF);
            const float b = __fdividef(nrkj, dot3(n, n) + kEpsF);
            const float3 gi = mul3(m, -a), gl = mul3(n, -b);
            const float pp = dot3(rij, rkj) * nrkj_2, qq = dot3(rkj, rkl) * nrkj_2;
            const float3 sv = sub3(mul3(gi, pp), mul3(gl, qq));
            const float3 gj = mul3(sub3(gi, sv), -1.f), gk = mul3(add3(gl, sv), -1.f);
            const int2 tr = __ldg(&t.dih_terms[s]);
            float de = 0.f, et = 0.f;
            for (int u = 0; u < tr.y; ++u) {
                const float4 term = __ldg(&t.dih_term[tr.x + u]);  // k, periodicity, phase
                const float delta = theta * term.y - term.z;
                float sd, cd;
                __sincosf(delta, &sd, &cd);  // |delta| <= 7 pi: fast path within FP32 parity
                et += term.x * (1.f + cd);
                de += term.x * term.y * sd;
            }
            ds_add(e, et);
            add_rec(&G0[q.x], mul3(gi, -de));
            add_rec(&G1[q.y], mul3(gj, -de));
            add_rec(&G2[q.z], mul3(gk, -de));
            add_rec(&G3[q.w], mul3(gl, -de));
        }
        __syncwarp();
    }
    // 1-4 and all other pairs: Coulomb + LJ 12-6 (interaction.cpp:127-168, pair.h:25-60).
    // The next round's record is loaded while this round computes, so its L1/L2 latency
    // is not exposed at the round's barrier (the pair rounds are the most numerous).
    int2 ij_n = first < t.n_pair_slots ? __ldg(&t.pair_ij[first]) : make_int2(-1, -1);
    float4 p_n = first < t.n_pair_slots ? __ldg(&t.pair_p[first]) : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int s = first; s < t.n_pair_slots; s += step) {
        const int2 ij = ij_n;
        const float4 pp = p_n;
        if (s + step < t.n_pair_slots) {
            ij_n = __ldg(&t.pair_ij[s + step]);
            p_n = __ldg(&t.pair_p[s + step]);
        }
        if (ij.x >= 0) {
            float en;
            const float3 g = pair_grad(pp, X[ij.x], X[ij.y], en);
            ds_add(e, en);
            sub_rec(&G0[ij.x], g);
            add_rec(&G1[ij.y], g);
        }
        __syncwarp();
    }
}

// Trilinear blend of the stored {E, grad} records of one map (grid.cpp:273-303).
__device__ __forceinline__ float4 trilinear(const float4* __restrict__ m, const int* off,
                                            const float* w) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const float4 v = __ldg(&m[off[c]]);
        acc.x = fmaf(v.x, w[c], acc.x);
        acc.y = fmaf(v.y, w[c], acc.y);
        acc.z = fmaf(v.z, w[c], acc.z);
        acc.w = fmaf(v.w, w[c], acc.w);
    }
    return acc;
}

// receptor_cache::get (grid.cpp:197-262) in FP32. Returns energy; adds the gradient.
__device__ __forceinline__ float grid_lookup(const DevGrid& g, int slot, float q, float3 p,
                                             float3& grad) {
    float f[3] = {(p.x - g.init.x) * g.spacing_inv, (p.y - g.init.y) * g.spacing_inv,
                  (p.z - g.init.z) * g.spacing_inv};
    // distance beyond the low / high face in A, exact near the face (Sterbenz): with
    // slope 1e6 a rounded grid coordinate would misplace the penalty by ~1 kcal/mol
    const float below[3] = {(g.lo_h.x - p.x) + g.lo_l.x, (g.lo_h.y - p.y) + g.lo_l.y, (g.lo_h.z - p.z) + g.lo_l.z};
    const float above[3] = {(p.x - g.hi_h.x) - g.hi_l.x, (p.y - g.hi_h.y) - g.hi_l.y, (p.z - g.hi_h.z) - g.hi_l.z};
    const int npm1[3] = {g.npts.x - 1, g.npts.y - 1, g.npts.z - 1};
    int lo[3];
    float gs[3];
    float penalty = 0.f;  // A beyond the box, summed over axes
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (below[d] > 0.f) {
            lo[d] = 0;
            gs[d] = -1.f;
            penalty += below[d];
            f[d] = 0.f;
        } else if (above[d] < 0.f) {
            f[d] = fminf(fmaxf(f[d], 0.f), static_cast<float>(npm1[d]));
            lo[d] = min(static_cast<int>(f[d]), npm1[d] - 1);
            gs[d] = 0.f;
        } else {
            lo[d] = npm1[d] - 1;
            gs[d] = 1.f;
            penalty += above[d];
            f[d] = static_cast<float>(npm1[d]);
        }
    }
    const int sy = g.npts.z, sx = g.npts.y * g.npts.z;
    const int base = lo[0] * sx + lo[1] * sy + lo[2];
    const int off[8] = {base,          base + sx,          base + sy,      base + sx + sy,
                        base + 1,      base + sx + 1,      base + sy + 1,  base + sx + sy + 1};
    const float x = f[0] - lo[0], y = f[1] - lo[1], z = f[2] - lo[2];
    const float mx = 1.f - x, my = 1.f - y, mz = 1.f - z;
    const float w[8] = {mx * my * mz, x * my * mz, mx * y * mz, x * y * mz,
                        mx * my * z,  x * my * z,  mx * y * z,  x * y * z};
    float e = 0.f;
    bool hit = true;
    if (penalty > 0.f) {
        e += penalty * g.slope;  // (grid units x spacing) x slope, grid.cpp:211-236
        grad.x += gs[0] * g.slope;
        grad.y += gs[1] * g.slope;
        grad.z += gs[2] * g.slope;
        hit = false;
    }
    const float4 c = trilinear(g.maps, off, w);
    e += c.x * q;
    const float4 v = slot > 0 ? trilinear(g.maps + static_cast<size_t>(slot) * g.P, off, w)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
    e += v.x;
    if (hit) {
        grad.x += c.y * q + v.y;
        grad.y += c.z * q + v.z;
        grad.z += c.w * q + v.w;
    }
    return e;
}

// A team of warps of one block that evaluate one pose together (the single-walker
// search): the shared barrier state and each member's energy partial.
struct TeamShared {
    int count, gen, abort, slot;
    double gmin;
    float2 e[4];
    float2 terms[4][PXD_NUM_TERMS - 1];  // members' pose-score partials (score_pose)
};

// Spin limit of a team barrier: ~0.1 s at the loop's pace, far beyond any wait of members
// doing the same work. A member that is not seen by then sets abort: the team's later
// barriers return at once and its evaluations return NaN, so the search ends.
constexpr long long kTeamSpin = 1LL << 22;

// Barrier of the nw warps of a team (all lanes of each member call it). Orders the
// members' earlier shared-memory writes before their later reads. Returns false once the
// team has aborted.
static __device__ __noinline__ bool team_sync(TeamShared* ts, int nw, int lane) {
    __threadfence_block();
    __syncwarp();
    int ok = 1;
    if (lane == 0) {
        volatile int* vgen = &ts->gen;
        volatile int* vabort = &ts->abort;
        if (*vabort) {
            ok = 0;
        } else {
            const int g = *vgen;
            if (atomicAdd(&ts->count, 1) == nw - 1) {
                atomicExch(&ts->count, 0);
                __threadfence_block();
                atomicAdd(&ts->gen, 1);
            } else {
                for (long long it = 0; *vgen == g; ++it) {
                    if (it > kTeamSpin || *vabort) {
                        atomicExch(&ts->abort, 1);
                        ok = 0;
                        break;
                    }
                }
            }
        }
    }
    __syncwarp();
    __threadfence_block();
    return __shfl_sync(kFull, ok, 0) != 0;
}

// Per-warp shared-memory slice for one pose evaluation.
struct PoseBufs {
    float4* lig_xyz;   // [N]
    float4* lig_grad;  // [4][N]: one array per term position (topo_terms)
    float4* loc_xyz;   // [n_local]
    float4* loc_grad;  // [4][n_local]
    float4* mov_jac;   // [n_mov]
    int lig_gs, loc_gs;  // array strides
};

// A warp's place in a team evaluation: its index, the team's size, the float4 distance
// between members' slices and the team's shared state. Kept out of PoseBufs, which the
// batched optimiser reads from its stack frame on every evaluation.
struct Team {
    int w, n, f4;
    TeamShared* ts;
};

struct EvalEnv {
    DevReceptor rec;
    DevGrid grid;
};

// Energy and flat gradient [dE/dxyz (3N) | dE/dtorsion (R)] at x0 + t * d (d may be
// null: evaluate at x0). With gdir, *gdot receives gradient . gdir (the line search's
// directional derivative), accumulated while the flat gradient is written. Replaces
// binding_system_interactions::put_gradients as the optimiser's closure calls it
// (optimizer.cpp:155-167).
__device__ __forceinline__ double eval_pose_body(const EvalEnv& env, const DevLigand& L, const float* x0,
                                                const float* d, float t, float* gout, const PoseBufs& b,
                                                int lane, const float* gdir = nullptr, double* gdot = nullptr) {
    const int N = L.n_atoms;
    const int n3 = 3 * N;
    const DevReceptor& R = env.rec;
    for (int a = lane; a < N; a += kWarp) {
        float px = x0[3 * a], py = x0[3 * a + 1], pz = x0[3 * a + 2];
        if (d) {
            px = fmaf(d[3 * a], t, px);
            py = fmaf(d[3 * a + 1], t, py);
            pz = fmaf(d[3 * a + 2], t, pz);
        }
        b.lig_xyz[a] = make_float4(px, py, pz, 0.f);
#pragma unroll
        for (int k = 0; k < 4; ++k) b.lig_grad[k * b.lig_gs + a] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // receptor rotors (receptor_torsion2xyz, interaction.cpp:316-336)
    for (int l = lane; l < R.n_local; l += kWarp) {
        const float4 v = __ldg(&R.local_xyz0[l]);
        if (l < R.n_mov) {
            const int r = __float_as_int(v.w);
            float th = x0[n3 + r];
            if (d) th = fmaf(d[n3 + r], t, th);
            Mat3 Rm, Jm;
            rotation_and_jacobian(xyz(__ldg(&R.rotor_axis[r])), th, Rm, Jm);
            const float3 rel = xyz(v);
            const float3 pos = add3(mat_apply(Rm, rel), xyz(__ldg(&R.rotor_origin[r])));
            b.loc_xyz[l] = make_float4(pos.x, pos.y, pos.z, 0.f);
            const float3 jac = mat_apply(Jm, rel);
            b.mov_jac[l] = make_float4(jac.x, jac.y, jac.z, 0.f);
        } else {
            b.loc_xyz[l] = v;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) b.loc_grad[k * b.loc_gs + l] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncwarp();
    DS e{0.f, 0.f};
    topo_terms(L.topo, b.lig_xyz, b.lig_grad, b.lig_gs, e, lane);
    if (R.n_local > 0) topo_terms(R.intra, b.loc_xyz, b.loc_grad, b.loc_gs, e, lane);
    // grid lookups (inter_molecular_interactions, cached branch)
    if (env.grid.has_grid) {
        for (int a = lane; a < N; a += kWarp) {
            float3 g = make_float3(0.f, 0.f, 0.f);
            const float ea = grid_lookup(env.grid, __ldg(&L.map_slot[a]), __ldg(&L.charge[a]),
                                         xyz(b.lig_xyz[a]), g);
            ds_add(e, ea);
            add_rec(&b.lig_grad[a], g);  // one lane per atom; topo_terms ended on a barrier
        }
        __syncwarp();  // the explicit pairs below add to the same records atomically
    }
    // explicit inter pairs (rotor atoms with maps, every receptor atom without)
    const int M = R.n_explicit;
    if (M >= kWarp) {
        for (int i = 0; i < N; ++i) {
            const float3 xi = xyz(b.lig_xyz[i]);
            const float qi = __ldg(&L.charge[i]);
            const float2 sei = __ldg(&L.se[i]);
            float3 gi = make_float3(0.f, 0.f, 0.f);
            for (int j = lane; j < M; j += kWarp) {
                const int loc = __ldg(&R.ex_local[j]);
                const float4 rj = __ldg(&R.ex_xyzq[j]);
                const float3 xj = loc >= 0 ? xyz(b.loc_xyz[loc]) : xyz(rj);
                const float2 sej = __ldg(&R.ex_se[j]);
                const float3 rij = sub3(xj, xi);
                const float r2 = fmaxf(dot3(rij, rij), kPairR2Floor);
                const float rinv = rsqrtf(r2);
                const float rinv2 = rinv * rinv;
                const float s = (sei.x + sej.x) * 0.5f;
                const float xx = s * s * rinv2;
                const float u6 = xx * xx * xx, u12 = u6 * u6;
                const float C = sqrtf(sei.y * sej.y) * 4.f;
                const float ec = kCoulombF * qi * rj.w * rinv;
                ds_add(e, ec);
                ds_add(e, C * (u12 - u6));
                const float3 g = mul3(rij, (C * (6.f * u6 - 12.f * u12) - ec) * rinv2);
                gi = sub3(gi, g);
                if (loc >= 0) atomic_add3(&b.loc_grad[loc], g);
            }
            gi.x = warp_sum_f(gi.x);
            gi.y = warp_sum_f(gi.y);
            gi.z = warp_sum_f(gi.z);
            if (lane == 0) atomic_add3(&b.lig_grad[i], gi);
        }
    } else if (M > 0) {
        for (int i = lane; i < N; i += kWarp) {
            const float3 xi = xyz(b.lig_xyz[i]);
            const float qi = __ldg(&L.charge[i]);
            const float2 sei = __ldg(&L.se[i]);
            float3 gi = make_float3(0.f, 0.f, 0.f);
            for (int j = 0; j < M; ++j) {
                const int loc = __ldg(&R.ex_local[j]);
                const float4 rj = __ldg(&R.ex_xyzq[j]);
                const float3 xj = loc >= 0 ? xyz(b.loc_xyz[loc]) : xyz(rj);
                const float2 sej = __ldg(&R.ex_se[j]);
                const float3 rij = sub3(xj, xi);
                const float r2 = fmaxf(dot3(rij, rij), kPairR2Floor);
                const float rinv = rsqrtf(r2);
                const float rinv2 = rinv * rinv;
                const float s = (sei.x + sej.x) * 0.5f;
                const float xx = s * s * rinv2;
                const float u6 = xx * xx * xx, u12 = u6 * u6;
                const float C = sqrtf(sei.y * sej.y) * 4.f;
                const float ec = kCoulombF * qi * rj.w * rinv;
                ds_add(e, ec);
                ds_add(e, C * (u12 - u6));
                const float3 g = mul3(rij, (C * (6.f * u6 - 12.f * u12) - ec) * rinv2);
                gi = sub3(gi, g);
                if (loc >= 0) atomic_add3(&b.loc_grad[loc], g);
            }
            atomic_add3(&b.lig_grad[i], gi);
        }
    }
    __syncwarp();
    // flat gradient and the receptor-torsion chain rule (interaction.cpp:338-350)
    DS gd{0.f, 0.f};
    for (int a = lane; a < N; a += kWarp) {
        const float4 g0 = b.lig_grad[a], g1 = b.lig_grad[b.lig_gs + a];
        const float4 g2 = b.lig_grad[2 * b.lig_gs + a], g3 = b.lig_grad[3 * b.lig_gs + a];
        const float gx = (g0.x + g1.x) + (g2.x + g3.x);
        const float gy = (g0.y + g1.y) + (g2.y + g3.y);
        const float gz = (g0.z + g1.z) + (g2.z + g3.z);
        gout[3 * a] = gx;
        gout[3 * a + 1] = gy;
        gout[3 * a + 2] = gz;
        if (gdir) {
            ds_dot_acc(gd, gx, gdir[3 * a]);
            ds_dot_acc(gd, gy, gdir[3 * a + 1]);
            ds_dot_acc(gd, gz, gdir[3 * a + 2]);
        }
    }
    for (int r = lane; r < R.n_rotors; r += kWarp) {
        float acc = 0.f;
        const int l0 = __ldg(&R.rotor_mov[r]), l1 = __ldg(&R.rotor_mov[r + 1]);
        for (int l = l0; l < l1; ++l) {
            const float4 g0 = b.loc_grad[l], g1 = b.loc_grad[b.loc_gs + l];
            const float4 g2 = b.loc_grad[2 * b.loc_gs + l], g3 = b.loc_grad[3 * b.loc_gs + l];
            const float3 g = make_float3((g0.x + g1.x) + (g2.x + g3.x), (g0.y + g1.y) + (g2.y + g3.y),
                                         (g0.z + g1.z) + (g2.z + g3.z));
            acc += dot3(xyz(b.mov_jac[l]), g);
        }
        gout[n3 + r] = acc;
        if (gdir) ds_dot_acc(gd, acc, gdir[n3 + r]);
    }
    __syncwarp();
    if (gdir) *gdot = ds_warp_sum(gd);
    return ds_warp_sum(e) + R.e_const;
}

// eval_pose_body for a team of warps (Team): the members split the terms, lookups and
// explicit pairs and sum each other's parts in member order. Kept apart from
// eval_pose_body so that the one-warp kernels compile exactly as before.
__device__ __forceinline__ double eval_pose_team_body(const EvalEnv& env, const DevLigand& L, const float* x0,
                                                     const float* d, float t, float* gout, const PoseBufs& b,
                                                     int lane, const float* gdir, double* gdot, const Team* team) {
    const int N = L.n_atoms;
    const int n3 = 3 * N;
    const DevReceptor& R = env.rec;
    for (int a = lane; a < N; a += kWarp) {
        float px = x0[3 * a], py = x0[3 * a + 1], pz = x0[3 * a + 2];
        if (d) {
            px = fmaf(d[3 * a], t, px);
            py = fmaf(d[3 * a + 1], t, py);
            pz = fmaf(d[3 * a + 2], t, pz);
        }
        b.lig_xyz[a] = make_float4(px, py, pz, 0.f);
#pragma unroll
        for (int k = 0; k < 4; ++k) b.lig_grad[k * b.lig_gs + a] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // receptor rotors (receptor_torsion2xyz, interaction.cpp:316-336)
    for (int l = lane; l < R.n_local; l += kWarp) {
        const float4 v = __ldg(&R.local_xyz0[l]);
        if (l < R.n_mov) {
            const int r = __float_as_int(v.w);
            float th = x0[n3 + r];
            if (d) th = fmaf(d[n3 + r], t, th);
            Mat3 Rm, Jm;
            rotation_and_jacobian(xyz(__ldg(&R.rotor_axis[r])), th, Rm, Jm);
            const float3 rel = xyz(v);
            const float3 pos = add3(mat_apply(Rm, rel), xyz(__ldg(&R.rotor_origin[r])));
            b.loc_xyz[l] = make_float4(pos.x, pos.y, pos.z, 0.f);
            const float3 jac = mat_apply(Jm, rel);
            b.mov_jac[l] = make_float4(jac.x, jac.y, jac.z, 0.f);
        } else {
            b.loc_xyz[l] = v;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) b.loc_grad[k * b.loc_gs + l] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncwarp();
    // a team splits the terms, lookups and explicit pairs among its warps (tw of tn)
    const int tw = team->w, tn = team->n;
    const int tf4 = team->f4;
    TeamShared* ts = team->ts;
    DS e{0.f, 0.f};
    topo_terms_split(L.topo, b.lig_xyz, b.lig_grad, b.lig_gs, e, lane, tw, tn);
    if (R.n_local > 0) topo_terms_split(R.intra, b.loc_xyz, b.loc_grad, b.loc_gs, e, lane, tw, tn);
    // grid lookups (inter_molecular_interactions, cached branch)
    if (env.grid.has_grid) {
        for (int a = lane + tw * kWarp; a < N; a += tn * kWarp) {
            float3 g = make_float3(0.f, 0.f, 0.f);
            const float ea = grid_lookup(env.grid, __ldg(&L.map_slot[a]), __ldg(&L.charge[a]),
                                         xyz(b.lig_xyz[a]), g);
            ds_add(e, ea);
            add_rec(&b.lig_grad[a], g);  // one lane per atom; topo_terms ended on a barrier
        }
        __syncwarp();  // the explicit pairs below add to the same records atomically
    }
    // explicit inter pairs (rotor atoms with maps, every receptor atom without)
    const int M = R.n_explicit;
    if (M >= kWarp) {
        for (int i = tw; i < N; i += tn) {
            const float3 xi = xyz(b.lig_xyz[i]);
            const float qi = __ldg(&L.charge[i]);
            const float2 sei = __ldg(&L.se[i]);
            float3 gi = make_float3(0.f, 0.f, 0.f);
            for (int j = lane; j < M; j += kWarp) {
                const int loc = __ldg(&R.ex_local[j]);
                const float4 rj = __ldg(&R.ex_xyzq[j]);
                const float3 xj = loc >= 0 ? xyz(b.loc_xyz[loc]) : xyz(rj);
                const float2 sej = __ldg(&R.ex_se[j]);
                const float3 rij = sub3(xj, xi);
                const float r2 = fmaxf(dot3(rij, rij), kPairR2Floor);
                const float rinv = rsqrtf(r2);
                const float rinv2 = rinv * rinv;
                const float s = (sei.x + sej.x) * 0.5f;
                const float xx = s * s * rinv2;
                const float u6 = xx * xx * xx, u12 = u6 * u6;
                const float C = sqrtf(sei.y * sej.y) * 4.f;
                const float ec = kCoulombF * qi * rj.w * rinv;
                ds_add(e, ec);
                ds_add(e, C * (u12 - u6));
                const float3 g = mul3(rij, (C * (6.f * u6 - 12.f * u12) - ec) * rinv2);
                gi = sub3(gi, g);
                if (loc >= 0) atomic_add3(&b.loc_grad[loc], g);
            }
            gi.x = warp_sum_f(gi.x);
            gi.y = warp_sum_f(gi.y);
            gi.z = warp_sum_f(gi.z);
            if (lane == 0) atomic_add3(&b.lig_grad[i], gi);
        }
    } else if (M > 0) {
        for (int i = lane + tw * kWarp; i < N; i += tn * kWarp) {
            const float3 xi = xyz(b.lig_xyz[i]);
            const float qi = __ldg(&L.charge[i]);
            const float2 sei = __ldg(&L.se[i]);
            float3 gi = make_float3(0.f, 0.f, 0.f);
            for (int j = 0; j < M; ++j) {
                const int loc = __ldg(&R.ex_local[j]);
                const float4 rj = __ldg(&R.ex_xyzq[j]);
                const float3 xj = loc >= 0 ? xyz(b.loc_xyz[loc]) : xyz(rj);
                const float2 sej = __ldg(&R.ex_se[j]);
                const float3 rij = sub3(xj, xi);
                const float r2 = fmaxf(dot3(rij, rij), kPairR2Floor);
                const float rinv = rsqrtf(r2);
                const float rinv2 = rinv * rinv;
                const float s = (sei.x + sej.x) * 0.5f;
                const float xx = s * s * rinv2;
                const float u6 = xx * xx * xx, u12 = u6 * u6;
                const float C = sqrtf(sei.y * sej.y) * 4.f;
                const float ec = kCoulombF * qi * rj.w * rinv;
                ds_add(e, ec);
                ds_add(e, C * (u12 - u6));
                const float3 g = mul3(rij, (C * (6.f * u6 - 12.f * u12) - ec) * rinv2);
                gi = sub3(gi, g);
                if (loc >= 0) atomic_add3(&b.loc_grad[loc], g);
            }
            atomic_add3(&b.lig_grad[i], gi);
        }
    }
    __syncwarp();
    DS et = e;  // the pose's energy (the team's partials summed in member order)
    if (tn > 1) {
        const DS ew = ds_warp_reduce(e);
        if (lane == 0) ts->e[tw] = make_float2(ew.hi, ew.lo);
        if (!team_sync(ts, tn, lane)) {  // the team aborted: NaN ends the caller's search
            if (gdot) *gdot = __longlong_as_double(0x7ff8000000000000LL);
            return __longlong_as_double(0x7ff8000000000000LL);
        }
        et = DS{ts->e[0].x, ts->e[0].y};
        for (int u = 1; u < tn; ++u) ds_add_ds(et, DS{ts->e[u].x, ts->e[u].y});
    }
    // flat gradient and the receptor-torsion chain rule (interaction.cpp:338-350), the
    // team's arrays summed in member order
    DS gd{0.f, 0.f};
    for (int a = lane; a < N; a += kWarp) {
        float gx = 0.f, gy = 0.f, gz = 0.f;
        for (int u = 0; u < tn; ++u) {
            const float4* G = b.lig_grad + (u - tw) * tf4;
            const float4 g0 = G[a], g1 = G[b.lig_gs + a];
            const float4 g2 = G[2 * b.lig_gs + a], g3 = G[3 * b.lig_gs + a];
            const float sx = (g0.x + g1.x) + (g2.x + g3.x);
            const float sy = (g0.y + g1.y) + (g2.y + g3.y);
            const float sz = (g0.z + g1.z) + (g2.z + g3.z);
            gx = u == 0 ? sx : gx + sx;
            gy = u == 0 ? sy : gy + sy;
            gz = u == 0 ? sz : gz + sz;
        }
        gout[3 * a] = gx;
        gout[3 * a + 1] = gy;
        gout[3 * a + 2] = gz;
        if (gdir) {
            ds_dot_acc(gd, gx, gdir[3 * a]);
            ds_dot_acc(gd, gy, gdir[3 * a + 1]);
            ds_dot_acc(gd, gz, gdir[3 * a + 2]);
        }
    }
    for (int r = lane; r < R.n_rotors; r += kWarp) {
        float acc = 0.f;
        const int l0 = __ldg(&R.rotor_mov[r]), l1 = __ldg(&R.rotor_mov[r + 1]);
        for (int l = l0; l < l1; ++l) {
            float3 g = make_float3(0.f, 0.f, 0.f);
            for (int u = 0; u < tn; ++u) {
                const float4* G = b.loc_grad + (u - tw) * tf4;
                const float4 g0 = G[l], g1 = G[b.loc_gs + l];
                const float4 g2 = G[2 * b.loc_gs + l], g3 = G[3 * b.loc_gs + l];
                const float3 gu = make_float3((g0.x + g1.x) + (g2.x + g3.x), (g0.y + g1.y) + (g2.y + g3.y),
                                              (g0.z + g1.z) + (g2.z + g3.z));
                g = u == 0 ? gu : add3(g, gu);
            }
            acc += dot3(xyz(b.mov_jac[l]), g);
        }
        gout[n3 + r] = acc;
        if (gdir) ds_dot_acc(gd, acc, gdir[n3 + r]);
    }
    __syncwarp();
    // no member clears its arrays for the next evaluation before every member has read them
    if (tn > 1 && !team_sync(ts, tn, lane)) {
        if (gdot) *gdot = __longlong_as_double(0x7ff8000000000000LL);
        return __longlong_as_double(0x7ff8000000000000LL);
    }
    if (gdir) *gdot = ds_warp_sum(gd);
    if (tn > 1) return static_cast<double>(et.hi) + static_cast<double>(et.lo) + R.e_const;
    return ds_warp_sum(e) + R.e_const;
}

// Kept out of line: the optimiser calls it from five places, and inlined copies of this
// much code overflow the instruction cache (the top stall of the batched kernel).
// kTeam: the evaluation is shared by a team of warps (PoseBufs' team fields).
template <bool kTeam = false>
static __device__ __noinline__ double eval_pose(const EvalEnv& env, const DevLigand& L, const float* x0,
                                                const float* d, float t, float* gout, const PoseBufs& b,
                                                int lane, double* gdot = nullptr, const Team* team = nullptr) {
    if constexpr (kTeam)
        return eval_pose_team_body(env, L, x0, d, t, gout, b, lane, gdot ? d : nullptr, gdot, team);
    else
        return eval_pose_body(env, L, x0, d, t, gout, b, lane, gdot ? d : nullptr, gdot);
}

// Shared-memory floats needed by PoseBufs for a ligand of up to n_atoms atoms.
__host__ __device__ inline int pose_bufs_floats(int n_atoms, int n_local) {
    return 20 * n_atoms + 24 * n_local;
}

__device__ inline PoseBufs carve_pose_bufs(float* base, int n_atoms, int n_local) {
    PoseBufs b;
    b.lig_xyz = reinterpret_cast<float4*>(base);
    b.lig_grad = b.lig_xyz + n_atoms;
    b.loc_xyz = b.lig_grad + 4 * n_atoms;
    b.loc_grad = b.loc_xyz + n_local;
    b.mov_jac = b.loc_grad + 4 * n_local;
    b.lig_gs = n_atoms;
    b.loc_gs = n_local;
    return b;
}

}  // namespace pxd
