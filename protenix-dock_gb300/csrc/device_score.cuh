// Warp-cooperative empirical score of one pose (pose selection / affinity): the device
// restatement of root_scorer::combine with its leaf scorers (scorer.cpp:53-724).
//
// Ligand coordinates come from the warp's shared-memory slice, receptor coordinates from
// the all-atom table with rotor atoms substituted from the slice. Receptor ring centroids
// and normals are precomputed on the host (ring atoms never sit on a rotor). Every term
// is summed per lane in a compensated FP32 pair and reduced over the warp.
#pragma once

#include "device_eval.cuh"

namespace pxd {

// get_reversed_linear_percent (math.h:196-215)
__device__ __forceinline__ float ramp_down(float v, float lo, float hi) {
    if (v < lo) return 1.f;
    if (v <= hi) return 1.f - (v - lo) / (hi - lo);
    return 0.f;
}
__device__ __forceinline__ float ramp_down_c(float v, float c, float lo, float hi) {
    return v < c ? ramp_down(c - v, lo, hi) : ramp_down(v - c, lo, hi);
}
__device__ __forceinline__ float dist3(float3 a, float3 b) {
    const float3 d = sub3(a, b);
    return sqrtf(dot3(d, d));
}

struct ScoreEnv {
    DevRecScore rs;
    const DevSf* sf;
};

__device__ __forceinline__ float3 rec_pos(const DevRecScore& rs, const float4* loc_xyz, int j) {
    const int l = __ldg(&rs.all_local[j]);
    return l >= 0 ? xyz(loc_xyz[l]) : xyz(__ldg(&rs.all_xyzq[j]));
}

__device__ __forceinline__ void lig_ring(const float4* X, const int* r, float3& c, float3& n) {
    int sz = 0;
    c = make_float3(0.f, 0.f, 0.f);
    for (int k = 0; k < 6; ++k) {
        const int a = __ldg(&r[k]);
        if (a < 0) break;
        c = add3(c, xyz(X[a]));
        ++sz;
    }
    c = mul3(c, 1.f / sz);
    const float3 p0 = xyz(X[__ldg(&r[0])]), p1 = xyz(X[__ldg(&r[1])]), p2 = xyz(X[__ldg(&r[2])]);
    n = cross3(sub3(p1, p0), sub3(p1, p2));
    n = mul3(n, 1.f / sqrtf(dot3(n, n)));
}

__device__ __forceinline__ float projected(float3 n1, float3 c1, float3 c2) {
    const float3 t = sub3(c2, c1);
    const float dp = dot3(n1, t);
    return sqrtf(dot3(t, t) - dp * dp);
}

// pi_stacking_batch::calculate (scorer.cpp:698-724) for one ring pair
__device__ __forceinline__ float stack_pair(float3 rc, float3 rn, float3 lc, float3 ln,
                                            const float* p, float center) {
    float d = dist3(rc, lc);
    if (d > p[1]) return 0.f;
    d = ramp_down(d, p[0], p[1]);
    const float s1 = projected(rn, rc, lc), s2 = projected(ln, lc, rc);
    float sg = s1 < s2 ? s1 : s2;
    if (sg > p[5]) return 0.f;
    sg = ramp_down(sg, p[4], p[5]);
    float th = acosf(fminf(fmaxf(dot3(rn, ln), -1.f), 1.f)) * (180.f / 3.14159265358979f);
    th = fminf(th, 180.f - th);
    th = ramp_down_c(th, center, p[2], p[3]);
    return -d * sg * th;
}

// hbond_interactions_ga_tuning_param::calculate, one (donor, acceptor) pair
__device__ __forceinline__ float hbond_pair(float3 dpos, float3 hpos, float3 apos, const float* p) {
    const float dd = ramp_down_c(dist3(hpos, apos), p[4], p[0], p[1]);
    if (dd < kEpsF) return 0.f;
    const float3 h2d = sub3(dpos, hpos), h2a = sub3(apos, hpos);
    const float ll = sqrtf(dot3(h2d, h2d)) * sqrtf(dot3(h2a, h2a));
    const float c = fminf(fmaxf(dot3(h2d, h2a) / (ll + kEpsF), -1.f), 1.f);
    const float ang = acosf(c) * (180.f / 3.14159265358979f);
    return -dd * ramp_down_c(ang, p[5], p[2], p[3]);
}

__device__ __forceinline__ float signed_dihedral(float3 pi, float3 pj, float3 pk, float3 pl) {
    const float3 rij = sub3(pj, pi), rkj = sub3(pj, pk), w0 = sub3(pl, pk);
    const float3 m = cross3(rij, rkj), n = cross3(rkj, w0);
    const float3 w = cross3(m, n);
    const float phi = atan2f(sqrtf(dot3(w, w)), dot3(m, n) + kEpsF);
    return dot3(rij, n) < 0.f ? phi : -phi;
}

// Score of the pose in X (ligand, smem) with receptor rotor atoms in loc_xyz (smem).
// Returns sum(coef * term) over the active terms except GB/SA; when `terms` is given,
// lane 0 stores the unweighted values.
//
// kTeam (a team of warps of one block, PoseBufs' team fields in tw / tn / ts): the members
// split the all-pairs Coulomb / LJ loop, members 1, 2 and 3 add the hydrophobic, the
// ionic / cation-pi / stacking and the hydrogen-bond / torsion-strain terms, and the
// partials are summed in member order, so every member returns the same score.
template <bool kTeam = false>
static __device__ double score_pose(const ScoreEnv& env, const DevLigand& L, const DevLigScore& ls,
                             const float4* X, const float4* loc_xyz, int lane, double* terms,
                             int tw = 0, int tn = 1, TeamShared* ts = nullptr) {
    const DevRecScore& rs = env.rs;
    const DevSf& sf = *env.sf;
    const int N = L.n_atoms;
    if (!kTeam) {
        tw = 0;
        tn = 1;
    }
    // the members that add the terms other than Coulomb / LJ (all of them on a lone warp)
    const bool own_hyd = tw == 1 % tn, own_ion = tw == 2 % tn, own_hb = tw == 3 % tn;
    DS acc[PXD_NUM_TERMS - 1];
#pragma unroll
    for (int k = 0; k < PXD_NUM_TERMS - 1; ++k) acc[k] = DS{0.f, 0.f};
    const bool coul = sf.coef[PXD_TERM_COULOMB] != 0.f, vdw = sf.coef[PXD_TERM_VDW] != 0.f;
    // Coulomb and clamped LJ over every ligand x receptor pair (scorer.cpp:222-276). Each
    // lane takes receptor atoms and walks the ligand atoms (shared memory and L1-resident
    // records, read by every lane at once): a receptor atom's records are loaded once per
    // call instead of once per ligand atom, which leaves a lone warp (the single-walker
    // search) arithmetic instead of load latency. The pairs are the same; their sum runs
    // in another order.
    if (coul || vdw) {
        for (int j = lane + tw * kWarp; j < rs.n_all; j += tn * kWarp) {
            const float4 rj = __ldg(&rs.all_xyzq[j]);
            const int l = __ldg(&rs.all_local[j]);
            const float3 xj = l >= 0 ? xyz(loc_xyz[l]) : xyz(rj);
            const float2 sej = __ldg(&rs.all_se[j]);
            float ec = 0.f, ev = 0.f;
#pragma unroll 4
            for (int i = 0; i < N; ++i) {
                const float3 xi = xyz(X[i]);
                const float qi = __ldg(&L.charge[i]);
                const float2 ti = sf.vdw_type[__ldg(&L.type[i])];
                const float d = dist3(xi, xj);
                const float rinv = 1.f / (d + kEpsF);
                ec = fmaf(qi * rj.w, rinv, ec);
                const float s = (ti.x + sej.x) * 0.5f * rinv;
                const float s2 = s * s;
                const float u6 = s2 * s2 * s2;
                const float v = (u6 * u6 - u6) * (sqrtf(ti.y * sej.y) * 4.f);
                ev += fminf(fmaxf(v, -sf.vdw_cutoff), sf.vdw_cutoff);
            }
            ds_add(acc[PXD_TERM_COULOMB], ec * kCoulombF);
            ds_add(acc[PXD_TERM_VDW], ev);
        }
    }
    // hydrophobic contacts (scorer.cpp:278-311)
    if (own_hyd && sf.coef[PXD_TERM_HYDROPHOBIC] != 0.f) {
        for (int a = 0; a < ls.n_hyd; ++a) {
            const int i = __ldg(&ls.hyd[a]);
            const float3 xi = xyz(X[i]);
            const float s1 = sf.vdw_sigma_raw[__ldg(&L.type[i])];
            float e = 0.f;
            for (int b = lane; b < rs.n_hyd; b += kWarp) {
                const int j = __ldg(&rs.hyd[b]);
                const float r1 = (s1 + __ldg(&rs.all_se[j]).x) * sf.hydro_factor + sf.hydro_min;
                e -= ramp_down(dist3(xi, rec_pos(rs, loc_xyz, j)), r1, r1 + sf.hydro_max);
            }
            ds_add(acc[PXD_TERM_HYDROPHOBIC], e);
        }
    }
    // ionic (scorer.cpp:313-368): ligand cations x receptor anions, receptor cations x ligand anions
    if (own_ion && sf.coef[PXD_TERM_IONIC] != 0.f) {
        float e = 0.f;
        for (int a = 0; a < ls.n_cat; ++a) {
            const float3 xi = xyz(X[__ldg(&ls.cat[a])]);
            for (int b = lane; b < rs.n_an; b += kWarp)
                e -= sf.ionic_coef[0] *
                     ramp_down(dist3(xi, rec_pos(rs, loc_xyz, __ldg(&rs.an[b]))), sf.ionic[0][0], sf.ionic[0][1]);
        }
        for (int a = 0; a < ls.n_an; ++a) {
            const float3 xi = xyz(X[__ldg(&ls.an[a])]);
            for (int b = lane; b < rs.n_cat; b += kWarp)
                e -= sf.ionic_coef[1] *
                     ramp_down(dist3(rec_pos(rs, loc_xyz, __ldg(&rs.cat[b])), xi), sf.ionic[1][0], sf.ionic[1][1]);
        }
        ds_add(acc[PXD_TERM_IONIC], e);
    }
    // cation-pi (scorer.cpp:370-462)
    if (own_ion && sf.coef[PXD_TERM_PI_CATION] != 0.f) {
        float e = 0.f;
        for (int a = 0; a < ls.n_cat; ++a) {
            const float3 xi = xyz(X[__ldg(&ls.cat[a])]);
            for (int b = lane; b < rs.n_r5; b += kWarp)
                e -= sf.picat_coef[0] * ramp_down(dist3(xyz(__ldg(&rs.r5c[b])), xi), sf.picat[0][0], sf.picat[0][1]);
            for (int b = lane; b < rs.n_r6; b += kWarp)
                e -= sf.picat_coef[1] * ramp_down(dist3(xyz(__ldg(&rs.r6c[b])), xi), sf.picat[1][0], sf.picat[1][1]);
        }
        for (int r = 0; r < ls.n_r5 + ls.n_r6; ++r) {
            const bool five = r < ls.n_r5;
            float3 c, n;
            lig_ring(X, five ? ls.r5 + 6 * r : ls.r6 + 6 * (r - ls.n_r5), c, n);
            const int k = five ? 2 : 3;
            for (int b = lane; b < rs.n_cat; b += kWarp)
                e -= sf.picat_coef[k] *
                     ramp_down(dist3(c, rec_pos(rs, loc_xyz, __ldg(&rs.cat[b]))), sf.picat[k][0], sf.picat[k][1]);
        }
        ds_add(acc[PXD_TERM_PI_CATION], e);
    }
    // pi stacking, face-to-face (centre 0) and edge-to-face (centre 90) (scorer.cpp:638-724)
    for (int w = 0; w < 2; ++w) {
        if (!own_ion || sf.coef[PXD_TERM_F2F + w] == 0.f) continue;
        const float center = w == 0 ? 0.f : 90.f;
        float e = 0.f;
        for (int r = 0; r < ls.n_r5 + ls.n_r6; ++r) {
            const bool five = r < ls.n_r5;
            float3 lc, ln;
            lig_ring(X, five ? ls.r5 + 6 * r : ls.r6 + 6 * (r - ls.n_r5), lc, ln);
            // l5r5, l5r6, l6r5, l6r6 in the reference's argument order
            const int k5 = five ? 0 : 2, k6 = five ? 1 : 3;
            for (int b = lane; b < rs.n_r5; b += kWarp)
                e += sf.stack_coef[w][k5] * stack_pair(xyz(__ldg(&rs.r5c[b])), xyz(__ldg(&rs.r5n[b])), lc, ln,
                                                       sf.stack[w][k5], center);
            for (int b = lane; b < rs.n_r6; b += kWarp)
                e += sf.stack_coef[w][k6] * stack_pair(xyz(__ldg(&rs.r6c[b])), xyz(__ldg(&rs.r6n[b])), lc, ln,
                                                       sf.stack[w][k6], center);
        }
        ds_add(acc[PXD_TERM_F2F + w], e);
    }
    // hydrogen bonds, 8 donor/acceptor classes (scorer.cpp:464-577)
    if (own_hb && sf.coef[PXD_TERM_HBOND] != 0.f) {
        float e = 0.f;
        for (int c = 0; c < 2; ++c) {  // ligand donors (charged, neutral)
            const int nd = c == 0 ? ls.n_donc : ls.n_donn;
            const int2* dl = c == 0 ? ls.donc : ls.donn;
            for (int a = 0; a < nd; ++a) {
                const int2 dh = __ldg(&dl[a]);
                const float3 dp = xyz(X[dh.x]), hp = xyz(X[dh.y]);
                for (int u = 0; u < 2; ++u) {  // receptor acceptors (charged, neutral)
                    const int na = u == 0 ? rs.n_accc : rs.n_accn;
                    const int* al = u == 0 ? rs.accc : rs.accn;
                    const int k = 2 * c + u;
                    float s = 0.f;
                    for (int b = lane; b < na; b += kWarp)
                        s += hbond_pair(dp, hp, rec_pos(rs, loc_xyz, __ldg(&al[b])), sf.hbond[k]);
                    e += sf.hbond_coef[k] * s;
                }
            }
        }
        for (int u = 0; u < 2; ++u) {  // ligand acceptors (charged, neutral)
            const int na = u == 0 ? ls.n_accc : ls.n_accn;
            const int* al = u == 0 ? ls.accc : ls.accn;
            for (int a = 0; a < na; ++a) {
                const float3 ap = xyz(X[__ldg(&al[a])]);
                for (int c = 0; c < 2; ++c) {  // receptor donors (charged, neutral)
                    const int nd = c == 0 ? rs.n_donc : rs.n_donn;
                    const int2* dl = c == 0 ? rs.donc : rs.donn;
                    const int k = 4 + 2 * c + u;
                    float s = 0.f;
                    for (int b = lane; b < nd; b += kWarp) {
                        const int2 dh = __ldg(&dl[b]);
                        s += hbond_pair(rec_pos(rs, loc_xyz, dh.x), rec_pos(rs, loc_xyz, dh.y), ap, sf.hbond[k]);
                    }
                    e += sf.hbond_coef[k] * s;
                }
            }
        }
        ds_add(acc[PXD_TERM_HBOND], e * sf.hbond_scale);
    }
    // torsion strain (scorer.cpp:579-613)
    if (own_hb && sf.coef[PXD_TERM_TSTRAIN] != 0.f) {
        for (int t = lane; t < ls.n_ts; t += kWarp) {
            const float4 co = __ldg(&ls.ts_coef[t]);
            const int2 rg = __ldg(&ls.ts_range[t]);
            float tmp = 0.f;
            int j = 0;
            for (; j < rg.y; ++j) {
                const int4 q = __ldg(&ls.ts_quad[rg.x + j]);
                if (q.x == q.y) break;
                const float th = signed_dihedral(xyz(X[q.x]), xyz(X[q.y]), xyz(X[q.z]), xyz(X[q.w]));
                tmp += (1.f + cosf(th)) * co.x + (1.f + cosf(2.f * th - 3.14159265358979f)) * co.y +
                       (1.f + cosf(3.f * th)) * co.z + (1.f + cosf(4.f * th - 3.14159265358979f)) * co.w;
            }
            if (j > 0) ds_add(acc[PXD_TERM_TSTRAIN], tmp / j);
        }
    }
    double total = 0.0;
    double vals[PXD_NUM_TERMS];
    if (kTeam && tn > 1) {
#pragma unroll
        for (int k = 0; k < PXD_NUM_TERMS - 1; ++k) {
            const DS r = ds_warp_reduce(acc[k]);
            if (lane == 0) ts->terms[tw][k] = make_float2(r.hi, r.lo);
        }
        const bool ok = team_sync(ts, tn, lane);
#pragma unroll
        for (int k = 0; k < PXD_NUM_TERMS - 1; ++k) {
            DS t{ts->terms[0][k].x, ts->terms[0][k].y};
            for (int u = 1; u < tn; ++u) ds_add_ds(t, DS{ts->terms[u][k].x, ts->terms[u][k].y});
            vals[k] = static_cast<double>(t.hi) + static_cast<double>(t.lo);
        }
        // read by every member before any member writes its next partials; an aborted
        // team scores NaN
        if (!team_sync(ts, tn, lane) || !ok) return __longlong_as_double(0x7ff8000000000000LL);
    } else {
#pragma unroll
        for (int k = 0; k < PXD_NUM_TERMS - 1; ++k) vals[k] = ds_warp_sum(acc[k]);
    }
    vals[PXD_TERM_VDW] *= sf.vdw_scale;
    vals[PXD_TERM_HYDROPHOBIC] *= sf.hydro_scale;
    vals[PXD_TERM_ROTATABLE] = sf.coef[PXD_TERM_ROTATABLE] != 0.f ? -1.0 / (2.620643 + ls.n_rot) : 0.0;
    vals[PXD_TERM_GBSA] = 0.0;
#pragma unroll
    for (int k = 0; k < PXD_NUM_TERMS; ++k) total += static_cast<double>(sf.coef[k]) * vals[k];
    if (terms && lane == 0) {
        for (int k = 0; k < PXD_NUM_TERMS; ++k) terms[k] = vals[k];
    }
    return total;
}

}  // namespace pxd
