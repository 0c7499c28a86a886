// Energy of one pose in FP64, no gradient: the value of
// binding_system_interactions::put_gradients (interaction.cpp:259-350) at the pose that an
// optimiser or a search returns, to within 1e-3 kcal/mol of the FP64 reference at any
// energy. The optimiser steers on the FP32 evaluation (device_eval.cuh); this evaluation
// gives the reported number. One warp per pose, every lane returns the same value.
//
// Precision per term, against the FP64 objective:
//   - grid lookups (grid.cpp:197-303): FP64 box geometry, penalty and trilinear weights over
//     map energies E = FP32 record + FP32 residual of the FP64 sum (grid build);
//   - bonds (interaction.cpp:27-47): FP64 (unbounded in a stretched bond);
//   - pairs, intra and explicit inter (pair.h:25-60): FP32, recomputed in FP64 from FP64
//     parameters when the FP32 term exceeds 1 kcal/mol (FP32 carries ~1e-6 of a term, so
//     a 1e6 clash would be off by 1 kcal/mol; terms under 1 kcal/mol stay below 1e-6);
//   - angles and dihedrals (interaction.cpp:49-117): FP32 geometry, FP64 sums. These are
//     bounded (0.5 k pi^2, 2 sum k): an FP32 angle error of ~1e-7 rad moves a term by at
//     most k |theta - theta0| 1e-7, ~1e-5 kcal/mol;
//   - receptor rotor atoms (interaction.cpp:316-336): FP64 rotations of FP64 coordinates.
// Every per-lane sum is FP64 and the warp sum is a fixed butterfly, so the value repeats
// bit for bit.
#pragma once

#include "device_eval.cuh"

namespace pxd {

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 d3_sub(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ double d3_dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 d3_of(float3 v) {
    return D3{static_cast<double>(v.x), static_cast<double>(v.y), static_cast<double>(v.z)};
}

// Sum over the warp in FP64 (xor butterfly: every lane adds the same two values in the
// same order, so all lanes hold the same sum).
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    return v;
}

constexpr double kCoulombD64 = 332.0637141491396;  // kCoulombFactor, system.h:83
constexpr float kPairFp64 = 1.f;                   // kcal/mol: larger pair terms go FP64

// Pair energy A/r + C((S2/r^2)^6 - (S2/r^2)^3) from FP64 parameters and coordinates.
__device__ __forceinline__ double pair_energy64(double4 p, D3 xi, D3 xj) {
    const D3 r = d3_sub(xj, xi);
    const double r2 = d3_dot(r, r);
    const double x = p.z / r2;
    const double u6 = x * x * x;
    return p.x / sqrt(r2) + p.y * (u6 * u6 - u6);
}

// Energy of the terms of `t` (intra_molecular_interactions) with positions given in FP32
// (P32) and FP64 (P64) by index.
template <class P32, class P64>
__device__ double topo_energy64(const DevTopo& t, const P32& pos32, const P64& pos64, int lane) {
    double e = 0.0;
    for (int s = lane; s < t.n_bond_slots; s += kWarp) {
        const int2 ij = __ldg(&t.bond_ij[s]);
        if (ij.x < 0) continue;
        const double2 p = __ldg(&t.bond_p64[s]);
        const D3 d = d3_sub(pos64(ij.y), pos64(ij.x));
        const double dr = sqrt(d3_dot(d, d)) - p.y;
        e += 0.5 * p.x * (dr * dr);
    }
    for (int s = lane; s < t.n_angle_slots; s += kWarp) {
        const int4 ijk = __ldg(&t.angle_ijk[s]);
        if (ijk.x < 0) continue;
        const float2 p = __ldg(&t.angle_p[s]);
        const float3 xi = pos32(ijk.x), xj = pos32(ijk.y), xk = pos32(ijk.z);
        const float3 v0 = sub3(xj, xi), v1 = sub3(xj, xk);
        const float3 c = cross3(v0, v1);
        const float theta = atan2f(sqrtf(dot3(c, c)), dot3(v0, v1) + kEpsF);
        const double delta = static_cast<double>(theta) - __ldg(&t.angle_p64[s]).y;
        e += 0.5 * static_cast<double>(p.x) * (delta * delta);
    }
    for (int s = lane; s < t.n_dih_slots; s += kWarp) {
        const int4 q = __ldg(&t.dih_ijkl[s]);
        if (q.x < 0) continue;
        const float3 pi = pos32(q.x), pj = pos32(q.y), pk = pos32(q.z), pl = pos32(q.w);
        const float3 rij = sub3(pj, pi), rkj = sub3(pj, pk), rkl = sub3(pl, pk);
        const float3 m = cross3(rij, rkj), n = cross3(rkj, rkl);
        const float3 w = cross3(m, n);
        const float phi = atan2f(sqrtf(dot3(w, w)), dot3(m, n) + kEpsF);
        const float theta = dot3(rij, n) < 0.f ? phi : -phi;
        const int2 tr = __ldg(&t.dih_terms[s]);
        for (int u = 0; u < tr.y; ++u) {
            const double4 term = t.dih_term64[tr.x + u];  // k, periodicity, phase
            const float delta = theta * static_cast<float>(term.y) - static_cast<float>(term.z);
            e += term.x * (1.0 + static_cast<double>(cosf(delta)));
        }
    }
    for (int s = lane; s < t.n_pair_slots; s += kWarp) {
        const int2 ij = __ldg(&t.pair_ij[s]);
        if (ij.x < 0) continue;
        const float3 xi = pos32(ij.x), xj = pos32(ij.y);
        const float4 p = __ldg(&t.pair_p[s]);
        const float3 rij = sub3(xj, xi);
        const float r2 = dot3(rij, rij);
        const float rinv = rsqrtf(r2);
        const float x = p.z * rinv * rinv;
        const float u6 = x * x * x;
        const float en = fmaf(p.y, u6 * u6 - u6, p.x * rinv);
        if (fabsf(en) <= kPairFp64)
            e += static_cast<double>(en);
        else  // also inf / NaN
            e += pair_energy64(t.pair_p64[s], pos64(ij.x), pos64(ij.y));
    }
    return e;
}

// receptor_cache::get (grid.cpp:197-262) energy in FP64 for an atom of charge q at p.
__device__ __forceinline__ double grid_energy64(const DevGrid& g, int slot, double q, D3 p) {
    const double sinv = 1.0 / g.spacing64;
    double f[3] = {(p.x - g.init64.x) * sinv, (p.y - g.init64.y) * sinv, (p.z - g.init64.z) * sinv};
    const int npm1[3] = {g.npts.x - 1, g.npts.y - 1, g.npts.z - 1};
    int lo[3];
    double penalty = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (f[d] < 0.0) {
            lo[d] = 0;
            penalty -= f[d];
            f[d] = 0.0;
        } else if (f[d] < static_cast<double>(npm1[d])) {
            lo[d] = static_cast<int>(f[d]);
        } else {
            lo[d] = npm1[d] - 1;
            penalty += f[d] - npm1[d];
            f[d] = npm1[d];
        }
    }
    const double x = f[0] - lo[0], y = f[1] - lo[1], z = f[2] - lo[2];
    const double mx = 1.0 - x, my = 1.0 - y, mz = 1.0 - z;
    const double w[8] = {mx * my * mz, x * my * mz, mx * y * mz, x * y * mz,
                         mx * my * z,  x * my * z,  mx * y * z,  x * y * z};
    const int sy = g.npts.z, sx = g.npts.y * g.npts.z;
    const int base = lo[0] * sx + lo[1] * sy + lo[2];
    const int off[8] = {base,     base + sx,     base + sy,     base + sx + sy,
                        base + 1, base + sx + 1, base + sy + 1, base + sx + sy + 1};
    double e = penalty > 0.0 ? penalty * g.spacing64 * g.slope64 : 0.0;
    double ec = 0.0, ev = 0.0;
    const size_t P = static_cast<size_t>(g.P);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        ec += (static_cast<double>(__ldg(&g.maps[off[c]].x)) + static_cast<double>(__ldg(&g.e_lo[off[c]]))) * w[c];
        if (slot > 0)
            ev += (static_cast<double>(__ldg(&g.maps[slot * P + off[c]].x)) +
                   static_cast<double>(__ldg(&g.e_lo[slot * P + off[c]]))) *
                  w[c];
    }
    return e + ec * q + ev;
}

// FP64 energy of the pose x = [ligand xyz (3N) | receptor torsions] (shared memory, the
// optimiser's flat layout). b.loc_grad serves as scratch for the FP64 positions of the
// receptor's local atoms (24 of its 64 bytes per atom); the next evaluation clears it.
static __device__ __noinline__ double energy64(const EvalEnv& env, const DevLigand& L, const float* x,
                                               const PoseBufs& b, int lane) {
    const int N = L.n_atoms;
    const int n3 = 3 * N;
    const DevReceptor& R = env.rec;
    double* loc64 = reinterpret_cast<double*>(b.loc_grad);
    // receptor rotor atoms (receptor_torsion2xyz, interaction.cpp:316-336; the Rodrigues
    // matrix of math.cpp:62-94)
    for (int l = lane; l < R.n_local; l += kWarp) {
        const double4 v = R.local_xyz064[l];
        double px = v.x, py = v.y, pz = v.z;
        if (l < R.n_mov) {
            const int r = static_cast<int>(v.w);
            const double4 k = R.rotor_axis64[r];
            const double4 o = R.rotor_origin64[r];
            double st, ct;
            sincos(static_cast<double>(x[n3 + r]), &st, &ct);
            const double omc = 1.0 - ct;
            const double r00 = ct + k.x * k.x * omc, r01 = k.x * k.y * omc - k.z * st, r02 = k.x * k.z * omc + k.y * st;
            const double r10 = k.y * k.x * omc + k.z * st, r11 = ct + k.y * k.y * omc, r12 = k.y * k.z * omc - k.x * st;
            const double r20 = k.z * k.x * omc - k.y * st, r21 = k.z * k.y * omc + k.x * st, r22 = ct + k.z * k.z * omc;
            px = r00 * v.x + r01 * v.y + r02 * v.z + o.x;
            py = r10 * v.x + r11 * v.y + r12 * v.z + o.y;
            pz = r20 * v.x + r21 * v.y + r22 * v.z + o.z;
        }
        loc64[3 * l] = px;
        loc64[3 * l + 1] = py;
        loc64[3 * l + 2] = pz;
    }
    __syncwarp();
    auto lig32 = [x](int i) { return make_float3(x[3 * i], x[3 * i + 1], x[3 * i + 2]); };
    auto lig64 = [x](int i) {
        return D3{static_cast<double>(x[3 * i]), static_cast<double>(x[3 * i + 1]), static_cast<double>(x[3 * i + 2])};
    };
    auto loc64f = [loc64](int l) { return D3{loc64[3 * l], loc64[3 * l + 1], loc64[3 * l + 2]}; };
    auto loc32 = [loc64](int l) {
        return make_float3(static_cast<float>(loc64[3 * l]), static_cast<float>(loc64[3 * l + 1]),
                           static_cast<float>(loc64[3 * l + 2]));
    };
    double e = topo_energy64(L.topo, lig32, lig64, lane);
    if (R.n_local > 0) e += topo_energy64(R.intra, loc32, loc64f, lane);
    if (env.grid.has_grid) {
        for (int a = lane; a < N; a += kWarp)
            e += grid_energy64(env.grid, __ldg(&L.map_slot[a]), __ldg(&L.charge64[a]), lig64(a));
    }
    // explicit inter pairs, one (ligand atom, receptor atom) pair per lane and step
    const int M = R.n_explicit;
    const int pairs = N * M;
    for (int k = lane; k < pairs; k += kWarp) {
        const int i = k / M, j = k - i * M;
        const int loc = __ldg(&R.ex_local[j]);
        const float4 rj = __ldg(&R.ex_xyzq[j]);
        const float3 xj = loc >= 0 ? loc32(loc) : xyz(rj);
        const float3 xi = lig32(i);
        const float2 sei = __ldg(&L.se[i]), sej = __ldg(&R.ex_se[j]);
        const float3 rij = sub3(xj, xi);
        const float rinv = rsqrtf(dot3(rij, rij));
        const float s = (sei.x + sej.x) * 0.5f;
        const float xx = s * s * rinv * rinv;
        const float u6 = xx * xx * xx;
        const float en = fmaf(sqrtf(sei.y * sej.y) * 4.f, u6 * u6 - u6, kCoulombF * __ldg(&L.charge[i]) * rj.w * rinv);
        if (fabsf(en) <= kPairFp64) {
            e += static_cast<double>(en);
        } else {
            const double4 r64 = R.ex_xyzq64[j];
            const double2 se64i = __ldg(&L.se64[i]), se64j = __ldg(&R.ex_se64[j]);
            const double sm = (se64i.x + se64j.x) * 0.5;
            const double4 p = make_double4(kCoulombD64 * __ldg(&L.charge64[i]) * r64.w,
                                           sqrt(se64i.y * se64j.y) * 4.0, sm * sm, 0.0);
            e += pair_energy64(p, lig64(i), loc >= 0 ? loc64f(loc) : D3{r64.x, r64.y, r64.z});
        }
    }
    return warp_sum_d(e) + R.e_const;
}

}  // namespace pxd
