// Receptor map build on the GPU: replaces receptor_cache::populate and
// partial_worker::populate (grid.cpp:115-195).
//
// One thread per (grid point, map); a block covers 128 consecutive points (k fastest)
// of one map, so all its threads read the same receptor-atom tile from shared memory
// (broadcast). Pair terms are FP32; each 256-atom tile's partial sums are folded into
// FP64 accumulators, which keeps the Coulomb sum over ~2k atoms of mixed sign accurate.
// Atom and point coordinates travel as FP32 hi + lo pairs, so each difference
// atom - point is formed to FP32 relative precision: a plain FP32 coordinate carries
// ~1e-6 A of rounding, which the 12th power of the LJ term would amplify 12-fold.
// The Coulomb map is summed in FP64 (see the loop).
// The squared distance is floored at 1e-4 A^2 so that a grid point sitting on an atom
// cannot overflow FP32, and records are clamped to +-1e30 before the FP32 store.
//
// The energy channel is also kept in FP64 for the final FP64 energy of a pose: every LJ
// pair term above kFp64Term kcal/mol in magnitude is recomputed in FP64 from FP64 sigma,
// epsilon and coordinates (an FP32 term carries ~1e-6 of its size, 100 kcal/mol on a
// 1e8 clash), the smaller ones stay FP32 (each under ~1e-8 kcal/mol of rounding, ~1e-6
// over a point's atoms), and the record's energy is the FP64 sum rounded to FP32 with the
// remainder stored in e_lo. The FP64 terms (atoms within ~6.5 A of the point) bound the
// build by the FP64 pipe.
#include "device_eval.cuh"
#include "../../include/pxdock_gb300_vdw.h"

namespace pxd {

constexpr int kGridThreads = 128;
constexpr int kGridTile = 256;
constexpr float kR2Floor = 1e-4f;
constexpr double kRecordCeil = 1e30;
constexpr double kCoulombD = 332.0637141491396;  // kCoulombFactor, system.h:83
constexpr float kFp64Term = 1e-2f;

struct GridArgs {
    const float4* atoms;   // x, y, z, charge of every non-rotor receptor atom (FP32 hi part)
    const float4* atoms_lo;// x, y, z, charge residuals: value - hi, in FP32
    const float2* se;      // sigma, epsilon
    const double2* se64;   // sigma, epsilon in FP64
    int n_atoms;
    int3 npts;
    double3 init;
    double spacing;
    const int* slot_type;  // [n_slots] ligand type, or -1 for the Coulomb map
    const float2* type_se; // [99] sigma, epsilon of the ligand types
    const double2* type_se64;
    float4* maps;
    float* e_lo;           // [n_slots][P] FP64 energy - FP32 record energy
    int P;
};

__device__ __forceinline__ float clampf_rec(double v) {
    return static_cast<float>(fmin(fmax(v, -kRecordCeil), kRecordCeil));
}

__global__ void __launch_bounds__(kGridThreads) grid_build_kernel(const GridArgs a) {
    __shared__ float4 s_xyzq[kGridTile];
    __shared__ float4 s_lo[kGridTile];
    __shared__ float2 s_se[kGridTile];
    __shared__ double2 s_se64[kGridTile];
    const int p = blockIdx.x * kGridThreads + threadIdx.x;
    const int slot = blockIdx.y;
    const int type = a.slot_type[slot];
    const bool coul = type < 0;
    const float2 tse = coul ? make_float2(0.f, 0.f) : a.type_se[type];
    const double2 tse64 = coul ? make_double2(0.0, 0.0) : a.type_se64[type];
    const int nz = a.npts.z, ny = a.npts.y;
    const int k = p % nz;
    const int j = (p / nz) % ny;
    const int i = p / (nz * ny);
    // grid.cpp:159-163: point = init + spacing * index, formed in FP64
    const double px = a.init.x + a.spacing * i, py = a.init.y + a.spacing * j, pz = a.init.z + a.spacing * k;
    const float3 pt = make_float3(static_cast<float>(px), static_cast<float>(py), static_cast<float>(pz));
    const float3 pl = make_float3(static_cast<float>(px - pt.x), static_cast<float>(py - pt.y),
                                  static_cast<float>(pz - pt.z));
    double E = 0.0, GX = 0.0, GY = 0.0, GZ = 0.0;
    double E64 = 0.0;  // LJ terms recomputed in FP64
    for (int t0 = 0; t0 < a.n_atoms; t0 += kGridTile) {
        const int n = min(kGridTile, a.n_atoms - t0);
        __syncthreads();
        for (int u = threadIdx.x; u < n; u += kGridThreads) {
            s_xyzq[u] = a.atoms[t0 + u];
            s_lo[u] = a.atoms_lo[t0 + u];
            s_se[u] = a.se[t0 + u];
            s_se64[u] = a.se64[t0 + u];
        }
        __syncthreads();
        float e = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
        if (coul) {
            // FP64 per pair: the map is a sum of ~M terms q/r of both signs that cancel
            // to a small fraction of their magnitudes, so FP32 rounding of each term
            // (~1e-7 relative) would leave ~1e-3 kcal/mol in the records
            double ce = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
            for (int u = 0; u < n; ++u) {
                const float4 at = s_xyzq[u];
                const float4 lo = s_lo[u];
                const double vx = (static_cast<double>(at.x) - px) + static_cast<double>(lo.x);
                const double vy = (static_cast<double>(at.y) - py) + static_cast<double>(lo.y);
                const double vz = (static_cast<double>(at.z) - pz) + static_cast<double>(lo.z);
                const double r2 = fmax(vx * vx + vy * vy + vz * vz, static_cast<double>(kR2Floor));
                const double rinv = rsqrt(r2);
                const double qr = (static_cast<double>(at.w) + static_cast<double>(lo.w)) * rinv;
                ce += qr;
                // dE/dpoint = q (atom - point) / r^3 (pair.h:25-40 with grad_i -= ...)
                const double w = qr * rinv * rinv;
                cx = fma(vx, w, cx);
                cy = fma(vy, w, cy);
                cz = fma(vz, w, cz);
            }
            E += ce * kCoulombD;
            GX += cx * kCoulombD;
            GY += cy * kCoulombD;
            GZ += cz * kCoulombD;
        } else {
            for (int u = 0; u < n; ++u) {
                const float4 at = s_xyzq[u];
                const float4 lo = s_lo[u];
                const float2 se = s_se[u];
                const float vx = (at.x - pt.x) + (lo.x - pl.x), vy = (at.y - pt.y) + (lo.y - pl.y),
                            vz = (at.z - pt.z) + (lo.z - pl.z);
                const float r2 = fmaxf(vx * vx + vy * vy + vz * vz, kR2Floor);
                const float rinv2 = 1.f / r2;
                const float s = (tse.x + se.x) * 0.5f;
                const float x = s * s * rinv2;
                const float u6 = x * x * x;
                const float u12 = u6 * u6;
                const float C = sqrtf(tse.y * se.y) * 4.f;
                const float ep = C * (u12 - u6);
                if (fabsf(ep) > kFp64Term) {
                    const double2 se64 = s_se64[u];
                    const double dx = (static_cast<double>(at.x) - px) + static_cast<double>(lo.x);
                    const double dy = (static_cast<double>(at.y) - py) + static_cast<double>(lo.y);
                    const double dz = (static_cast<double>(at.z) - pz) + static_cast<double>(lo.z);
                    const double r2d = fmax(dx * dx + dy * dy + dz * dz, static_cast<double>(kR2Floor));
                    const double sd = (tse64.x + se64.x) * 0.5;
                    const double xd = sd * sd / r2d;
                    const double u6d = xd * xd * xd;
                    E64 += sqrt(tse64.y * se64.y) * 4.0 * (u6d * u6d - u6d);
                } else {
                    e += ep;
                }
                // grad_point -= vec * de_dr_r, de_dr_r = C(-12 u12 + 6 u6) / r^2 (pair.h:42-60)
                const float w = C * (12.f * u12 - 6.f * u6) * rinv2;
                gx = fmaf(vx, w, gx);
                gy = fmaf(vy, w, gy);
                gz = fmaf(vz, w, gz);
            }
            E += e;
            GX += gx;
            GY += gy;
            GZ += gz;
        }
    }
    if (p < a.P) {
        const double Ef = E + E64;
        const float hi = clampf_rec(Ef);
        a.maps[static_cast<size_t>(slot) * a.P + p] = make_float4(hi, clampf_rec(GX), clampf_rec(GY), clampf_rec(GZ));
        const double rest = Ef - static_cast<double>(hi);
        a.e_lo[static_cast<size_t>(slot) * a.P + p] =
            fabs(Ef) < kRecordCeil ? static_cast<float>(rest) : 0.f;
    }
}

int launch_grid_build(pxd_context* ctx, const float4* atoms, const float4* atoms_lo, const float2* se,
                      const double2* se64, int n_atoms, const int* slot_type, int n_slots, float4* maps,
                      float* e_lo) {
    GridArgs a{};
    a.atoms = atoms;
    a.atoms_lo = atoms_lo;
    a.se = se;
    a.se64 = se64;
    a.e_lo = e_lo;
    a.n_atoms = n_atoms;
    a.npts = make_int3(ctx->box.npoints[0], ctx->box.npoints[1], ctx->box.npoints[2]);
    a.init = make_double3(ctx->box.init_xyz[0], ctx->box.init_xyz[1], ctx->box.init_xyz[2]);
    a.spacing = ctx->box.spacing;
    a.slot_type = slot_type;
    a.maps = maps;
    a.P = ctx->grid.P;
    // ligand type table on the device (sigma, epsilon)
    struct Tables {
        float2 f32[PXD_NUM_VDW_TYPES];
        double2 f64[PXD_NUM_VDW_TYPES];
    } table;
    for (int t = 0; t < PXD_NUM_VDW_TYPES; ++t) {
        table.f32[t] = make_float2(static_cast<float>(PXD_VDW_SIGMA[t]), static_cast<float>(PXD_VDW_EPSILON[t]));
        table.f64[t] = make_double2(PXD_VDW_SIGMA[t], PXD_VDW_EPSILON[t]);
    }
    Tables* d_table = nullptr;
    int rc = cuda_check(ctx, cudaMallocAsync(&d_table, sizeof(table), ctx->stream), "type table");
    if (rc) return rc;
    rc = cuda_check(ctx, cudaMemcpyAsync(d_table, &table, sizeof(table), cudaMemcpyHostToDevice,
                                         ctx->stream),
                    "type table copy");
    if (rc) {
        cudaFreeAsync(d_table, ctx->stream);
        return rc;
    }
    a.type_se = d_table->f32;
    a.type_se64 = d_table->f64;
    dim3 grid((a.P + kGridThreads - 1) / kGridThreads, n_slots);
    grid_build_kernel<<<grid, kGridThreads, 0, ctx->stream>>>(a);
    rc = cuda_check(ctx, cudaGetLastError(), "grid_build_kernel launch");
    cudaFreeAsync(d_table, ctx->stream);
    if (rc) return rc;
    return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "grid build");
}

}  // namespace pxd
