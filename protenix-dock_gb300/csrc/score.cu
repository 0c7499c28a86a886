// Empirical scores on the GPU: the pose-selection / affinity score kernel (one warp per
// pose) and the FP64 generalised-Born / surface-area term, with their C ABI.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pxdock_gb300_vdw.h"
#include "device_score.cuh"

namespace pxd {

// ------------------------------------------------------------------ uploads
struct Pack {
    std::vector<unsigned char> bytes;
    template <class T>
    size_t put(const std::vector<T>& v) {
        size_t off = (bytes.size() + 15) / 16 * 16;
        bytes.resize(off + v.size() * sizeof(T) + 16);
        if (!v.empty()) std::memcpy(bytes.data() + off, v.data(), v.size() * sizeof(T));
        return off;
    }
};

template <class T>
static const T* at(void* base, size_t off) {
    return reinterpret_cast<const T*>(static_cast<const unsigned char*>(base) + off);
}

static std::vector<int> ints(const int32_t* p, int n) {
    return n > 0 ? std::vector<int>(p, p + n) : std::vector<int>();
}

static std::vector<int2> pairs2(const int32_t* p, int n) {
    std::vector<int2> v;
    for (int i = 0; i < n; ++i) v.push_back(make_int2(p[2 * i], p[2 * i + 1]));
    return v;
}

// fill_atom_properties (scorer.cpp:737-753): GB radius by element, 1.3 for H bonded to N.
void gbsa_properties(const pxd_score_lists* l, int n, std::vector<double>& radius,
                     std::vector<double>& screen) {
    static const double kR[18] = {1.5, 1.2, 1.5, 1.5, 1.5, 1.5, 1.7, 1.55, 1.5,
                                  1.5, 1.5, 1.5, 1.5, 1.5, 2.1, 1.85, 1.8, 1.7};
    static const double kS[17] = {0.8, 0.85, 0.8, 0.8, 0.8, 0.8, 0.72, 0.79, 0.85,
                                  0.88, 0.8, 0.8, 0.8, 0.8, 0.8, 0.86, 0.96};
    radius.assign(n, -1.0);
    screen.assign(n, kS[0]);
    if (!l || !l->atomic_numbers) return;
    for (int b = 0; b < l->n_all_bonds; ++b) {
        const int i = l->all_bonds[2 * b], j = l->all_bonds[2 * b + 1];
        if (i < 0 || j < 0 || i >= n || j >= n) continue;
        const int ea = l->atomic_numbers[i], eb = l->atomic_numbers[j];
        if (ea == 1 && eb == 7) radius[i] = 1.3;
        else if (ea == 7 && eb == 1) radius[j] = 1.3;
    }
    for (int i = 0; i < n; ++i) {
        const int e = l->atomic_numbers[i];
        if (radius[i] < 0.0) radius[i] = (e >= 0 && e <= 17) ? kR[e] : kR[0];
        screen[i] = (e >= 0 && e <= 16) ? kS[e] : kS[0];
    }
}

// Pair-table class of an atom: ligand C N O S P F Cl other-heavy (0-7), receptor
// C N O other-heavy (0-3); hydrogens (and unknown elements, Z < 2) take none (-1).
int pair_class(int is_receptor, int z) {
    if (z < 2) return -1;
    switch (z) {
        case 6: return 0;
        case 7: return 1;
        case 8: return 2;
        default: break;
    }
    if (is_receptor) return 3;
    switch (z) {
        case 16: return 3;
        case 15: return 4;
        case 9: return 5;
        case 17: return 6;
        default: return 7;
    }
}

static float __int_as_float_host(int v) {
    float f;
    std::memcpy(&f, &v, sizeof(f));
    return f;
}

static std::vector<int> pair_classes(const pxd_score_lists* l, int n, int is_receptor) {
    std::vector<int> c;
    if (!l || !l->atomic_numbers) return c;
    c.resize(n);
    for (int i = 0; i < n; ++i) {
        const int k = pair_class(is_receptor, l->atomic_numbers[i]);
        c[i] = k < 0 ? -1 : (is_receptor ? k : 4 * k);
    }
    return c;
}

static bool ids_ok(const int32_t* p, int n, int limit) {
    for (int i = 0; i < n; ++i)
        if (p[i] < 0 || p[i] >= limit) return false;
    return true;
}

static bool lists_ok(const pxd_score_lists* l, int n_atoms) {
    if (!ids_ok(l->hydrophobic, l->n_hydrophobic, n_atoms) || !ids_ok(l->cation, l->n_cation, n_atoms) ||
        !ids_ok(l->anion, l->n_anion, n_atoms) || !ids_ok(l->don_charged, 2 * l->n_don_charged, n_atoms) ||
        !ids_ok(l->don_neutral, 2 * l->n_don_neutral, n_atoms) ||
        !ids_ok(l->acc_charged, l->n_acc_charged, n_atoms) || !ids_ok(l->acc_neutral, l->n_acc_neutral, n_atoms))
        return false;
    for (int k = 0; k < 2; ++k) {
        const int n = k ? l->n_ring6 : l->n_ring5;
        const int32_t* r = k ? l->ring6 : l->ring5;
        for (int i = 0; i < n; ++i) {
            int sz = 0;
            while (sz < 6 && r[6 * i + sz] >= 0) {
                if (r[6 * i + sz] >= n_atoms) return false;
                ++sz;
            }
            if (sz < 3) return false;
        }
    }
    for (int e = 0; e < l->n_tstrain; ++e) {
        if (l->tstrain_offsets[e] > l->tstrain_offsets[e + 1]) return false;
        for (int q = l->tstrain_offsets[e]; q < l->tstrain_offsets[e + 1]; ++q)
            if (!ids_ok(l->tstrain_quads + 4 * q, 4, n_atoms)) return false;
    }
    return true;
}

int upload_receptor_scoring(pxd_context* ctx, const pxd_score_lists* l, const std::vector<int>& local_of) {
    DevRecScore& d = ctx->rec_score;
    d = DevRecScore{};
    if (ctx->rec_score_mem) cudaFree(ctx->rec_score_mem);
    ctx->rec_score_mem = nullptr;
    const int M = ctx->n_rec;
    d.n_all = M;
    d.all_xyzq = at<float4>(ctx->rec_ex_all, ctx->ex_all_off[0]);
    d.all_se = at<float2>(ctx->rec_ex_all, ctx->ex_all_off[1]);
    d.all_local = at<int>(ctx->rec_ex_all, ctx->ex_all_off[2]);
    gbsa_properties(l, M, ctx->rec_gb_radius, ctx->rec_gb_screen);
    if (l && !lists_ok(l, M)) return set_error(ctx, PXD_ERR_INVALID, "receptor interaction list atom out of range");
    // per-atom record of the differentiable score's pair loop: sigma, sqrt(epsilon),
    // pair-table class, rotor-atom local index (-1: fixed)
    const std::vector<int> pcls = pair_classes(l, M, 1);
    std::vector<float4> pairrec(M);
    for (int a = 0; a < M; ++a)
        pairrec[a] = make_float4(static_cast<float>(ctx->rec_sigma[a]),
                                 static_cast<float>(std::sqrt(ctx->rec_epsilon[a])),
                                 __int_as_float_host(pcls.empty() ? -1 : pcls[a]),
                                 __int_as_float_host(ctx->is_mov[a] ? local_of[a] : -1));
    Pack pk;
    const size_t o_pair = pk.put(pairrec);
    if (!l) {
        int rc0 = cuda_check(ctx, cudaMalloc(&ctx->rec_score_mem, pk.bytes.size()), "receptor score lists");
        if (rc0) return rc0;
        rc0 = cuda_check(ctx, cudaMemcpy(ctx->rec_score_mem, pk.bytes.data(), pk.bytes.size(), cudaMemcpyHostToDevice),
                         "receptor score lists copy");
        if (rc0) return rc0;
        d.pair_rec = at<float4>(ctx->rec_score_mem, o_pair);
        return PXD_OK;
    }
    // ring centroids and normals (to_ring_centroid / to_ring_normal, scorer.cpp:128-172)
    std::vector<float4> rc[2], rn[2];
    for (int k = 0; k < 2; ++k) {
        const int n = k ? l->n_ring6 : l->n_ring5;
        const int32_t* r = k ? l->ring6 : l->ring5;
        for (int i = 0; i < n; ++i) {
            double c[3] = {0, 0, 0};
            int sz = 0;
            while (sz < 6 && r[6 * i + sz] >= 0) {
                const int a = r[6 * i + sz];
                if (ctx->is_mov[a]) return set_error(ctx, PXD_ERR_INVALID, "receptor ring atom on a rotor");
                for (int u = 0; u < 3; ++u) c[u] += ctx->rec_xyz[3 * a + u];
                ++sz;
            }
            for (int u = 0; u < 3; ++u) c[u] /= sz;
            const double* p0 = &ctx->rec_xyz[3 * r[6 * i]];
            const double* p1 = &ctx->rec_xyz[3 * r[6 * i + 1]];
            const double* p2 = &ctx->rec_xyz[3 * r[6 * i + 2]];
            const double e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
            const double e2[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
            double nn[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                            e1[0] * e2[1] - e1[1] * e2[0]};
            const double len = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
            rc[k].push_back(make_float4(static_cast<float>(c[0]), static_cast<float>(c[1]),
                                        static_cast<float>(c[2]), 0.f));
            rn[k].push_back(make_float4(static_cast<float>(nn[0] / len), static_cast<float>(nn[1] / len),
                                        static_cast<float>(nn[2] / len), 0.f));
        }
    }
    const size_t o_hyd = pk.put(ints(l->hydrophobic, l->n_hydrophobic));
    const size_t o_cat = pk.put(ints(l->cation, l->n_cation));
    const size_t o_an = pk.put(ints(l->anion, l->n_anion));
    const size_t o_r5c = pk.put(rc[0]), o_r5n = pk.put(rn[0]), o_r6c = pk.put(rc[1]), o_r6n = pk.put(rn[1]);
    const size_t o_donc = pk.put(pairs2(l->don_charged, l->n_don_charged));
    const size_t o_donn = pk.put(pairs2(l->don_neutral, l->n_don_neutral));
    const size_t o_accc = pk.put(ints(l->acc_charged, l->n_acc_charged));
    const size_t o_accn = pk.put(ints(l->acc_neutral, l->n_acc_neutral));
    const size_t o_pcl = pk.put(pcls);
    int rc_ = cuda_check(ctx, cudaMalloc(&ctx->rec_score_mem, pk.bytes.size()), "receptor score lists");
    if (rc_) return rc_;
    rc_ = cuda_check(ctx, cudaMemcpy(ctx->rec_score_mem, pk.bytes.data(), pk.bytes.size(), cudaMemcpyHostToDevice),
                     "receptor score lists copy");
    if (rc_) return rc_;
    void* b = ctx->rec_score_mem;
    d.has = 1;
    d.n_hyd = l->n_hydrophobic;
    d.n_cat = l->n_cation;
    d.n_an = l->n_anion;
    d.n_r5 = l->n_ring5;
    d.n_r6 = l->n_ring6;
    d.n_donc = l->n_don_charged;
    d.n_donn = l->n_don_neutral;
    d.n_accc = l->n_acc_charged;
    d.n_accn = l->n_acc_neutral;
    d.hyd = at<int>(b, o_hyd);
    d.cat = at<int>(b, o_cat);
    d.an = at<int>(b, o_an);
    d.r5c = at<float4>(b, o_r5c);
    d.r5n = at<float4>(b, o_r5n);
    d.r6c = at<float4>(b, o_r6c);
    d.r6n = at<float4>(b, o_r6n);
    d.donc = at<int2>(b, o_donc);
    d.donn = at<int2>(b, o_donn);
    d.accc = at<int>(b, o_accc);
    d.accn = at<int>(b, o_accn);
    d.pclass = pcls.empty() ? nullptr : at<int>(b, o_pcl);
    d.pair_rec = at<float4>(b, o_pair);
    return PXD_OK;
}

// Appends the ligand's lists to its device allocation image is not possible after the
// fact, so the lists get their own allocation owned by the ligand entry.
int upload_ligand_scoring(pxd_context* ctx, LigandEntry& e, const pxd_score_lists* l) {
    DevLigScore& d = e.dev.score;
    d = DevLigScore{};
    gbsa_properties(l, e.n_atoms, e.gb_radius, e.gb_screen);
    if (!l) return PXD_OK;
    if (!lists_ok(l, e.n_atoms)) return set_error(ctx, PXD_ERR_INVALID, "ligand interaction list atom out of range");
    std::vector<int> r5(6 * static_cast<size_t>(l->n_ring5)), r6(6 * static_cast<size_t>(l->n_ring6));
    for (size_t i = 0; i < r5.size(); ++i) r5[i] = l->ring5[i];
    for (size_t i = 0; i < r6.size(); ++i) r6[i] = l->ring6[i];
    std::vector<float4> tsc;
    std::vector<int2> tsr;
    std::vector<int4> tsq;
    for (int t = 0; t < l->n_tstrain; ++t) {
        const double* c = l->tstrain_coefs + 4 * t;
        tsc.push_back(make_float4(static_cast<float>(c[0]), static_cast<float>(c[1]), static_cast<float>(c[2]),
                                  static_cast<float>(c[3])));
        tsr.push_back(make_int2(l->tstrain_offsets[t], l->tstrain_offsets[t + 1] - l->tstrain_offsets[t]));
    }
    const int nq = l->n_tstrain ? l->tstrain_offsets[l->n_tstrain] : 0;
    for (int q = 0; q < nq; ++q)
        tsq.push_back(make_int4(l->tstrain_quads[4 * q], l->tstrain_quads[4 * q + 1], l->tstrain_quads[4 * q + 2],
                                l->tstrain_quads[4 * q + 3]));
    Pack pk;
    const size_t o_hyd = pk.put(ints(l->hydrophobic, l->n_hydrophobic));
    const size_t o_cat = pk.put(ints(l->cation, l->n_cation));
    const size_t o_an = pk.put(ints(l->anion, l->n_anion));
    const size_t o_r5 = pk.put(r5), o_r6 = pk.put(r6);
    const size_t o_donc = pk.put(pairs2(l->don_charged, l->n_don_charged));
    const size_t o_donn = pk.put(pairs2(l->don_neutral, l->n_don_neutral));
    const size_t o_accc = pk.put(ints(l->acc_charged, l->n_acc_charged));
    const size_t o_accn = pk.put(ints(l->acc_neutral, l->n_acc_neutral));
    const size_t o_tsc = pk.put(tsc), o_tsr = pk.put(tsr), o_tsq = pk.put(tsq);
    const std::vector<int> pcls = pair_classes(l, e.n_atoms, 0);
    const size_t o_pcl = pk.put(pcls);
    void* b = nullptr;
    int rc = cuda_check(ctx, cudaMalloc(&b, pk.bytes.size()), "ligand score lists");
    if (rc) return rc;
    rc = cuda_check(ctx, cudaMemcpy(b, pk.bytes.data(), pk.bytes.size(), cudaMemcpyHostToDevice),
                    "ligand score lists copy");
    if (rc) {
        cudaFree(b);
        return rc;
    }
    e.score_mem = b;
    d.has = 1;
    d.n_hyd = l->n_hydrophobic;
    d.n_cat = l->n_cation;
    d.n_an = l->n_anion;
    d.n_r5 = l->n_ring5;
    d.n_r6 = l->n_ring6;
    d.n_donc = l->n_don_charged;
    d.n_donn = l->n_don_neutral;
    d.n_accc = l->n_acc_charged;
    d.n_accn = l->n_acc_neutral;
    d.n_ts = l->n_tstrain;
    d.n_rot = l->n_rotatable;
    d.hyd = at<int>(b, o_hyd);
    d.cat = at<int>(b, o_cat);
    d.an = at<int>(b, o_an);
    d.r5 = at<int>(b, o_r5);
    d.r6 = at<int>(b, o_r6);
    d.donc = at<int2>(b, o_donc);
    d.donn = at<int2>(b, o_donn);
    d.accc = at<int>(b, o_accc);
    d.accn = at<int>(b, o_accn);
    d.ts_coef = at<float4>(b, o_tsc);
    d.ts_range = at<int2>(b, o_tsr);
    d.ts_quad = at<int4>(b, o_tsq);
    d.pclass = pcls.empty() ? nullptr : at<int>(b, o_pcl);
    return PXD_OK;
}

// ------------------------------------------------------------------ kernels
constexpr int kScoreWarps = 4;

struct EsArgs {
    ScoreEnv env;
    DevReceptor rec;
    const DevLigand* ligands;
    int n_ligands;
    const int* lig_ids;
    const float* xyz;
    const float* tors;
    int max_atoms;
    int n_poses;
    double* score;
    double* terms;
};

// Rotor atom positions for the torsions t (torsional_receptor::apply_parameters).
__device__ void receptor_rotors(const DevReceptor& R, const float* t, float4* loc, int lane) {
    for (int l = lane; l < R.n_mov; l += kWarp) {
        const float4 v = __ldg(&R.local_xyz0[l]);
        const int r = __float_as_int(v.w);
        Mat3 Rm, Jm;
        rotation_and_jacobian(xyz(__ldg(&R.rotor_axis[r])), t[r], Rm, Jm);
        const float3 p = add3(mat_apply(Rm, xyz(v)), xyz(__ldg(&R.rotor_origin[r])));
        loc[l] = make_float4(p.x, p.y, p.z, 0.f);
    }
    __syncwarp();
}

__global__ void __launch_bounds__(kScoreWarps * kWarp) empirical_score_kernel(const EsArgs a) {
    extern __shared__ __align__(16) float smem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int wib = threadIdx.x / kWarp;
    const int per_warp = 4 * (a.max_atoms + a.rec.n_mov + 1) + PXD_MAX_RECEPTOR_TORSIONS;
    float4* X = reinterpret_cast<float4*>(smem + wib * per_warp);
    float4* loc = X + a.max_atoms;
    float* tq = reinterpret_cast<float*>(loc + a.rec.n_mov + 1);
    const int R = a.rec.n_rotors;
    for (int pose = blockIdx.x * kScoreWarps + wib; pose < a.n_poses; pose += gridDim.x * kScoreWarps) {
        const int lid = a.lig_ids[pose];
        if (lid < 0 || lid >= a.n_ligands || !a.ligands[lid].score.has ||
            a.ligands[lid].n_atoms > a.max_atoms) {
            if (lane == 0) a.score[pose] = nan("");
            continue;
        }
        const DevLigand& L = a.ligands[lid];
        const float* px = a.xyz + static_cast<size_t>(pose) * a.max_atoms * 3;
        for (int i = lane; i < L.n_atoms; i += kWarp) X[i] = make_float4(px[3 * i], px[3 * i + 1], px[3 * i + 2], 0.f);
        for (int r = lane; r < R; r += kWarp) tq[r] = a.tors[static_cast<size_t>(pose) * R + r];
        __syncwarp();
        receptor_rotors(a.rec, tq, loc, lane);
        const double s = score_pose(a.env, L, L.score, X, loc, lane,
                                    a.terms ? a.terms + static_cast<size_t>(pose) * PXD_NUM_TERMS : nullptr);
        if (lane == 0) a.score[pose] = s;
        __syncwarp();
    }
}

// GB/SA (gbsa_total_energy::calculate, scorer.cpp:798-866) in FP64.
struct GbArgs {
    int n;
    const double* x;       // [n][3]
    const double* q;
    const double* radius;
    const double* screen;
    double* born;          // [n] out
    double* partial;       // [n] out: per-atom egb row + esa
};

__global__ void gb_born_kernel(const GbArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    const double offset = 0.09, alpha = 1.0, beta = 0.8, gamma = 4.85;
    const double orj = a.radius[j] - offset;
    const double xj = a.x[3 * j], yj = a.x[3 * j + 1], zj = a.x[3 * j + 2];
    double sum = 0.0;
    for (int i = 0; i < a.n; ++i) {
        if (i == j) continue;
        const double sr = (a.radius[i] - offset) * a.screen[i];
        const double dx = a.x[3 * i] - xj, dy = a.x[3 * i + 1] - yj, dz = a.x[3 * i + 2] - zj;
        const double r12 = sqrt(dx * dx + dy * dy + dz * dz);
        const double U = r12 + sr;
        if (U < orj) continue;
        const double r12i = 1.0 / r12;
        double D = fabs(r12 - sr);
        const double L = orj > D ? orj : D;
        const double Ui = 1.0 / U, Li = 1.0 / L;
        D = 0.25 * (r12 - sr * sr * r12i) * (Ui * Ui - Li * Li);
        D += (Li - Ui + 0.5 * log(L * Ui + 1e-20) * r12i);
        sum += 0.5 * D;
    }
    const double psi = sum * orj;
    const double t = tanh(alpha * psi - beta * psi * psi + gamma * psi * psi * psi);
    a.born[j] = 1.0 / (1.0 / orj - t / a.radius[j]);
}

__global__ void gb_energy_kernel(const GbArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const double kC = 332.0637141491396, solute = 1.0, solvent = 78.5;
    const double kappa = 0.09293963686178248, probe = 1.4, surface = 0.0678584012906;
    const double xi = a.x[3 * i], yi = a.x[3 * i + 1], zi = a.x[3 * i + 2];
    double egb = 0.0;
    for (int j = 0; j < a.n; ++j) {
        double f;
        if (i == j) {
            f = a.born[i];
        } else {
            const double dx = xi - a.x[3 * j], dy = yi - a.x[3 * j + 1], dz = zi - a.x[3 * j + 2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double bp = a.born[i] * a.born[j];
            f = sqrt(r2 + bp * exp(-0.25 * r2 / bp) + 1e-20);
        }
        const double pref = 0.5 * kC * (1.0 / solute - exp(-kappa * f) / solvent);
        egb -= a.q[i] * a.q[j] / f * pref;
    }
    const double rr = a.radius[i] + probe;
    a.partial[i] = egb + rr * rr * pow(a.radius[i] / a.born[i], 6.0) * surface;
}

static int gbsa_system(pxd_context* ctx, int n, const std::vector<double>& x, const std::vector<double>& q,
                       const std::vector<double>& radius, const std::vector<double>& screen, double* out) {
    if (n == 0) {
        *out = 0.0;
        return PXD_OK;
    }
    void* mem = nullptr;
    const size_t bytes = sizeof(double) * (3 * n + 5 * static_cast<size_t>(n));
    int rc = cuda_check(ctx, cudaMallocAsync(&mem, bytes, ctx->stream), "gbsa buffers");
    if (rc) return rc;
    double* d = static_cast<double*>(mem);
    GbArgs a{n, d, d + 3 * n, d + 4 * n, d + 5 * n, d + 6 * n, d + 7 * n};
    queue_copy(ctx, &rc, d, x.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream, "gbsa coordinates");
    queue_copy(ctx, &rc, d + 3 * n, q.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream, "gbsa charges");
    queue_copy(ctx, &rc, d + 4 * n, radius.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream,
               "gbsa radii");
    queue_copy(ctx, &rc, d + 5 * n, screen.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream,
               "gbsa screening");
    const int threads = 128, blocks = (n + threads - 1) / threads;
    if (!rc) {
        gb_born_kernel<<<blocks, threads, 0, ctx->stream>>>(a);
        gb_energy_kernel<<<blocks, threads, 0, ctx->stream>>>(a);
        rc = cuda_check(ctx, cudaGetLastError(), "gbsa kernels launch");
    }
    std::vector<double> part(n);
    queue_copy(ctx, &rc, part.data(), a.partial, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream, "gbsa sums");
    cudaFreeAsync(mem, ctx->stream);
    rc = sync_copies(ctx, rc, ctx->stream, "gbsa");
    if (rc) return rc;
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += part[i];
    *out = s;
    return PXD_OK;
}

}  // namespace pxd

using namespace pxd;

extern "C" {

int pxd_set_scoring_function(pxd_context* ctx, int32_t which, const pxd_sf_params* p) {
    if (!ctx || !p || which < 0 || which > 1) return PXD_ERR_INVALID;
    cudaSetDevice(ctx->device);
    DevSf h{};
    for (int k = 0; k < PXD_NUM_TERMS; ++k) h.coef[k] = static_cast<float>(p->coef[k]);
    h.vdw_scale = static_cast<float>(p->vdw_scale);
    h.vdw_cutoff = static_cast<float>(p->vdw_cutoff);
    for (int t = 0; t < PXD_NUM_VDW_TYPES; ++t) {
        // mm_interaction_vdw_energy constructor (scorer.cpp:207-220)
        h.vdw_type[t] = make_float2(static_cast<float>(PXD_VDW_SIGMA[t] * p->vdw_sigma_scale[t]),
                                    static_cast<float>(PXD_VDW_EPSILON[t] * p->vdw_epsilon_scale[t]));
        h.vdw_sigma_raw[t] = static_cast<float>(PXD_VDW_SIGMA[t]);
    }
    for (int k = 0; k < 2; ++k) {
        h.ionic_coef[k] = static_cast<float>(p->ionic_coef[k]);
        for (int u = 0; u < 2; ++u) h.ionic[k][u] = static_cast<float>(p->ionic[k][u]);
    }
    for (int k = 0; k < 4; ++k) {
        h.picat_coef[k] = static_cast<float>(p->picat_coef[k]);
        for (int u = 0; u < 2; ++u) h.picat[k][u] = static_cast<float>(p->picat[k][u]);
    }
    for (int w = 0; w < 2; ++w)
        for (int k = 0; k < 4; ++k) {
            h.stack_coef[w][k] = static_cast<float>(p->stack_coef[w][k]);
            for (int u = 0; u < 6; ++u) h.stack[w][k][u] = static_cast<float>(p->stack[w][k][u]);
        }
    h.hbond_scale = static_cast<float>(p->hbond_scale);
    for (int k = 0; k < 8; ++k) {
        h.hbond_coef[k] = static_cast<float>(p->hbond_coef[k]);
        for (int u = 0; u < 6; ++u) h.hbond[k][u] = static_cast<float>(p->hbond[k][u]);
    }
    h.hydro_scale = static_cast<float>(p->hydro_scale);
    h.hydro_min = static_cast<float>(p->hydro_dist_min);
    h.hydro_max = static_cast<float>(p->hydro_dist_max);
    h.hydro_factor = static_cast<float>(p->hydro_scale_factor);
    if (!ctx->d_sf[which]) {
        int rc = cuda_check(ctx, cudaMalloc(&ctx->d_sf[which], sizeof(DevSf)), "scoring function");
        if (rc) return rc;
    }
    int rc = cuda_check(ctx, cudaMemcpy(ctx->d_sf[which], &h, sizeof(DevSf), cudaMemcpyHostToDevice),
                        "scoring function copy");
    if (rc) return rc;
    ctx->sf_host[which] = *p;
    ctx->sf_set[which] = true;
    return PXD_OK;
}

int pxd_score_dev(pxd_context* ctx, int32_t which, int32_t n_poses, int32_t max_atoms, const int32_t* ids,
                  const float* xyz, const float* tors, double* score, double* terms, void* stream) {
    if (!ctx) return PXD_ERR_INVALID;
    if (which < 0 || which > 1 || n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS)
        return set_error(ctx, PXD_ERR_INVALID, "bad score batch");
    if (!ctx->has_receptor) return set_error(ctx, PXD_ERR_STATE, "set a receptor first");
    if (!ctx->sf_set[which]) return set_error(ctx, PXD_ERR_STATE, "set the scoring function first");
    if (ctx->rec.n_rotors > 0 && !tors) return set_error(ctx, PXD_ERR_INVALID, "receptor torsion buffer required");
    cudaSetDevice(ctx->device);
    if (n_poses == 0) return PXD_OK;
    int rc = sync_ligand_table(ctx);
    if (rc) return rc;
    EsArgs a{};
    a.env.rs = ctx->rec_score;
    a.env.sf = ctx->d_sf[which];
    a.rec = ctx->rec;
    a.ligands = ctx->d_ligands;
    a.n_ligands = static_cast<int>(ctx->ligands.size());
    a.lig_ids = ids;
    a.xyz = xyz;
    a.tors = tors;
    a.max_atoms = max_atoms;
    a.n_poses = n_poses;
    a.score = score;
    a.terms = terms;
    const int per_warp = 4 * (max_atoms + ctx->rec.n_mov + 1) + PXD_MAX_RECEPTOR_TORSIONS;
    const size_t smem = sizeof(float) * per_warp * kScoreWarps;
    if (smem > 48 * 1024) {
        rc = raise_smem_limit(ctx, reinterpret_cast<const void*>(empirical_score_kernel), smem, "score smem");
        if (rc) return rc;
    }
    int blocks = (n_poses + kScoreWarps - 1) / kScoreWarps;
    if (blocks > ctx->n_sm * 16) blocks = ctx->n_sm * 16;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    empirical_score_kernel<<<blocks, kScoreWarps * kWarp, smem, s>>>(a);
    return cuda_check(ctx, cudaGetLastError(), "empirical_score_kernel launch");
}

// Receptor coordinates for torsions t in FP64 (torsional_receptor::apply_parameters).
static std::vector<double> receptor_coords(pxd_context* ctx, const double* t) {
    std::vector<double> x = ctx->rec_xyz;
    for (int r = 0; r < ctx->rec.n_rotors; ++r) {
        const double* k = &ctx->rotor_axis[3 * r];
        const double* o = &ctx->rotor_origin[3 * r];
        const double st = std::sin(t[r]), ct = std::cos(t[r]), omc = 1 - ct;
        const double m[9] = {ct + k[0] * k[0] * omc,        k[0] * k[1] * omc - k[2] * st,
                             k[1] * st + k[0] * k[2] * omc, k[2] * st + k[0] * k[1] * omc,
                             ct + k[1] * k[1] * omc,        k[1] * k[2] * omc - k[0] * st,
                             k[0] * k[2] * omc - k[1] * st, k[0] * st + k[1] * k[2] * omc,
                             ct + k[2] * k[2] * omc};
        for (int u = ctx->rotor_mov_off[r]; u < ctx->rotor_mov_off[r + 1]; ++u) {
            double* p = &x[3 * static_cast<size_t>(ctx->mov_atoms[u])];
            const double v[3] = {p[0] - o[0], p[1] - o[1], p[2] - o[2]};
            for (int d = 0; d < 3; ++d) p[d] = m[3 * d] * v[0] + m[3 * d + 1] * v[1] + m[3 * d + 2] * v[2] + o[d];
        }
    }
    return x;
}

int pxd_score_gbsa(pxd_context* ctx, int32_t lig, const double* lig_xyz, const double* rec_tors, double* delta,
                   double* parts) {
    if (!ctx || !lig_xyz || !delta) return PXD_ERR_INVALID;
    if (!ctx->has_receptor) return set_error(ctx, PXD_ERR_STATE, "set a receptor first");
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size())) return set_error(ctx, PXD_ERR_INVALID, "ligand id");
    if (ctx->rec.n_rotors > 0 && !rec_tors) return set_error(ctx, PXD_ERR_INVALID, "receptor torsions required");
    cudaSetDevice(ctx->device);
    const LigandEntry& e = ctx->ligands[lig];
    const int nl = e.n_atoms, nr = ctx->n_rec;
    std::vector<double> rx = receptor_coords(ctx, rec_tors);
    std::vector<double> lx(lig_xyz, lig_xyz + 3 * static_cast<size_t>(nl));
    double e_pro = 0, e_lig = 0, e_com = 0;
    int rc = gbsa_system(ctx, nr, rx, ctx->rec_charge, ctx->rec_gb_radius, ctx->rec_gb_screen, &e_pro);
    if (rc) return rc;
    rc = gbsa_system(ctx, nl, lx, e.charge, e.gb_radius, e.gb_screen, &e_lig);
    if (rc) return rc;
    // complex: ligand atoms first, then the receptor (scorer.cpp:770-780)
    std::vector<double> cx = lx, cq = e.charge, cr = e.gb_radius, cs = e.gb_screen;
    cx.insert(cx.end(), rx.begin(), rx.end());
    cq.insert(cq.end(), ctx->rec_charge.begin(), ctx->rec_charge.end());
    cr.insert(cr.end(), ctx->rec_gb_radius.begin(), ctx->rec_gb_radius.end());
    cs.insert(cs.end(), ctx->rec_gb_screen.begin(), ctx->rec_gb_screen.end());
    rc = gbsa_system(ctx, nl + nr, cx, cq, cr, cs, &e_com);
    if (rc) return rc;
    *delta = e_com - e_lig - e_pro;
    if (parts) {
        parts[0] = e_com;
        parts[1] = e_lig;
        parts[2] = e_pro;
    }
    return PXD_OK;
}

int pxd_score(pxd_context* ctx, int32_t which, int32_t lig, int32_t n_poses, const double* xyz, const double* tors,
              double* score, double* terms) {
    if (!ctx) return PXD_ERR_INVALID;
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size()) || n_poses < 0 || which < 0 || which > 1)
        return set_error(ctx, PXD_ERR_INVALID, "ligand id / batch");
    if (!ctx->has_receptor) return set_error(ctx, PXD_ERR_STATE, "set a receptor first");
    cudaSetDevice(ctx->device);
    const int N = ctx->ligands[lig].n_atoms, R = ctx->rec.n_rotors;
    const size_t nx = static_cast<size_t>(n_poses) * N * 3, nt = static_cast<size_t>(n_poses) * R;
    std::vector<float> hx(nx), ht(nt);
    for (size_t i = 0; i < nx; ++i) hx[i] = static_cast<float>(xyz[i]);
    for (size_t i = 0; i < nt; ++i) ht[i] = static_cast<float>(tors[i]);
    std::vector<int> ids(n_poses, lig);
    void* mem = nullptr;
    const size_t bytes = 4 * (nx + nt + n_poses) + 8 * (n_poses + static_cast<size_t>(n_poses) * PXD_NUM_TERMS) + 64;
    int rc = cuda_check(ctx, cudaMallocAsync(&mem, bytes, ctx->stream), "score staging");
    if (rc) return rc;
    double* d_s = static_cast<double*>(mem);
    double* d_t = d_s + n_poses;
    float* d_x = reinterpret_cast<float*>(d_t + static_cast<size_t>(n_poses) * PXD_NUM_TERMS);
    float* d_r = d_x + nx;
    int* d_i = reinterpret_cast<int*>(d_r + nt + 1);
    queue_copy(ctx, &rc, d_x, hx.data(), 4 * nx, cudaMemcpyHostToDevice, ctx->stream, "score coordinates");
    if (nt) queue_copy(ctx, &rc, d_r, ht.data(), 4 * nt, cudaMemcpyHostToDevice, ctx->stream, "score torsions");
    queue_copy(ctx, &rc, d_i, ids.data(), 4 * static_cast<size_t>(n_poses), cudaMemcpyHostToDevice, ctx->stream,
               "score ligand ids");
    if (!rc) rc = pxd_score_dev(ctx, which, n_poses, N, d_i, d_x, d_r, d_s, d_t, ctx->stream);
    std::vector<double> ht2(static_cast<size_t>(n_poses) * PXD_NUM_TERMS);
    queue_copy(ctx, &rc, score, d_s, 8 * static_cast<size_t>(n_poses), cudaMemcpyDeviceToHost, ctx->stream,
               "scores");
    queue_copy(ctx, &rc, ht2.data(), d_t, 8 * ht2.size(), cudaMemcpyDeviceToHost, ctx->stream, "score terms");
    cudaFreeAsync(mem, ctx->stream);
    rc = sync_copies(ctx, rc, ctx->stream, "score");
    if (rc) return rc;
    const double gcoef = ctx->sf_host[which].coef[PXD_TERM_GBSA];
    for (int p = 0; p < n_poses; ++p) {
        if (gcoef > 1e-5 || gcoef < -1e-5) {
            double g = 0.0;
            rc = pxd_score_gbsa(ctx, lig, xyz + 3 * static_cast<size_t>(N) * p, tors + static_cast<size_t>(R) * p, &g,
                                nullptr);
            if (rc) return rc;
            ht2[static_cast<size_t>(p) * PXD_NUM_TERMS + PXD_TERM_GBSA] = g;
            score[p] += gcoef * g;
        }
        if (terms)
            for (int k = 0; k < PXD_NUM_TERMS; ++k)
                terms[static_cast<size_t>(p) * PXD_NUM_TERMS + k] = ht2[static_cast<size_t>(p) * PXD_NUM_TERMS + k];
    }
    return PXD_OK;
}

}  // extern "C"
