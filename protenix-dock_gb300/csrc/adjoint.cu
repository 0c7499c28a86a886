// Differentiable empirical score on the GPU: score_adjoint_kernel (one warp per pose,
// persistent blocks) with its deterministic reductions, the C ABI, and the
// device-buffer pose kinematics used by gradient pipelines.
//
// Per block, the weight gradient (36 doubles per warp, each warp adding its poses in
// order) and the pair-table gradient (8,192 floats, shared atomics) are accumulated in
// shared memory and written once as a per-block partial; partial_sum_kernel then adds
// the partials of all blocks in a fixed order, in FP64, into the caller's accumulators.
// No global atomics: scores, coordinate and weight gradients repeat bit for bit; the
// table gradient's shared atomics leave its last bits to the order of arrival.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "device_adjoint.cuh"

namespace pxd {

constexpr int kAdjWarps = 8;

// One receptor context as the kernel sees it.
struct AdjCtx {
    ScoreEnv env;
    DevReceptor rec;
    const DevLigand* ligands;
    int n_ligands;
};

struct AdjArgs {
    AdjCtx one;              // the context of every pose (single-context launch)
    const AdjCtx* ctxs;      // [n_contexts] (multi-context launch)
    const int* ctx_ids;      // [n_poses] (multi-context launch)
    int max_mov;             // largest rotor-atom count over the contexts
    int tors_stride;         // receptor torsions per pose row
    const int* lig_ids;
    const float* xyz;
    const float* xyz_t;      // [n_poses][max_atoms][3] direction (tangent launches)
    const float* tors;
    int max_atoms;
    int n_poses;
    const double* weights;   // [36]
    const float* tables;     // [32 * 256] or NULL
    const double* grad_out;  // [n_poses] (adjoint kernel only)
    double* score;           // [n_poses] or NULL
    double* features;        // [n_poses][28] or NULL
    float* dxyz;             // [n_poses][max_atoms][3] or NULL
    double* part_w;          // [gridDim][36] per-block weight-gradient partials
    float* part_t;           // [gridDim][32 * 256] per-block table-gradient partials or NULL
};

// Rotor atom positions for the torsions t (torsional_receptor::apply_parameters).
__device__ void adj_receptor_rotors(const DevReceptor& R, const float* t, float4* loc, int lane) {
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

// S = float: scores, features and gradients; S = Dual: their derivatives along xyz_t.
template <bool kGrad, bool kMulti, class S>
__global__ void __launch_bounds__(kAdjWarps * kWarp, 2) score_adjoint_kernel(const __grid_constant__ AdjArgs a) {
    extern __shared__ __align__(16) unsigned char adj_smem[];
    double* s_w = reinterpret_cast<double*>(adj_smem);  // [36] weights
    double* s_dw = s_w + kNumW;                         // [warps][36] weight gradient per warp
    float* s_wf = reinterpret_cast<float*>(s_dw + kAdjWarps * kNumW);  // [36] FP32 weights
    float* s_tg = s_wf + kNumW + 4;                     // [32 * 256] when table gradients are asked for
    const bool tgrad = kGrad && a.part_t && a.tables;
    float* warp_base = tgrad ? s_tg + kTabN : s_tg;
    const int lane = threadIdx.x & (kWarp - 1);
    const int wib = threadIdx.x / kWarp;
    constexpr int kSlices = IsDual<S>::value ? 3 : 2;  // X, G (and the tangents XT)
    const int per_warp = 4 * (kSlices * a.max_atoms + a.max_mov + 1) + PXD_MAX_RECEPTOR_TORSIONS;
    float4* X = reinterpret_cast<float4*>(warp_base + wib * per_warp);
    float4* G = X + a.max_atoms;
    float4* XT = G + a.max_atoms;
    float4* loc = G + (kSlices - 1) * a.max_atoms;
    float* tq = reinterpret_cast<float*>(loc + a.max_mov + 1);
    for (int k = threadIdx.x; k < kNumW; k += blockDim.x) {
        s_w[k] = a.weights[k];
        s_wf[k] = static_cast<float>(a.weights[k]);
    }
    for (int k = threadIdx.x; k < kAdjWarps * kNumW; k += blockDim.x) s_dw[k] = 0.0;
    if (tgrad)
        for (int k = threadIdx.x; k < kTabN; k += blockDim.x) s_tg[k] = 0.f;
    __syncthreads();
    for (int pose = blockIdx.x * kAdjWarps + wib; pose < a.n_poses; pose += gridDim.x * kAdjWarps) {
        const AdjCtx& C = kMulti ? a.ctxs[a.ctx_ids[pose]] : a.one;
        const int R = C.rec.n_rotors;
        const int lid = a.lig_ids[pose];
        float* dx = kGrad && a.dxyz ? a.dxyz + static_cast<size_t>(pose) * a.max_atoms * 3 : nullptr;
        if (lid < 0 || lid >= C.n_ligands || !C.ligands[lid].score.has || C.ligands[lid].n_atoms > a.max_atoms) {
            if (lane == 0 && a.score) a.score[pose] = nan("");
            if (dx)
                for (int e = lane; e < 3 * a.max_atoms; e += kWarp) dx[e] = 0.f;
            continue;
        }
        const DevLigand& L = C.ligands[lid];
        const float* px = a.xyz + static_cast<size_t>(pose) * a.max_atoms * 3;
        for (int i = lane; i < L.n_atoms; i += kWarp) {
            X[i] = make_float4(px[3 * i], px[3 * i + 1], px[3 * i + 2], 0.f);
            G[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        if (IsDual<S>::value) {
            const float* pt = a.xyz_t + static_cast<size_t>(pose) * a.max_atoms * 3;
            for (int i = lane; i < L.n_atoms; i += kWarp) XT[i] = make_float4(pt[3 * i], pt[3 * i + 1], pt[3 * i + 2], 0.f);
        }
        for (int r = lane; r < R; r += kWarp) tq[r] = a.tors[static_cast<size_t>(pose) * a.tors_stride + r];
        __syncwarp();
        adj_receptor_rotors(C.rec, tq, loc, lane);
        AdjPose ap;
        ap.wf = s_wf;
        ap.tab = a.tables;
        ap.tgrad = tgrad ? s_tg : nullptr;
        ap.g = kGrad ? static_cast<float>(a.grad_out[pose]) : 0.f;
        double f[kNumF];
        score_adjoint_pose<kGrad, S>(C.env, L, X, XT, loc, ap, G, lane, f);
        if (!IsDual<S>::value && a.score && lane == 0) a.score[pose] = combine_features(s_w, f);
        if (a.features) {
            double* fo = a.features + static_cast<size_t>(pose) * kNumF;
#pragma unroll
            for (int k = 0; k < kNumF; ++k)
                if (lane == (k & (kWarp - 1))) fo[k] = f[k];
        }
        if (kGrad) {
            if (lane == 0) combine_grad(s_w, f, a.grad_out[pose], s_dw + wib * kNumW);
            __syncwarp();
            if (dx) {
                for (int i = lane; i < a.max_atoms; i += kWarp) {
                    const float4 g = i < L.n_atoms ? G[i] : make_float4(0.f, 0.f, 0.f, 0.f);
                    dx[3 * i] = g.x;
                    dx[3 * i + 1] = g.y;
                    dx[3 * i + 2] = g.z;
                }
            }
        }
        __syncwarp();
    }
    if (!kGrad) return;
    __syncthreads();
    for (int k = threadIdx.x; k < kNumW; k += blockDim.x) {
        double t = 0.0;
        for (int w = 0; w < kAdjWarps; ++w) t += s_dw[w * kNumW + k];
        a.part_w[static_cast<size_t>(blockIdx.x) * kNumW + k] = t;
    }
    if (tgrad) {
        float* pt = a.part_t + static_cast<size_t>(blockIdx.x) * kTabN;
        for (int k = threadIdx.x; k < kTabN; k += blockDim.x) pt[k] = s_tg[k];
    }
}

// out[k] += sum over blocks b (in order) of part[b][k], in FP64.
template <class T>
__global__ void partial_sum_kernel(const T* __restrict__ part, int n_blocks, int n, double* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double s = 0.0;
    for (int b = 0; b < n_blocks; ++b) s += static_cast<double>(part[static_cast<size_t>(b) * n + k]);
    out[k] += s;
}

static size_t adj_smem_bytes(int max_atoms, int n_mov, bool tgrad, bool tangent) {
    const size_t per_warp =
        4 * ((tangent ? 3 : 2) * static_cast<size_t>(max_atoms) + n_mov + 1) + PXD_MAX_RECEPTOR_TORSIONS;
    return sizeof(double) * (1 + kAdjWarps) * kNumW + sizeof(float) * (kNumW + 4) +
           (tgrad ? sizeof(float) * kTabN : 0) +
           sizeof(float) * per_warp * kAdjWarps;
}

}  // namespace pxd

using namespace pxd;

extern "C" {

void pxd_sf_weights(const pxd_sf_params* p, double* w) {
    if (!p || !w) return;
    for (int k = 0; k < PXD_NUM_TERMS; ++k) w[PXD_W_COEF + k] = p->coef[k];
    w[PXD_W_VDW_SCALE] = p->vdw_scale;
    w[PXD_W_HYDRO_SCALE] = p->hydro_scale;
    w[PXD_W_HBOND_SCALE] = p->hbond_scale;
    for (int k = 0; k < 2; ++k) w[PXD_W_IONIC + k] = p->ionic_coef[k];
    for (int k = 0; k < 4; ++k) w[PXD_W_PICAT + k] = p->picat_coef[k];
    for (int q = 0; q < 2; ++q)
        for (int k = 0; k < 4; ++k) w[PXD_W_STACK + 4 * q + k] = p->stack_coef[q][k];
    for (int k = 0; k < 8; ++k) w[PXD_W_HBOND + k] = p->hbond_coef[k];
}

int pxd_score_adjoint_dev(pxd_context* ctx, int32_t which, int32_t n_poses, int32_t max_atoms, const int32_t* ids,
                          const float* xyz, const float* tors, const double* weights, const float* tables,
                          const double* grad_out, double* score, double* features, float* dxyz, double* dweights,
                          double* dtables, void* stream) {
    if (!ctx) return PXD_ERR_INVALID;
    pxd_context* one[1] = {ctx};
    return pxd_score_adjoint_multi_dev(one, 1, which, n_poses, max_atoms, nullptr, ids, xyz, tors, weights, tables,
                                       grad_out, score, features, dxyz, dweights, dtables, stream);
}

}  // extern "C"

namespace pxd {

// Shared launcher of the value, adjoint (xyz_t NULL) and tangent (xyz_t set) launches.
static int launch_adjoint(pxd_context* const* ctxs, int32_t n_ctx, int32_t which, int32_t n_poses,
                          int32_t max_atoms, const int32_t* ctx_ids, const int32_t* ids, const float* xyz,
                          const float* xyz_t, const float* tors, const double* weights, const float* tables,
                          const double* grad_out, double* score, double* features, float* dxyz, double* dweights,
                          double* dtables, void* stream) {
    if (!ctxs || n_ctx < 1 || !ctxs[0]) return PXD_ERR_INVALID;
    pxd_context* ctx = ctxs[0];  // errors are reported here
    if (which < 0 || which > 1 || n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS || !weights ||
        (n_ctx > 1 && !ctx_ids))
        return set_error(ctx, PXD_ERR_INVALID, "bad adjoint batch");
    if (grad_out && !dweights && !dxyz && !dtables)
        return set_error(ctx, PXD_ERR_INVALID, "adjoint call without a gradient output");
    const bool tangent = xyz_t != nullptr;
    if (tangent && !grad_out) return set_error(ctx, PXD_ERR_INVALID, "a tangent launch needs grad_out");
    cudaSetDevice(ctx->device);
    const bool multi = n_ctx > 1;
    std::vector<AdjCtx> table(n_ctx);
    int max_mov = 0, max_rot = 0;
    for (int c = 0; c < n_ctx; ++c) {
        pxd_context* k = ctxs[c];
        if (!k || k->device != ctx->device)
            return set_error(ctx, PXD_ERR_INVALID, "contexts must be distinct, non-null and on one device");
        if (!k->has_receptor) return set_error(ctx, PXD_ERR_STATE, "set a receptor first");
        if (!k->sf_set[which]) return set_error(ctx, PXD_ERR_STATE, "set the scoring function first");
        if (k->rec.n_rotors > 0 && !tors) return set_error(ctx, PXD_ERR_INVALID, "receptor torsion buffer required");
        int rc = sync_ligand_table(k);
        if (rc) return set_error(ctx, rc, k->error);
        table[c].env.rs = k->rec_score;
        table[c].env.sf = k->d_sf[which];
        table[c].rec = k->rec;
        table[c].ligands = k->d_ligands;
        table[c].n_ligands = static_cast<int>(k->ligands.size());
        max_mov = std::max(max_mov, k->rec.n_mov);
        max_rot = std::max(max_rot, k->rec.n_rotors);
    }
    if (n_poses == 0) return PXD_OK;
    const bool grad = grad_out != nullptr;
    const bool tgrad = grad && dtables && tables;
    const size_t smem = adj_smem_bytes(max_atoms, max_mov, tgrad, tangent);
    if (smem > 227 * 1024) return set_error(ctx, PXD_ERR_INVALID, "adjoint shared memory beyond 227 KB: lower max_atoms");
    const void* fn;
    if (tangent)
        fn = multi ? reinterpret_cast<const void*>(score_adjoint_kernel<true, true, Dual>)
                   : reinterpret_cast<const void*>(score_adjoint_kernel<true, false, Dual>);
    else if (grad)
        fn = multi ? reinterpret_cast<const void*>(score_adjoint_kernel<true, true, float>)
                   : reinterpret_cast<const void*>(score_adjoint_kernel<true, false, float>);
    else
        fn = multi ? reinterpret_cast<const void*>(score_adjoint_kernel<false, true, float>)
                   : reinterpret_cast<const void*>(score_adjoint_kernel<false, false, float>);
    int rc = raise_smem_limit(ctx, fn, smem, "adjoint smem");
    if (rc) return rc;
    int per_sm = 0;
    rc = cuda_check(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kAdjWarps * kWarp, smem),
                    "adjoint occupancy");
    if (rc) return rc;
    if (per_sm < 1) per_sm = 1;
    int blocks = (n_poses + kAdjWarps - 1) / kAdjWarps;
    if (blocks > ctx->n_sm * per_sm) blocks = ctx->n_sm * per_sm;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    AdjArgs a{};
    a.one = table[0];
    a.ctxs = nullptr;
    a.ctx_ids = ctx_ids;
    a.max_mov = max_mov;
    a.tors_stride = max_rot;
    a.lig_ids = ids;
    a.xyz = xyz;
    a.xyz_t = xyz_t;
    a.tors = tors;
    a.max_atoms = max_atoms;
    a.n_poses = n_poses;
    a.weights = weights;
    a.tables = tables;
    a.grad_out = grad_out;
    a.score = tangent ? nullptr : score;
    a.features = features;
    a.dxyz = dxyz;
    a.part_w = nullptr;
    a.part_t = nullptr;
    // one stream-ordered allocation: context table, weight and table partials
    const size_t cbytes = multi ? (sizeof(AdjCtx) * n_ctx + 255) / 256 * 256 : 0;
    const size_t wbytes = grad ? (sizeof(double) * kNumW * blocks + 255) / 256 * 256 : 0;
    const size_t tbytes = tgrad ? sizeof(float) * kTabN * blocks : 0;
    void* mem = nullptr;
    if (cbytes + wbytes + tbytes) {
        rc = cuda_check(ctx, cudaMallocAsync(&mem, cbytes + wbytes + tbytes, s), "adjoint scratch");
        if (rc) return rc;
    }
    char* base = static_cast<char*>(mem);
    if (multi) {
        rc = cuda_check(ctx, cudaMemcpyAsync(base, table.data(), sizeof(AdjCtx) * n_ctx, cudaMemcpyHostToDevice, s),
                        "context table copy");
        a.ctxs = reinterpret_cast<const AdjCtx*>(base);
    }
    if (grad) a.part_w = reinterpret_cast<double*>(base + cbytes);
    if (tgrad) a.part_t = reinterpret_cast<float*>(base + cbytes + wbytes);
    if (!rc) {
        void* params[] = {&a};
        rc = cuda_check(ctx, cudaLaunchKernel(fn, dim3(blocks), dim3(kAdjWarps * kWarp), params, smem, s),
                        "score_adjoint_kernel launch");
    }
    if (!rc && grad && dweights) {
        partial_sum_kernel<double><<<1, 64, 0, s>>>(a.part_w, blocks, kNumW, dweights);
        rc = cuda_check(ctx, cudaGetLastError(), "partial_sum_kernel launch");
    }
    if (!rc && tgrad) {
        partial_sum_kernel<float><<<(kTabN + 255) / 256, 256, 0, s>>>(a.part_t, blocks, kTabN, dtables);
        rc = cuda_check(ctx, cudaGetLastError(), "partial_sum_kernel launch");
    }
    if (mem) cudaFreeAsync(mem, s);
    return rc;
}

}  // namespace pxd

extern "C" {

int pxd_score_adjoint_multi_dev(pxd_context* const* ctxs, int32_t n_ctx, int32_t which, int32_t n_poses,
                                int32_t max_atoms, const int32_t* ctx_ids, const int32_t* ids, const float* xyz,
                                const float* tors, const double* weights, const float* tables,
                                const double* grad_out, double* score, double* features, float* dxyz,
                                double* dweights, double* dtables, void* stream) {
    return launch_adjoint(ctxs, n_ctx, which, n_poses, max_atoms, ctx_ids, ids, xyz, nullptr, tors, weights, tables,
                          grad_out, score, features, dxyz, dweights, dtables, stream);
}

int pxd_score_hvp_multi_dev(pxd_context* const* ctxs, int32_t n_ctx, int32_t which, int32_t n_poses,
                            int32_t max_atoms, const int32_t* ctx_ids, const int32_t* ids, const float* xyz,
                            const float* xyz_dir, const float* tors, const double* weights, const float* tables,
                            const double* grad_out, double* features_dir, float* dxyz_dir, double* dweights_dir,
                            double* dtables_dir, void* stream) {
    if (!xyz_dir) return ctxs && ctxs[0] ? set_error(ctxs[0], PXD_ERR_INVALID, "direction required") : PXD_ERR_INVALID;
    return launch_adjoint(ctxs, n_ctx, which, n_poses, max_atoms, ctx_ids, ids, xyz, xyz_dir, tors, weights, tables,
                          grad_out, nullptr, features_dir, dxyz_dir, dweights_dir, dtables_dir, stream);
}

int pxd_score_adjoint(pxd_context* ctx, int32_t which, int32_t lig, int32_t n_poses, const double* xyz,
                      const double* tors, const double* weights, const double* tables, const double* grad_out,
                      double* score, double* features, double* dxyz, double* dweights, double* dtables) {
    if (!ctx) return PXD_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size()) || n_poses < 0 || !weights)
        return set_error(ctx, PXD_ERR_INVALID, "ligand id");
    if (n_poses == 0) return PXD_OK;
    const int N = ctx->ligands[lig].n_atoms, R = ctx->rec.n_rotors;
    const size_t nx = static_cast<size_t>(n_poses) * N * 3;
    std::vector<float> hx(nx), ht(static_cast<size_t>(n_poses) * R), htab;
    for (size_t i = 0; i < nx; ++i) hx[i] = static_cast<float>(xyz[i]);
    for (size_t i = 0; i < ht.size(); ++i) ht[i] = static_cast<float>(tors[i]);
    if (tables) htab.assign(tables, tables + kTabN);
    std::vector<float> htabf(htab.begin(), htab.end());
    std::vector<double> hg(n_poses, 1.0);
    if (grad_out) hg.assign(grad_out, grad_out + n_poses);
    std::vector<int> ids(n_poses, lig);
    const bool grad = dxyz || dweights || dtables;
    int rc;
    Staging st{ctx, {}};
    float* d_x = st.alloc<float>(nx, &rc);
    if (rc) return rc;
    float* d_t = st.alloc<float>(ht.size(), &rc);
    if (rc) return rc;
    int* d_ids = st.alloc<int>(n_poses, &rc);
    if (rc) return rc;
    double* d_w = st.alloc<double>(kNumW, &rc);
    if (rc) return rc;
    float* d_tab = tables ? st.alloc<float>(kTabN, &rc) : nullptr;
    if (rc) return rc;
    double* d_g = st.alloc<double>(n_poses, &rc);
    if (rc) return rc;
    double* d_s = st.alloc<double>(n_poses, &rc);
    if (rc) return rc;
    double* d_f = st.alloc<double>(static_cast<size_t>(n_poses) * kNumF, &rc);
    if (rc) return rc;
    float* d_dx = st.alloc<float>(nx, &rc);
    if (rc) return rc;
    double* d_dw = st.alloc<double>(kNumW, &rc);
    if (rc) return rc;
    double* d_dt = st.alloc<double>(kTabN, &rc);
    if (rc) return rc;
    cudaStream_t s = ctx->stream;
    queue_copy(ctx, &rc, d_x, hx.data(), nx * 4, cudaMemcpyHostToDevice, s);
    if (!ht.empty()) queue_copy(ctx, &rc, d_t, ht.data(), ht.size() * 4, cudaMemcpyHostToDevice, s);
    queue_copy(ctx, &rc, d_ids, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice, s);
    queue_copy(ctx, &rc, d_w, weights, kNumW * 8, cudaMemcpyHostToDevice, s);
    if (tables) queue_copy(ctx, &rc, d_tab, htabf.data(), kTabN * 4, cudaMemcpyHostToDevice, s);
    queue_copy(ctx, &rc, d_g, hg.data(), hg.size() * 8, cudaMemcpyHostToDevice, s);
    if (!rc) rc = cuda_check(ctx, cudaMemsetAsync(d_dw, 0, kNumW * 8, s), "weight gradient clear");
    if (!rc) rc = cuda_check(ctx, cudaMemsetAsync(d_dt, 0, kTabN * 8, s), "table gradient clear");
    if (rc) return rc;
    rc = pxd_score_adjoint_dev(ctx, which, n_poses, N, d_ids, d_x, d_t, d_w, d_tab, grad ? d_g : nullptr, d_s, d_f,
                               grad ? d_dx : nullptr, grad ? d_dw : nullptr, grad ? d_dt : nullptr, s);
    if (rc) return rc;
    std::vector<double> os(n_poses), of(static_cast<size_t>(n_poses) * kNumF), odw(kNumW), odt(kTabN);
    std::vector<float> odx(grad ? nx : 0);
    queue_copy(ctx, &rc, os.data(), d_s, os.size() * 8, cudaMemcpyDeviceToHost, s);
    queue_copy(ctx, &rc, of.data(), d_f, of.size() * 8, cudaMemcpyDeviceToHost, s);
    if (grad) {
        queue_copy(ctx, &rc, odx.data(), d_dx, nx * 4, cudaMemcpyDeviceToHost, s);
        queue_copy(ctx, &rc, odw.data(), d_dw, kNumW * 8, cudaMemcpyDeviceToHost, s);
        queue_copy(ctx, &rc, odt.data(), d_dt, kTabN * 8, cudaMemcpyDeviceToHost, s);
    }
    rc = sync_copies(ctx, rc, s, "score adjoint");
    if (rc) return rc;
    if (score) std::copy(os.begin(), os.end(), score);
    if (features) std::copy(of.begin(), of.end(), features);
    if (dxyz)
        for (size_t i = 0; i < nx; ++i) dxyz[i] = odx[i];
    if (dweights)
        for (int k = 0; k < kNumW; ++k) dweights[k] += odw[k];
    if (dtables)
        for (int k = 0; k < kTabN; ++k) dtables[k] += odt[k];
    return PXD_OK;
}

int pxd_ligand_pose_dev(pxd_context* ctx, int32_t lig, int32_t n_poses, const float* xyz_in, const float* centers,
                        const float* quats, const float* torsions, float* xyz_out, void* stream) {
    if (!ctx) return PXD_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size()) || n_poses < 0 || !quats)
        return set_error(ctx, PXD_ERR_INVALID, "ligand id");
    if (ctx->ligands[lig].dev.n_frags == 0) return set_error(ctx, PXD_ERR_STATE, "ligand has no torsion tree");
    if (n_poses == 0) return PXD_OK;
    return launch_ligand_pose(ctx, lig, n_poses, xyz_in, centers, quats, torsions, xyz_out,
                              stream ? static_cast<cudaStream_t>(stream) : ctx->stream);
}

int pxd_ligand_pose_backward_dev(pxd_context* ctx, int32_t lig, int32_t n_poses, const float* xyz,
                                 const float* centers, const float* quats, const float* atom_grad, float* center_grad,
                                 float* quat_grad, float* torsion_grad, void* stream) {
    if (!ctx) return PXD_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (lig < 0 || lig >= static_cast<int>(ctx->ligands.size()) || n_poses < 0 || !quats || !quat_grad ||
        !center_grad || !torsion_grad)
        return set_error(ctx, PXD_ERR_INVALID, "ligand id or output");
    if (ctx->ligands[lig].dev.n_frags == 0) return set_error(ctx, PXD_ERR_STATE, "ligand has no torsion tree");
    if (n_poses == 0) return PXD_OK;
    return launch_ligand_pose_backward(ctx, lig, n_poses, xyz, centers, quats, atom_grad, center_grad, quat_grad,
                                       torsion_grad, stream ? static_cast<cudaStream_t>(stream) : ctx->stream);
}

}  // extern "C"
