// Pose clustering on the GPU: pose_cluster::preprocess (writer.cpp:99-177) for many ligands
// at once, one warp per ligand.
//
// The rule is sequential within a ligand: walk the candidates in order, skip failed walkers
// (nevals == 0), and keep a candidate as a new mode, in place of its closest mode (RMSD
// below min_rmsd and a better pose score), or in place of the worst mode (when num_modes
// are kept already and it scores better); the kept list stays sorted by pose score. Across
// ligands it is independent, so a search's ligands run side by side. Lane k holds the k-th
// best kept pose: the RMSDs of a candidate to all kept poses are formed at once (each
// lane summing over atoms in the reference's order, with non-contracted FP64 operations so
// that every comparison is the host rule's), the closest is a warp arg-min that keeps the
// first of equal minima (find_closest_pose takes a later one only when strictly closer),
// and a changed list is re-sorted by a compare-exchange pass across lanes.
#include <cfloat>

#include "pxd_internal.h"

namespace pxd {

namespace {

constexpr int kClusterWarps = 4;

struct ClusterArgs {
    const float* xyz;      // [poses][stride][3]
    const double* pscore;  // [poses]
    const int* nevals;     // [poses]
    const int* start;      // [n_groups + 1]: the candidates of group g are start[g] .. start[g + 1] - 1
    const int* n_atoms;    // [n_groups]
    int stride, n_groups, num_modes;
    double min_rmsd;
    int* kept;             // [n_groups][num_modes], best first, -1 past n_kept
    int* n_kept;           // [n_groups]
};

// calculate_rmsd_upper_bound (writer.cpp:99-106): sqrt(sum_i |a_i - b_i|^2 / n), the sum
// taken atom by atom as ((dx dx + dy dy) + dz dz) without fused multiply-adds.
__device__ double pose_rmsd(const float* a, const float* b, int n) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) {
        const double dx = __dsub_rn(a[3 * i], b[3 * i]);
        const double dy = __dsub_rn(a[3 * i + 1], b[3 * i + 1]);
        const double dz = __dsub_rn(a[3 * i + 2], b[3 * i + 2]);
        s = __dadd_rn(s, __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    }
    return sqrt(s / static_cast<double>(n));
}

__global__ void __launch_bounds__(kClusterWarps * 32) cluster_kernel(const ClusterArgs a) {
    const int lane = threadIdx.x & 31;
    const int g = blockIdx.x * kClusterWarps + threadIdx.x / 32;
    if (g >= a.n_groups) return;  // the whole warp
    const int n = a.n_atoms[g];
    const size_t stride = static_cast<size_t>(a.stride) * 3;
    int kk = -1;            // this lane's kept candidate (lane k: the k-th best)
    double ks = DBL_MAX;    // and its pose score
    int cnt = 0;
    for (int c = a.start[g]; c < a.start[g + 1]; ++c) {
        if (a.nevals[c] == 0) continue;  // failure mark from the searcher
        const double pc = a.pscore[c];
        if (cnt == 0) {
            if (lane == 0) {
                kk = c;
                ks = pc;
            }
            cnt = 1;
            continue;
        }
        double r = DBL_MAX;
        if (lane < cnt) r = pose_rmsd(a.xyz + static_cast<size_t>(kk) * stride, a.xyz + static_cast<size_t>(c) * stride, n);
        // arg-min over the kept lanes, the lowest lane among equal minima
        double best = r;
        int off = lane;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, d);
            const int oo = __shfl_xor_sync(0xffffffffu, off, d);
            if (ob < best || (ob == best && oo < off)) {
                best = ob;
                off = oo;
            }
        }
        bool updated = false;
        if (best < a.min_rmsd) {
            const double ko = __shfl_sync(0xffffffffu, ks, off);
            if (pc < ko) {
                if (lane == off) {
                    kk = c;
                    ks = pc;
                }
                updated = true;
            }
        } else if (cnt < a.num_modes) {
            if (lane == cnt) {
                kk = c;
                ks = pc;
            }
            ++cnt;
            updated = true;
        } else {
            const double kl = __shfl_sync(0xffffffffu, ks, cnt - 1);
            if (pc < kl) {
                if (lane == cnt - 1) {
                    kk = c;
                    ks = pc;
                }
                updated = true;
            }
        }
        if (updated) {
            // odd-even transposition sort of lanes 0 .. cnt-1 by pose score (cnt passes)
            for (int pass = 0; pass < cnt; ++pass) {
                const int partner = ((lane & 1) == (pass & 1)) ? lane + 1 : lane - 1;
                const double ps = __shfl_sync(0xffffffffu, ks, partner & 31);
                const int pk = __shfl_sync(0xffffffffu, kk, partner & 31);
                if (partner >= 0 && partner < cnt && lane < cnt) {
                    const bool lower = lane < partner;
                    if (lower ? ps < ks : ks < ps) {
                        ks = ps;
                        kk = pk;
                    }
                }
            }
        }
    }
    if (lane < a.num_modes) a.kept[static_cast<size_t>(g) * a.num_modes + lane] = lane < cnt ? kk : -1;
    if (lane == 0) a.n_kept[g] = cnt;
}

}  // namespace

int launch_cluster(pxd_context* ctx, int n_groups, const int* start, const int* n_atoms, int stride, const float* xyz,
                   const double* pscore, const int* nevals, int num_modes, double min_rmsd, int* kept, int* n_kept,
                   cudaStream_t s) {
    if (n_groups <= 0) return PXD_OK;
    ClusterArgs a{xyz, pscore, nevals, start, n_atoms, stride, n_groups, num_modes, min_rmsd, kept, n_kept};
    const int blocks = (n_groups + kClusterWarps - 1) / kClusterWarps;
    cluster_kernel<<<blocks, kClusterWarps * 32, 0, s>>>(a);
    return cuda_check(ctx, cudaGetLastError(), "cluster_kernel launch");
}

}  // namespace pxd

using namespace pxd;

extern "C" int pxd_cluster_poses_dev(pxd_context* ctx, int32_t n_groups, const int32_t* group_start,
                                     const int32_t* group_atoms, int32_t stride_atoms, const float* xyz,
                                     const double* pscore, const int32_t* nevals, int32_t num_modes, double min_rmsd,
                                     int32_t* kept, int32_t* n_kept, void* stream) {
    if (!ctx) return PXD_ERR_INVALID;
    if (n_groups < 0 || num_modes < 1 || num_modes > 32 || stride_atoms <= 0)
        return set_error(ctx, PXD_ERR_INVALID, "clustering: n_groups >= 0, 1 <= num_modes <= 32, stride > 0");
    if (n_groups > 0 && (!group_start || !group_atoms || !xyz || !pscore || !nevals || !kept || !n_kept))
        return set_error(ctx, PXD_ERR_INVALID, "clustering: null buffer");
    cudaSetDevice(ctx->device);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    return launch_cluster(ctx, n_groups, group_start, group_atoms, stride_atoms, xyz, pscore, nevals, num_modes,
                          min_rmsd, kept, n_kept, s);
}

extern "C" int pxd_cluster_poses_batch(pxd_context* ctx, int32_t n_groups, const int32_t* group_start,
                                       const int32_t* group_atoms, int32_t stride_atoms, const double* xyz,
                                       const double* pscore, const int32_t* nevals, int32_t num_modes,
                                       double min_rmsd, int32_t* kept, int32_t* n_kept) {
    if (!ctx) return PXD_ERR_INVALID;
    if (n_groups < 0 || num_modes < 1 || num_modes > 32 || stride_atoms <= 0)
        return set_error(ctx, PXD_ERR_INVALID, "clustering: n_groups >= 0, 1 <= num_modes <= 32, stride > 0");
    if (n_groups == 0) return PXD_OK;
    if (!group_start || !group_atoms || !xyz || !pscore || !nevals || !kept || !n_kept)
        return set_error(ctx, PXD_ERR_INVALID, "clustering: null buffer");
    cudaSetDevice(ctx->device);
    const int n_poses = group_start[n_groups];
    for (int g = 0; g < n_groups; ++g)
        if (group_start[g] < 0 || group_start[g] > group_start[g + 1] || group_atoms[g] <= 0 ||
            group_atoms[g] > stride_atoms)
            return set_error(ctx, PXD_ERR_INVALID, "clustering: bad group " + std::to_string(g));
    // coordinates narrowed to FP32 (search outputs are FP32 values, so exactly)
    std::vector<float> hx(static_cast<size_t>(n_poses) * stride_atoms * 3);
    for (size_t i = 0; i < hx.size(); ++i) hx[i] = static_cast<float>(xyz[i]);
    int rc;
    Staging st{ctx, {}};
    float* dx = st.alloc<float>(hx.size(), &rc);
    double* dp = rc ? nullptr : st.alloc<double>(n_poses, &rc);
    int* dn = rc ? nullptr : st.alloc<int>(n_poses, &rc);
    int* ds = rc ? nullptr : st.alloc<int>(n_groups + 1, &rc);
    int* da = rc ? nullptr : st.alloc<int>(n_groups, &rc);
    int* dk = rc ? nullptr : st.alloc<int>(static_cast<size_t>(n_groups) * num_modes, &rc);
    int* dc = rc ? nullptr : st.alloc<int>(n_groups, &rc);
    if (rc) return rc;
    queue_copy(ctx, &rc, dx, hx.data(), hx.size() * 4, cudaMemcpyHostToDevice, ctx->stream, "clustering poses");
    queue_copy(ctx, &rc, dp, pscore, 8 * static_cast<size_t>(n_poses), cudaMemcpyHostToDevice, ctx->stream,
               "clustering scores");
    queue_copy(ctx, &rc, dn, nevals, 4 * static_cast<size_t>(n_poses), cudaMemcpyHostToDevice, ctx->stream,
               "clustering evaluations");
    queue_copy(ctx, &rc, ds, group_start, 4 * static_cast<size_t>(n_groups + 1), cudaMemcpyHostToDevice, ctx->stream,
               "clustering groups");
    queue_copy(ctx, &rc, da, group_atoms, 4 * static_cast<size_t>(n_groups), cudaMemcpyHostToDevice, ctx->stream,
               "clustering atom counts");
    if (!rc)
        rc = launch_cluster(ctx, n_groups, ds, da, stride_atoms, dx, dp, dn, num_modes, min_rmsd, dk, dc, ctx->stream);
    queue_copy(ctx, &rc, kept, dk, 4 * static_cast<size_t>(n_groups) * num_modes, cudaMemcpyDeviceToHost,
               ctx->stream, "kept poses");
    queue_copy(ctx, &rc, n_kept, dc, 4 * static_cast<size_t>(n_groups), cudaMemcpyDeviceToHost, ctx->stream,
               "kept counts");
    return sync_copies(ctx, rc, ctx->stream, "clustering");
}
