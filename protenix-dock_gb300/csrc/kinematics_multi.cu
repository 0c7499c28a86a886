// Pose kinematics batched over poses of many receptor contexts, each pose with its own
// ligand (gradient pipelines over many complexes in one launch):
//
//   pose_multi_kernel           torsion-tree forward kinematics from (centre, quaternion,
//                               torsions), one warp per pose;
//   pose_backward_multi_kernel  its backward: atom gradients to centre, quaternion (through
//                               the normalisation) and torsion gradients.
#include <algorithm>
#include <vector>

#include "device_kin.cuh"

namespace pxd {

constexpr int kPoseWarps = 4;
constexpr int kMaxPoseDof = 39;  // 3 + 4 + up to 32 torsions

struct PoseMultiArgs {
    const DevLigand* const* tabs;  // [n_ctx] each context's device ligand table
    const int* ctx_ids;            // [P]
    const int* lig_ids;            // [P]
    int n_poses, max_atoms, dof;   // dof = row stride of the DOF arrays (3 + 4 + max torsions)
    const float* xyz_ref;          // [P][max_atoms][3] reference pose (atom order)
    const float* dofs;             // [P][dof]: centre, quaternion (w, x, y, z), torsions
    float* out;                    // [P][max_atoms][3]
    // backward
    const float* grad;             // [P][max_atoms][3] dE/dx at out
    float* dofs_grad;              // [P][dof]
};

__device__ __forceinline__ Mat3 unit_quat_rotation(const float* q4) {
    const float inv = rsqrtf(q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
    const float a = q4[0] * inv, b = q4[1] * inv, c = q4[2] * inv, d = q4[3] * inv;
    Mat3 m;  // get_rotation_matrix (math.cpp:22-42)
    m.r0 = make_float3(a * a + b * b - c * c - d * d, 2.f * (b * c - a * d), 2.f * (a * c + b * d));
    m.r1 = make_float3(2.f * (a * d + b * c), a * a - b * b + c * c - d * d, 2.f * (c * d - a * b));
    m.r2 = make_float3(2.f * (b * d - a * c), 2.f * (a * b + c * d), a * a - b * b - c * c + d * d);
    return m;
}

__global__ void __launch_bounds__(kPoseWarps * kWarp) pose_multi_kernel(const __grid_constant__ PoseMultiArgs a) {
    extern __shared__ __align__(16) float umem[];
    const int lane = threadIdx.x & (kWarp - 1);
    const int w = threadIdx.x / kWarp;
    const int per_warp = 4 * a.max_atoms + static_cast<int>(sizeof(KinShared) / sizeof(float));
    float4* c = reinterpret_cast<float4*>(umem + w * per_warp);
    KinShared& ks = *reinterpret_cast<KinShared*>(c + a.max_atoms);
    for (int pose = blockIdx.x * kPoseWarps + w; pose < a.n_poses; pose += gridDim.x * kPoseWarps) {
        const DevLigand& L = a.tabs[a.ctx_ids[pose]][a.lig_ids[pose]];
        const int N = L.n_atoms;
        const float* xr = a.xyz_ref + static_cast<size_t>(pose) * a.max_atoms * 3;
        for (int p = lane; p < N; p += kWarp) {
            const int atom = __ldg(&L.perm[p]);
            c[p] = make_float4(xr[3 * atom], xr[3 * atom + 1], xr[3 * atom + 2], 0.f);
        }
        __syncwarp();
        const float* q = a.dofs + static_cast<size_t>(pose) * a.dof;
        ligand_forward(L, c, L.frag_of, L.frag_mine, L.frag_parent, make_float3(q[0], q[1], q[2]),
                       unit_quat_rotation(q + 3), q + 7, ks, lane);
        float* o = a.out + static_cast<size_t>(pose) * a.max_atoms * 3;
        for (int p = lane; p < N; p += kWarp) {
            const int atom = __ldg(&L.perm[p]);
            o[3 * atom] = c[p].x;
            o[3 * atom + 1] = c[p].y;
            o[3 * atom + 2] = c[p].z;
        }
        for (int e = 3 * N + lane; e < 3 * a.max_atoms; e += kWarp) o[e] = 0.f;
        __syncwarp();
    }
}

// dE/dcentre = sum_i g_i; torque t = sum_i (x_i - centre) x g_i, mapped to the quaternion
// (a perturbation dq of the unit quaternion (w, v) turns the pose by 2 (w dv - dw v + v x dv),
// so dE/dw = -2 t.v, dE/dv = 2 (w t + t x v), then projected for the normalisation);
// dE/dtheta_k = u_k . sum over the torsion's subtree of (x_i - x_bond) x g_i.
__global__ void __launch_bounds__(kPoseWarps * kWarp)
    pose_backward_multi_kernel(const __grid_constant__ PoseMultiArgs a) {
    __shared__ float3 s_f[kPoseWarps][kMaxFrags];
    __shared__ float3 s_t[kPoseWarps][kMaxFrags];
    const int lane = threadIdx.x & (kWarp - 1);
    const int w = threadIdx.x / kWarp;
    for (int pose = blockIdx.x * kPoseWarps + w; pose < a.n_poses; pose += gridDim.x * kPoseWarps) {
        const DevLigand& L = a.tabs[a.ctx_ids[pose]][a.lig_ids[pose]];
        const int N = L.n_atoms;
        const float* x = a.out + static_cast<size_t>(pose) * a.max_atoms * 3;
        const float* g = a.grad + static_cast<size_t>(pose) * a.max_atoms * 3;
        const float* q = a.dofs + static_cast<size_t>(pose) * a.dof;
        const float3 c = make_float3(q[0], q[1], q[2]);
        for (int f = lane; f < L.n_frags; f += kWarp) {
            s_f[w][f] = make_float3(0.f, 0.f, 0.f);
            s_t[w][f] = make_float3(0.f, 0.f, 0.f);
        }
        __syncwarp();
        float3 ftot = make_float3(0.f, 0.f, 0.f), ttot = ftot;
        for (int p = lane; p < N; p += kWarp) {
            const int atom = __ldg(&L.perm[p]);
            const float3 xi = make_float3(x[3 * atom], x[3 * atom + 1], x[3 * atom + 2]);
            const float3 gi = make_float3(g[3 * atom], g[3 * atom + 1], g[3 * atom + 2]);
            const float3 ti = cross3(sub3(xi, c), gi);
            const int f = __ldg(&L.frag_of[p]);
            atomicAdd(&s_f[w][f].x, gi.x);
            atomicAdd(&s_f[w][f].y, gi.y);
            atomicAdd(&s_f[w][f].z, gi.z);
            atomicAdd(&s_t[w][f].x, ti.x);
            atomicAdd(&s_t[w][f].y, ti.y);
            atomicAdd(&s_t[w][f].z, ti.z);
            ftot = add3(ftot, gi);
            ttot = add3(ttot, ti);
        }
        ftot = make_float3(warp_sum_f(ftot.x), warp_sum_f(ftot.y), warp_sum_f(ftot.z));
        ttot = make_float3(warp_sum_f(ttot.x), warp_sum_f(ttot.y), warp_sum_f(ttot.z));
        __syncwarp();
        if (lane == 0) {
            float* og = a.dofs_grad + static_cast<size_t>(pose) * a.dof;
            for (int k = 7 + L.n_tors; k < a.dof; ++k) og[k] = 0.f;
            for (int k = L.n_tors - 1; k >= 0; --k) {
                const int4 tq = __ldg(&L.tors[k]);  // fragment, parent fragment, parent atom, bond atom
                const int ap = __ldg(&L.perm[tq.z]), am = __ldg(&L.perm[tq.w]);
                const float3 xp = make_float3(x[3 * ap], x[3 * ap + 1], x[3 * ap + 2]);
                const float3 xm = make_float3(x[3 * am], x[3 * am + 1], x[3 * am + 2]);
                float3 u = sub3(xm, xp);
                u = mul3(u, rsqrtf(dot3(u, u)));
                const float3 sf = s_f[w][tq.x], st = s_t[w][tq.x];
                og[7 + k] = dot3(u, sub3(st, cross3(sub3(xm, c), sf)));
                s_f[w][tq.y] = add3(s_f[w][tq.y], sf);
                s_t[w][tq.y] = add3(s_t[w][tq.y], st);
            }
            og[0] = ftot.x;
            og[1] = ftot.y;
            og[2] = ftot.z;
            const float len = sqrtf(q[3] * q[3] + q[4] * q[4] + q[5] * q[5] + q[6] * q[6]);
            const float qw = q[3] / len;
            const float3 v = make_float3(q[4] / len, q[5] / len, q[6] / len);
            const float gw = -2.f * dot3(ttot, v);
            const float3 gv = mul3(add3(mul3(ttot, qw), cross3(ttot, v)), 2.f);
            const float radial = gw * qw + dot3(gv, v);
            og[3] = (gw - radial * qw) / len;
            og[4] = (gv.x - radial * v.x) / len;
            og[5] = (gv.y - radial * v.y) / len;
            og[6] = (gv.z - radial * v.z) / len;
        }
        __syncwarp();
    }
}

static int ligand_tables(pxd_context* const* ctxs, int n_ctx, const DevLigand*** dev, cudaStream_t s) {
    pxd_context* ctx = ctxs[0];
    std::vector<const DevLigand*> tabs(n_ctx);
    for (int c = 0; c < n_ctx; ++c) {
        if (!ctxs[c] || ctxs[c]->device != ctx->device)
            return set_error(ctx, PXD_ERR_INVALID, "contexts must be non-null and on one device");
        int rc = sync_ligand_table(ctxs[c]);
        if (rc) return set_error(ctx, rc, ctxs[c]->error);
        tabs[c] = ctxs[c]->d_ligands;
    }
    int rc = cuda_check(ctx, cudaMallocAsync(reinterpret_cast<void**>(dev), sizeof(void*) * n_ctx, s), "ligand tables");
    if (rc) return rc;
    return cuda_check(ctx, cudaMemcpyAsync(*dev, tabs.data(), sizeof(void*) * n_ctx, cudaMemcpyHostToDevice, s),
                      "ligand tables copy");
}

}  // namespace pxd

using namespace pxd;

extern "C" {

int pxd_ligand_pose_multi_dev(pxd_context* const* ctxs, int32_t n_ctx, int32_t n_poses, int32_t max_atoms,
                              int32_t dof, const int32_t* ctx_ids, const int32_t* lig_ids, const float* xyz_ref,
                              const float* dofs, float* xyz_out, const float* atom_grad, float* dofs_grad,
                              void* stream) {
    if (!ctxs || n_ctx < 1 || !ctxs[0]) return PXD_ERR_INVALID;
    pxd_context* ctx = ctxs[0];
    if (n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS || dof < 7 || dof > kMaxPoseDof ||
        !ctx_ids || !lig_ids || !dofs || !xyz_out || (atom_grad && !dofs_grad) || (!atom_grad && !xyz_ref))
        return set_error(ctx, PXD_ERR_INVALID, "bad pose batch");
    for (int c = 0; c < n_ctx; ++c)
        for (const LigandEntry& e : ctxs[c]->ligands)
            if (e.dev.n_frags > kMaxFrags || e.dev.n_tors > kWarp || 7 + e.dev.n_tors > dof || e.n_atoms > max_atoms)
                return set_error(ctx, PXD_ERR_INVALID, "a ligand exceeds the pose batch's limits");
    cudaSetDevice(ctx->device);
    if (n_poses == 0) return PXD_OK;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const DevLigand** tabs = nullptr;
    int rc = ligand_tables(ctxs, n_ctx, &tabs, s);
    if (rc) return rc;
    PoseMultiArgs a{tabs, ctx_ids, lig_ids, n_poses, max_atoms, dof, xyz_ref, dofs, xyz_out, atom_grad, dofs_grad};
    int blocks = (n_poses + kPoseWarps - 1) / kPoseWarps;
    if (blocks > ctx->n_sm * 16) blocks = ctx->n_sm * 16;
    if (atom_grad) {
        pose_backward_multi_kernel<<<blocks, kPoseWarps * kWarp, 0, s>>>(a);
    } else {
        const size_t smem = sizeof(float) * kPoseWarps * (4 * max_atoms + sizeof(KinShared) / sizeof(float));
        rc = cuda_check(ctx, cudaFuncSetAttribute(pose_multi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  static_cast<int>(smem)), "pose smem");
        if (!rc) pose_multi_kernel<<<blocks, kPoseWarps * kWarp, smem, s>>>(a);
    }
    if (!rc) rc = cuda_check(ctx, cudaGetLastError(), "pose kinematics launch");
    cudaFreeAsync(tabs, s);
    return rc;
}

}  // extern "C"
