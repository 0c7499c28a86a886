// Pose kinematics batched over poses of many receptor contexts, each pose with its own
// ligand (gradient pipelines over many complexes in one launch):
//
//   pose_multi_kernel           torsion-tree forward kinematics from (centre, quaternion,
//                               torsions), one warp per pose;
//   pose_backward_multi_kernel  its backward: atom gradients to centre, quaternion (through
//                               the normalisation) and torsion gradients.
#include <algorithm>
#include <vector>

#include "device_dual.cuh"
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
    // directional derivatives (forward-mode)
    const float* dofs_dir;         // [P][dof] direction u of the DOFs
    const float* xyz_dir;          // [P][max_atoms][3] dx along u
    const float* grad_dir;         // [P][max_atoms][3] d(dE/dx) along u
    float* out_dir;                // [P][max_atoms][3] (JVP) or [P][dof] (backward's derivative)
};

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
        if (N > a.max_atoms || 7 + L.n_tors > a.dof) {  // the row cannot hold this ligand
            for (int e = lane; e < 3 * a.max_atoms; e += kWarp) a.out[static_cast<size_t>(pose) * a.max_atoms * 3 + e] = nanf("");
            continue;
        }
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
// S = Dual: x, g and the DOFs carry their derivatives along a DOF direction, and the
// kernel writes the derivative of dE/dq along it (with g's own derivative, H_x x_dir,
// this is the DOF-space Hessian-vector product).
__device__ __forceinline__ void atomic_add3(float3* p, float3 v) {
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
    atomicAdd(&p->z, v.z);
}
__device__ __forceinline__ void atomic_add3(D3* p, D3 v) {
    atomicAdd(&p->x.v, v.x.v);
    atomicAdd(&p->x.t, v.x.t);
    atomicAdd(&p->y.v, v.y.v);
    atomicAdd(&p->y.t, v.y.t);
    atomicAdd(&p->z.v, v.z.v);
    atomicAdd(&p->z.t, v.z.t);
}

template <class S>
__device__ __forceinline__ typename Vec<S>::type load3(const float* v, const float* t, size_t i);
template <>
__device__ __forceinline__ float3 load3<float>(const float* v, const float*, size_t i) {
    return make_float3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
}
template <>
__device__ __forceinline__ D3 load3<Dual>(const float* v, const float* t, size_t i) {
    return {Dual{v[3 * i], t[3 * i]}, Dual{v[3 * i + 1], t[3 * i + 1]}, Dual{v[3 * i + 2], t[3 * i + 2]}};
}
template <class S>
__device__ __forceinline__ S load1(const float* v, const float* t, size_t i);
template <>
__device__ __forceinline__ float load1<float>(const float* v, const float*, size_t i) { return v[i]; }
template <>
__device__ __forceinline__ Dual load1<Dual>(const float* v, const float* t, size_t i) { return Dual{v[i], t[i]}; }

template <class S>
__device__ __forceinline__ S warp_sum_s(S v);
template <>
__device__ __forceinline__ float warp_sum_s<float>(float v) { return warp_sum_f(v); }
template <>
__device__ __forceinline__ Dual warp_sum_s<Dual>(Dual v) { return Dual{warp_sum_f(v.v), warp_sum_f(v.t)}; }

template <class S>
__global__ void __launch_bounds__(kPoseWarps * kWarp)
    pose_backward_multi_kernel(const __grid_constant__ PoseMultiArgs a) {
    using V = typename Vec<S>::type;
    __shared__ V s_f[kPoseWarps][kMaxFrags];
    __shared__ V s_t[kPoseWarps][kMaxFrags];
    const int lane = threadIdx.x & (kWarp - 1);
    const int w = threadIdx.x / kWarp;
    for (int pose = blockIdx.x * kPoseWarps + w; pose < a.n_poses; pose += gridDim.x * kPoseWarps) {
        const DevLigand& L = a.tabs[a.ctx_ids[pose]][a.lig_ids[pose]];
        const int N = L.n_atoms;
        const size_t xo = static_cast<size_t>(pose) * a.max_atoms * 3, qo = static_cast<size_t>(pose) * a.dof;
        if (N > a.max_atoms || 7 + L.n_tors > a.dof) {
            float* og = (IsDual<S>::value ? a.out_dir : a.dofs_grad) + qo;
            for (int k = lane; k < a.dof; k += kWarp) og[k] = nanf("");
            continue;
        }
        const float* x = a.out + xo;
        const float* xt = a.xyz_dir ? a.xyz_dir + xo : nullptr;
        const float* g = a.grad + xo;
        const float* gt = a.grad_dir ? a.grad_dir + xo : nullptr;
        const float* q = a.dofs + qo;
        const float* qt = a.dofs_dir ? a.dofs_dir + qo : nullptr;
        const V c = {load1<S>(q, qt, 0), load1<S>(q, qt, 1), load1<S>(q, qt, 2)};
        for (int f = lane; f < L.n_frags; f += kWarp) {
            s_f[w][f] = zero3<S>();
            s_t[w][f] = zero3<S>();
        }
        __syncwarp();
        V ftot = zero3<S>(), ttot = zero3<S>();
        for (int p = lane; p < N; p += kWarp) {
            const int atom = __ldg(&L.perm[p]);
            const V xi = load3<S>(x, xt, atom), gi = load3<S>(g, gt, atom);
            const V ti = cross3(sub3(xi, c), gi);
            const int f = __ldg(&L.frag_of[p]);
            atomic_add3(&s_f[w][f], gi);
            atomic_add3(&s_t[w][f], ti);
            ftot = add3(ftot, gi);
            ttot = add3(ttot, ti);
        }
        ftot = {warp_sum_s(ftot.x), warp_sum_s(ftot.y), warp_sum_s(ftot.z)};
        ttot = {warp_sum_s(ttot.x), warp_sum_s(ttot.y), warp_sum_s(ttot.z)};
        __syncwarp();
        if (lane == 0) {
            float* og = (IsDual<S>::value ? a.out_dir : a.dofs_grad) + qo;
            for (int k = 7 + L.n_tors; k < a.dof; ++k) og[k] = 0.f;
            for (int k = L.n_tors - 1; k >= 0; --k) {
                const int4 tq = __ldg(&L.tors[k]);  // fragment, parent fragment, parent atom, bond atom
                const int ap = __ldg(&L.perm[tq.z]), am = __ldg(&L.perm[tq.w]);
                const V xp = load3<S>(x, xt, ap), xm = load3<S>(x, xt, am);
                V u = sub3(xm, xp);
                u = mul3(u, rsqrt_(dot3(u, u)));
                const V sf = s_f[w][tq.x], st = s_t[w][tq.x];
                og[7 + k] = part(dot3(u, sub3(st, cross3(sub3(xm, c), sf))));
                s_f[w][tq.y] = add3(s_f[w][tq.y], sf);
                s_t[w][tq.y] = add3(s_t[w][tq.y], st);
            }
            og[0] = part(ftot.x);
            og[1] = part(ftot.y);
            og[2] = part(ftot.z);
            const S q0 = load1<S>(q, qt, 3), q1 = load1<S>(q, qt, 4), q2 = load1<S>(q, qt, 5), q3 = load1<S>(q, qt, 6);
            const S len = sqrt_(q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3);
            const S qw = q0 / len;
            const V v = {q1 / len, q2 / len, q3 / len};
            const S gw = -2.f * dot3(ttot, v);
            const V gv = mul3(add3(mul3(ttot, qw), cross3(ttot, v)), 2.f);
            const S radial = gw * qw + dot3(gv, v);
            og[3] = part((gw - radial * qw) / len);
            og[4] = part((gv.x - radial * v.x) / len);
            og[5] = part((gv.y - radial * v.y) / len);
            og[6] = part((gv.z - radial * v.z) / len);
        }
        __syncwarp();
    }
}

// Forward-mode kinematics: dx along a DOF direction u at the poses x:
//   dx_i = dc + omega x (x_i - c) + sum over the torsions above atom i of
//          dtheta_k u_k x (x_i - x_bond,k),
// omega = 2 (w dv - dw v + v x dv) for the normalised quaternion (w, v) and its derivative.
__global__ void __launch_bounds__(kPoseWarps * kWarp) pose_jvp_multi_kernel(const __grid_constant__ PoseMultiArgs a) {
    __shared__ float3 s_ax[kPoseWarps][kMaxFrags];  // dtheta_k * unit axis of the fragment's torsion
    __shared__ float3 s_xm[kPoseWarps][kMaxFrags];  // the torsion's bond atom
    const int lane = threadIdx.x & (kWarp - 1);
    const int w = threadIdx.x / kWarp;
    for (int pose = blockIdx.x * kPoseWarps + w; pose < a.n_poses; pose += gridDim.x * kPoseWarps) {
        const DevLigand& L = a.tabs[a.ctx_ids[pose]][a.lig_ids[pose]];
        const int N = L.n_atoms;
        const size_t xo = static_cast<size_t>(pose) * a.max_atoms * 3, qo = static_cast<size_t>(pose) * a.dof;
        if (N > a.max_atoms || 7 + L.n_tors > a.dof) {
            for (int e = lane; e < 3 * a.max_atoms; e += kWarp) a.out_dir[xo + e] = nanf("");
            continue;
        }
        const float* x = a.out + xo;
        const float* q = a.dofs + qo;
        const float* u = a.dofs_dir + qo;
        for (int f = lane; f < L.n_frags; f += kWarp) {
            s_ax[w][f] = make_float3(0.f, 0.f, 0.f);
            s_xm[w][f] = make_float3(0.f, 0.f, 0.f);
        }
        __syncwarp();
        if (lane < L.n_tors) {
            const int4 tq = __ldg(&L.tors[lane]);
            const int ap = __ldg(&L.perm[tq.z]), am = __ldg(&L.perm[tq.w]);
            const float3 xp = make_float3(x[3 * ap], x[3 * ap + 1], x[3 * ap + 2]);
            const float3 xm = make_float3(x[3 * am], x[3 * am + 1], x[3 * am + 2]);
            float3 ax = sub3(xm, xp);
            ax = mul3(ax, rsqrtf(dot3(ax, ax)) * u[7 + lane]);
            s_ax[w][tq.x] = ax;
            s_xm[w][tq.x] = xm;
        }
        __syncwarp();
        const float3 c = make_float3(q[0], q[1], q[2]);
        const float3 dc = make_float3(u[0], u[1], u[2]);
        const float len = sqrtf(q[3] * q[3] + q[4] * q[4] + q[5] * q[5] + q[6] * q[6]);
        const float qw = q[3] / len;
        const float3 qv = make_float3(q[4] / len, q[5] / len, q[6] / len);
        const float radial = (u[3] * qw + u[4] * qv.x + u[5] * qv.y + u[6] * qv.z);
        const float dw = (u[3] - radial * qw) / len;
        const float3 dv = make_float3((u[4] - radial * qv.x) / len, (u[5] - radial * qv.y) / len,
                                      (u[6] - radial * qv.z) / len);
        const float3 om = mul3(add3(sub3(mul3(dv, qw), mul3(qv, dw)), cross3(qv, dv)), 2.f);
        float* o = a.out_dir + xo;
        for (int p = lane; p < N; p += kWarp) {
            const int atom = __ldg(&L.perm[p]);
            const float3 xi = make_float3(x[3 * atom], x[3 * atom + 1], x[3 * atom + 2]);
            float3 d = add3(dc, cross3(om, sub3(xi, c)));
            for (int f = __ldg(&L.frag_of[p]); f >= 0 && __ldg(&L.frag_mine[f]) >= 0; f = __ldg(&L.frag_parent[f]))
                d = add3(d, cross3(s_ax[w][f], sub3(xi, s_xm[w][f])));
            o[3 * atom] = d.x;
            o[3 * atom + 1] = d.y;
            o[3 * atom + 2] = d.z;
        }
        for (int e = 3 * N + lane; e < 3 * a.max_atoms; e += kWarp) o[e] = 0.f;
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
            if (e.dev.n_frags > kMaxFrags || e.dev.n_tors > kWarp)
                return set_error(ctx, PXD_ERR_INVALID, "a ligand exceeds the kinematics limits (64 fragments, 32 torsions)");
    cudaSetDevice(ctx->device);
    if (n_poses == 0) return PXD_OK;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const DevLigand** tabs = nullptr;
    int rc = ligand_tables(ctxs, n_ctx, &tabs, s);
    if (rc) return rc;
    PoseMultiArgs a{tabs, ctx_ids, lig_ids, n_poses, max_atoms, dof, xyz_ref, dofs, xyz_out, atom_grad, dofs_grad,
                    nullptr, nullptr, nullptr, nullptr};
    int blocks = (n_poses + kPoseWarps - 1) / kPoseWarps;
    if (blocks > ctx->n_sm * 16) blocks = ctx->n_sm * 16;
    if (atom_grad) {
        pose_backward_multi_kernel<float><<<blocks, kPoseWarps * kWarp, 0, s>>>(a);
    } else {
        const size_t smem = sizeof(float) * kPoseWarps * (4 * max_atoms + sizeof(KinShared) / sizeof(float));
        rc = raise_smem_limit(ctx, reinterpret_cast<const void*>(pose_multi_kernel), smem, "pose smem");
        if (!rc) pose_multi_kernel<<<blocks, kPoseWarps * kWarp, smem, s>>>(a);
    }
    if (!rc) rc = cuda_check(ctx, cudaGetLastError(), "pose kinematics launch");
    cudaFreeAsync(tabs, s);
    return rc;
}

int pxd_ligand_pose_dir_multi_dev(pxd_context* const* ctxs, int32_t n_ctx, int32_t n_poses, int32_t max_atoms,
                                  int32_t dof, const int32_t* ctx_ids, const int32_t* lig_ids, const float* xyz,
                                  const float* dofs, const float* dofs_dir, const float* xyz_dir,
                                  const float* atom_grad, const float* atom_grad_dir, float* out_dir, void* stream) {
    if (!ctxs || n_ctx < 1 || !ctxs[0]) return PXD_ERR_INVALID;
    pxd_context* ctx = ctxs[0];
    const bool back = atom_grad != nullptr;
    if (n_poses < 0 || max_atoms <= 0 || max_atoms > PXD_MAX_LIGAND_ATOMS || dof < 7 || dof > kMaxPoseDof ||
        !ctx_ids || !lig_ids || !xyz || !dofs || !dofs_dir || !out_dir || (back && (!xyz_dir || !atom_grad_dir)))
        return set_error(ctx, PXD_ERR_INVALID, "bad pose batch");
    for (int c = 0; c < n_ctx; ++c)
        for (const LigandEntry& e : ctxs[c]->ligands)
            if (e.dev.n_frags > kMaxFrags || e.dev.n_tors > kWarp)
                return set_error(ctx, PXD_ERR_INVALID, "a ligand exceeds the kinematics limits (64 fragments, 32 torsions)");
    cudaSetDevice(ctx->device);
    if (n_poses == 0) return PXD_OK;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const DevLigand** tabs = nullptr;
    int rc = ligand_tables(ctxs, n_ctx, &tabs, s);
    if (rc) return rc;
    PoseMultiArgs a{tabs, ctx_ids, lig_ids, n_poses, max_atoms, dof, nullptr, dofs, const_cast<float*>(xyz),
                    atom_grad, nullptr, dofs_dir, xyz_dir, atom_grad_dir, out_dir};
    int blocks = (n_poses + kPoseWarps - 1) / kPoseWarps;
    if (blocks > ctx->n_sm * 16) blocks = ctx->n_sm * 16;
    if (back) pose_backward_multi_kernel<Dual><<<blocks, kPoseWarps * kWarp, 0, s>>>(a);
    else pose_jvp_multi_kernel<<<blocks, kPoseWarps * kWarp, 0, s>>>(a);
    rc = cuda_check(ctx, cudaGetLastError(), "pose direction launch");
    cudaFreeAsync(tabs, s);
    return rc;
}

}  // extern "C"
