// Forward kinematics on the GPU.
//
// Ligand torsion tree (free_ligand::apply_parameters, data.cpp:592-641), one warp per
// pose. The reference walks the tree recursively; every coordinate subtraction there
// reads input coordinates, so here the relative coordinates are formed for all atoms
// in parallel, lane 0 composes the fragment frames in torsion (pre-)order
//   fused_f = Rot(fused_parent * axis_f, theta_f) * fused_parent,  fused_root = R
//   origin_f = fused_parent * rel(mine_f) + origin_parent,         origin_root = centre
// and all atoms are placed in parallel: world_i = fused_frag(i) * rel_i + origin_frag(i).
//
// Receptor rotors (torsional_receptor::apply_parameters, data.cpp:366-385), one
// thread per (pose, atom).
#include "device_kin.cuh"

namespace pxd {

constexpr int kKinWarps = 4;
struct LigKinArgs {
    DevLigand L;
    int n_poses;
    const float* xyz_in;   // [N][3] reference pose (atom order)
    const float* centers;  // [P][3]
    const float* rots;     // [P][9] (when quats is NULL)
    const float* tors;     // [P][T]
    float* out;            // [P][N][3]
    const float* quats;    // [P][4] (w, x, y, z) or NULL
};

// Rotation of the normalised quaternion q (get_rotation_matrix, math.cpp:22-42).
__device__ __forceinline__ Mat3 quat_rotation(const float* q4) {
    const float inv = rsqrtf(q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
    const float a = q4[0] * inv, b = q4[1] * inv, c = q4[2] * inv, d = q4[3] * inv;
    Mat3 m;
    m.r0 = make_float3(a * a + b * b - c * c - d * d, 2.f * (b * c - a * d), 2.f * (a * c + b * d));
    m.r1 = make_float3(2.f * (a * d + b * c), a * a - b * b + c * c - d * d, 2.f * (c * d - a * b));
    m.r2 = make_float3(2.f * (b * d - a * c), 2.f * (a * b + c * d), a * a - b * b - c * c + d * d);
    return m;
}

__global__ void __launch_bounds__(kKinWarps * kWarp) ligand_kinematics_kernel(const LigKinArgs a) {
    __shared__ float4 s_c[kKinWarps][PXD_MAX_LIGAND_ATOMS];
    __shared__ int s_frag[PXD_MAX_LIGAND_ATOMS];
    __shared__ int s_mine[kMaxFrags], s_parent[kMaxFrags];
    __shared__ KinShared s_ks[kKinWarps];
    const DevLigand& L = a.L;
    const int N = L.n_atoms;
    for (int f = threadIdx.x; f < L.n_frags; f += blockDim.x) {
        s_mine[f] = -1;
        s_parent[f] = -1;
        for (int p = L.frag_range[2 * f]; p < L.frag_range[2 * f + 1]; ++p) s_frag[p] = f;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < L.n_tors; k += blockDim.x) {
        const int4 q = L.tors[k];
        s_mine[q.x] = q.w;
        s_parent[q.x] = q.y;
    }
    __syncthreads();
    const int lane = threadIdx.x & (kWarp - 1);
    const int w = threadIdx.x / kWarp;
    for (int pose = blockIdx.x * kKinWarps + w; pose < a.n_poses; pose += gridDim.x * kKinWarps) {
        float4* c = s_c[w];
        for (int p = lane; p < N; p += kWarp) {
            const int atom = __ldg(&L.perm[p]);
            c[p] = make_float4(a.xyz_in[3 * atom], a.xyz_in[3 * atom + 1], a.xyz_in[3 * atom + 2], 0.f);
        }
        __syncwarp();
        Mat3 rot;
        if (a.quats) {
            rot = quat_rotation(a.quats + 4 * static_cast<size_t>(pose));
        } else {
            const float* r = a.rots + 9 * static_cast<size_t>(pose);
            rot.r0 = make_float3(r[0], r[1], r[2]);
            rot.r1 = make_float3(r[3], r[4], r[5]);
            rot.r2 = make_float3(r[6], r[7], r[8]);
        }
        const float* cc = a.centers + 3 * static_cast<size_t>(pose);
        ligand_forward(L, c, s_frag, s_mine, s_parent, make_float3(cc[0], cc[1], cc[2]), rot,
                       a.tors + static_cast<size_t>(pose) * L.n_tors, s_ks[w], lane);
        float* o = a.out + static_cast<size_t>(pose) * N * 3;
        for (int p = lane; p < N; p += kWarp) {
            const int atom = __ldg(&L.perm[p]);
            o[3 * atom] = c[p].x;
            o[3 * atom + 1] = c[p].y;
            o[3 * atom + 2] = c[p].z;
        }
        __syncwarp();
    }
}

int launch_ligand_kinematics(pxd_context* ctx, int lig, int n_poses, const float* xyz_in,
                             const float* centers, const float* rots, const float* tors,
                             float* xyz_out, cudaStream_t s) {
    const DevLigand& L = ctx->ligands[lig].dev;
    if (L.n_frags > kMaxFrags) return set_error(ctx, PXD_ERR_INVALID, "too many fragments");
    if (L.n_tors > kWarp) return set_error(ctx, PXD_ERR_INVALID, "more than 32 torsions");
    LigKinArgs a{L, n_poses, xyz_in, centers, rots, tors, xyz_out, nullptr};
    int blocks = (n_poses + kKinWarps - 1) / kKinWarps;
    if (blocks > ctx->n_sm * 8) blocks = ctx->n_sm * 8;
    if (blocks < 1) blocks = 1;
    ligand_kinematics_kernel<<<blocks, kKinWarps * kWarp, 0, s>>>(a);
    return cuda_check(ctx, cudaGetLastError(), "ligand_kinematics_kernel launch");
}

int launch_ligand_pose(pxd_context* ctx, int lig, int n_poses, const float* xyz_in, const float* centers,
                       const float* quats, const float* tors, float* xyz_out, cudaStream_t s) {
    const DevLigand& L = ctx->ligands[lig].dev;
    if (L.n_frags > kMaxFrags) return set_error(ctx, PXD_ERR_INVALID, "too many fragments");
    if (L.n_tors > kWarp) return set_error(ctx, PXD_ERR_INVALID, "more than 32 torsions");
    LigKinArgs a{L, n_poses, xyz_in, centers, nullptr, tors, xyz_out, quats};
    int blocks = (n_poses + kKinWarps - 1) / kKinWarps;
    if (blocks > ctx->n_sm * 8) blocks = ctx->n_sm * 8;
    if (blocks < 1) blocks = 1;
    ligand_kinematics_kernel<<<blocks, kKinWarps * kWarp, 0, s>>>(a);
    return cuda_check(ctx, cudaGetLastError(), "ligand_kinematics_kernel launch");
}

struct RecKinArgs {
    int n_poses, n_atoms, n_rotors;
    const float4* xyz0;       // [M] input coordinates
    const int* atom_rotor;    // [M] rotor of a rotor atom, -1 otherwise
    const float4* origin;
    const float4* axis;
    const float* tors;        // [P][R]
    float* out;               // [P][M][3]
};

__global__ void receptor_kinematics_kernel(const RecKinArgs a) {
    const size_t idx = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<size_t>(a.n_poses) * a.n_atoms) return;
    const int pose = static_cast<int>(idx / a.n_atoms);
    const int atom = static_cast<int>(idx % a.n_atoms);
    float3 p = xyz(a.xyz0[atom]);
    const int r = a.atom_rotor[atom];
    if (r >= 0) {
        const float3 o = xyz(a.origin[r]);
        const Mat3 R = rodrigues(xyz(a.axis[r]), a.tors[static_cast<size_t>(pose) * a.n_rotors + r]);
        p = add3(mat_apply(R, sub3(p, o)), o);
    }
    float* out = a.out + idx * 3;
    out[0] = p.x;
    out[1] = p.y;
    out[2] = p.z;
}

int launch_receptor_kinematics(pxd_context* ctx, int n_poses, const float* tors, float* out,
                               cudaStream_t s) {
    const int M = ctx->n_rec;
    std::vector<float4> xyz0(M);
    std::vector<int> rotor(M, -1);
    for (int i = 0; i < M; ++i)
        xyz0[i] = make_float4(static_cast<float>(ctx->rec_xyz[3 * i]),
                              static_cast<float>(ctx->rec_xyz[3 * i + 1]),
                              static_cast<float>(ctx->rec_xyz[3 * i + 2]), 0.f);
    for (size_t k = 0; k < ctx->mov_atoms.size(); ++k) rotor[ctx->mov_atoms[k]] = ctx->mov_rotor[k];
    void* mem = nullptr;
    const size_t b0 = sizeof(float4) * M, b1 = sizeof(int) * M;
    int rc = cuda_check(ctx, cudaMallocAsync(&mem, b0 + b1, s), "receptor kinematics tables");
    if (rc) return rc;
    queue_copy(ctx, &rc, mem, xyz0.data(), b0, cudaMemcpyHostToDevice, s);
    queue_copy(ctx, &rc, static_cast<char*>(mem) + b0, rotor.data(), b1, cudaMemcpyHostToDevice, s);
    if (rc) {
        cudaFreeAsync(mem, s);
        return rc;
    }
    RecKinArgs a{n_poses, M, ctx->rec.n_rotors, static_cast<float4*>(mem),
                 reinterpret_cast<int*>(static_cast<char*>(mem) + b0), ctx->rec.rotor_origin,
                 ctx->rec.rotor_axis, tors, out};
    const size_t total = static_cast<size_t>(n_poses) * M;
    const int threads = 256;
    const unsigned blocks = static_cast<unsigned>((total + threads - 1) / threads);
    if (blocks > 0) receptor_kinematics_kernel<<<blocks, threads, 0, s>>>(a);
    rc = cuda_check(ctx, cudaGetLastError(), "receptor_kinematics_kernel launch");
    cudaFreeAsync(mem, s);
    return rc;
}

// Backward kinematics: gradients of a function of the ligand's atom coordinates with
// respect to the pose parameters of the forward map above, one warp per pose.
//   dE/dcentre = sum_i g_i,   dE/domega = sum_i (x_i - centre) x g_i  (a rotation applied
//   on the left of the root orientation), and for torsion k, which turns the subtree of
//   its fragment about the unit axis u_k (parent atom -> bond atom) through the bond atom:
//   dE/dtheta_k = u_k . sum_{i in subtree} (x_i - x_bond) x g_i.
// Torques are summed about the centre; subtree sums are folded in reverse pre-order.
struct LigBackArgs {
    DevLigand L;
    int n_poses;
    const float* xyz;      // [P][N][3] current coordinates (atom order)
    const float* centers;  // [P][3]
    const float* grad;     // [P][N][3] dE/dx
    float* out_center;     // [P][3]
    float* out_torque;     // [P][3]
    float* out_tors;       // [P][T]
    const float* quats;    // [P][4] orientation used by the forward map, or NULL
    float* out_quat;       // [P][4] dE/dq through the normalisation (with quats)
};

__global__ void __launch_bounds__(kKinWarps * kWarp) ligand_backward_kernel(const LigBackArgs a) {
    __shared__ float3 s_f[kKinWarps][kMaxFrags];
    __shared__ float3 s_t[kKinWarps][kMaxFrags];
    const DevLigand& L = a.L;
    const int N = L.n_atoms;
    const int lane = threadIdx.x & (kWarp - 1);
    const int w = threadIdx.x / kWarp;
    for (int pose = blockIdx.x * kKinWarps + w; pose < a.n_poses; pose += gridDim.x * kKinWarps) {
        const float* x = a.xyz + static_cast<size_t>(pose) * N * 3;
        const float* g = a.grad + static_cast<size_t>(pose) * N * 3;
        const float3 c = make_float3(a.centers[3 * pose], a.centers[3 * pose + 1], a.centers[3 * pose + 2]);
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
            float* ot = a.out_tors + static_cast<size_t>(pose) * L.n_tors;
            for (int k = L.n_tors - 1; k >= 0; --k) {
                const int4 q = __ldg(&L.tors[k]);  // fragment, parent fragment, parent atom, bond atom
                const int ap = __ldg(&L.perm[q.z]), am = __ldg(&L.perm[q.w]);
                const float3 xp = make_float3(x[3 * ap], x[3 * ap + 1], x[3 * ap + 2]);
                const float3 xm = make_float3(x[3 * am], x[3 * am + 1], x[3 * am + 2]);
                float3 u = sub3(xm, xp);
                u = mul3(u, rsqrtf(dot3(u, u)));
                const float3 sf = s_f[w][q.x], st = s_t[w][q.x];
                ot[k] = dot3(u, sub3(st, cross3(sub3(xm, c), sf)));
                s_f[w][q.y] = add3(s_f[w][q.y], sf);
                s_t[w][q.y] = add3(s_t[w][q.y], st);
            }
            float* oc = a.out_center + 3 * static_cast<size_t>(pose);
            oc[0] = ftot.x;
            oc[1] = ftot.y;
            oc[2] = ftot.z;
            if (a.out_torque) {
                float* oq = a.out_torque + 3 * static_cast<size_t>(pose);
                oq[0] = ttot.x;
                oq[1] = ttot.y;
                oq[2] = ttot.z;
            }
            if (a.out_quat) {
                // A perturbation dq of the unit quaternion (w, v) turns the pose by the
                // rotation vector 2 vec(dq q*) = 2 (w dv - dw v + v x dv), so with torque t
                // dE/dw = -2 t.v and dE/dv = 2 (w t + t x v); the normalisation projects
                // out the radial part and divides by |q|.
                const float* q4 = a.quats + 4 * static_cast<size_t>(pose);
                const float len = sqrtf(q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
                const float w = q4[0] / len;
                const float3 v = make_float3(q4[1] / len, q4[2] / len, q4[3] / len);
                const float gw = -2.f * dot3(ttot, v);
                const float3 gv = mul3(add3(mul3(ttot, w), cross3(ttot, v)), 2.f);
                const float radial = gw * w + dot3(gv, v);
                float* og = a.out_quat + 4 * static_cast<size_t>(pose);
                og[0] = (gw - radial * w) / len;
                og[1] = (gv.x - radial * v.x) / len;
                og[2] = (gv.y - radial * v.y) / len;
                og[3] = (gv.z - radial * v.z) / len;
            }
        }
        __syncwarp();
    }
}

int launch_ligand_backward(pxd_context* ctx, int lig, int n_poses, const float* xyz, const float* centers,
                           const float* grad, float* out_center, float* out_torque, float* out_tors,
                           cudaStream_t s) {
    const DevLigand& L = ctx->ligands[lig].dev;
    if (L.n_frags > kMaxFrags) return set_error(ctx, PXD_ERR_INVALID, "too many fragments");
    LigBackArgs a{L, n_poses, xyz, centers, grad, out_center, out_torque, out_tors, nullptr, nullptr};
    int blocks = (n_poses + kKinWarps - 1) / kKinWarps;
    if (blocks > ctx->n_sm * 8) blocks = ctx->n_sm * 8;
    if (blocks < 1) blocks = 1;
    ligand_backward_kernel<<<blocks, kKinWarps * kWarp, 0, s>>>(a);
    return cuda_check(ctx, cudaGetLastError(), "ligand_backward_kernel launch");
}

int launch_ligand_pose_backward(pxd_context* ctx, int lig, int n_poses, const float* xyz, const float* centers,
                                const float* quats, const float* grad, float* out_center, float* out_quat,
                                float* out_tors, cudaStream_t s) {
    const DevLigand& L = ctx->ligands[lig].dev;
    if (L.n_frags > kMaxFrags) return set_error(ctx, PXD_ERR_INVALID, "too many fragments");
    LigBackArgs a{L, n_poses, xyz, centers, grad, out_center, nullptr, out_tors, quats, out_quat};
    int blocks = (n_poses + kKinWarps - 1) / kKinWarps;
    if (blocks > ctx->n_sm * 8) blocks = ctx->n_sm * 8;
    if (blocks < 1) blocks = 1;
    ligand_backward_kernel<<<blocks, kKinWarps * kWarp, 0, s>>>(a);
    return cuda_check(ctx, cudaGetLastError(), "ligand_backward_kernel launch");
}

}  // namespace pxd
