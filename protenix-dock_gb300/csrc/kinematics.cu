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
#include "device_eval.cuh"

namespace pxd {

constexpr int kKinWarps = 4;
constexpr int kMaxFrags = 64;

__device__ __forceinline__ Mat3 rodrigues(float3 k, float theta) {
    float st, ct;
    sincosf(theta, &st, &ct);
    const float omc = 1.f - ct;
    Mat3 m;
    m.r0 = make_float3(ct + k.x * k.x * omc, k.x * k.y * omc - k.z * st, k.y * st + k.x * k.z * omc);
    m.r1 = make_float3(k.z * st + k.x * k.y * omc, ct + k.y * k.y * omc, k.y * k.z * omc - k.x * st);
    m.r2 = make_float3(k.x * k.z * omc - k.y * st, k.x * st + k.y * k.z * omc, ct + k.z * k.z * omc);
    return m;
}

__device__ __forceinline__ Mat3 matmul(const Mat3& a, const Mat3& b) {
    // rows of a times columns of b (multiply_matrix_3x3, math.h:37-49)
    const float3 c0 = make_float3(b.r0.x, b.r1.x, b.r2.x);
    const float3 c1 = make_float3(b.r0.y, b.r1.y, b.r2.y);
    const float3 c2 = make_float3(b.r0.z, b.r1.z, b.r2.z);
    Mat3 m;
    m.r0 = make_float3(dot3(a.r0, c0), dot3(a.r0, c1), dot3(a.r0, c2));
    m.r1 = make_float3(dot3(a.r1, c0), dot3(a.r1, c1), dot3(a.r1, c2));
    m.r2 = make_float3(dot3(a.r2, c0), dot3(a.r2, c1), dot3(a.r2, c2));
    return m;
}

struct KinShared {
    Mat3 fused[kMaxFrags];
    float3 origin[kMaxFrags];
};

// Applies the torsion tree of L to the pose c (permuted order, smem, float4[N]) in place.
// frag_of[p] is the fragment of position p; mine_of[f] its bond atom (-1 for roots).
__device__ void ligand_forward(const DevLigand& L, float4* c, const int* frag_of,
                               const int* mine_of, const int* parent_of, float3 center,
                               const Mat3& rot, const float* tors, KinShared& ks, int lane) {
    const int N = L.n_atoms;
    // geometric centre over permuted order (calculate_geometric_center, data.h:101-106)
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int p = lane; p < N; p += kWarp) {
        sx += c[p].x;
        sy += c[p].y;
        sz += c[p].z;
    }
    const float3 old_center =
        mul3(make_float3(warp_sum_f(sx), warp_sum_f(sy), warp_sum_f(sz)), 1.f / N);
    // input-frame axes of every torsion (data.cpp:530-537), kept in .w-free float4 slots
    float3 axis_in = make_float3(0.f, 0.f, 0.f);
    int4 tq = make_int4(0, 0, 0, 0);
    if (lane < L.n_tors) {
        tq = __ldg(&L.tors[lane]);
        axis_in = sub3(xyz(c[tq.w]), xyz(c[tq.z]));
        axis_in = mul3(axis_in, 1.f / sqrtf(dot3(axis_in, axis_in)));
    }
    __syncwarp();
    // relative coordinates: every subtraction uses input coordinates (data.cpp:540-559)
    float4 rel[(PXD_MAX_LIGAND_ATOMS + kWarp - 1) / kWarp];
#pragma unroll
    for (int u = 0; u < (PXD_MAX_LIGAND_ATOMS + kWarp - 1) / kWarp; ++u) {
        const int p = lane + u * kWarp;
        if (p >= N) break;
        const int f = frag_of[p];
        float3 anchor;
        if (mine_of[f] < 0) {
            anchor = old_center;  // root fragment
        } else if (p != mine_of[f]) {
            anchor = xyz(c[mine_of[f]]);
        } else {
            const int pf = parent_of[f];
            anchor = mine_of[pf] < 0 ? old_center : xyz(c[mine_of[pf]]);
        }
        const float3 r = sub3(xyz(c[p]), anchor);
        rel[u] = make_float4(r.x, r.y, r.z, 0.f);
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < (PXD_MAX_LIGAND_ATOMS + kWarp - 1) / kWarp; ++u) {
        const int p = lane + u * kWarp;
        if (p >= N) break;
        c[p] = rel[u];
    }
    __syncwarp();
    // frames, pre-order
    if (lane == 0) {
        for (int f = 0; f < L.n_frags; ++f) {
            if (mine_of[f] < 0) {
                ks.fused[f] = rot;
                ks.origin[f] = center;
            }
        }
    }
    __syncwarp();
    for (int k = 0; k < L.n_tors; ++k) {
        const int4 q = make_int4(__shfl_sync(kFull, tq.x, k), __shfl_sync(kFull, tq.y, k),
                                 __shfl_sync(kFull, tq.z, k), __shfl_sync(kFull, tq.w, k));
        const float3 ax = make_float3(__shfl_sync(kFull, axis_in.x, k),
                                      __shfl_sync(kFull, axis_in.y, k),
                                      __shfl_sync(kFull, axis_in.z, k));
        if (lane == 0) {
            const Mat3 fp = ks.fused[q.y];
            const float3 axis_w = mat_apply(fp, ax);
            const float3 mine_w = add3(mat_apply(fp, xyz(c[q.w])), ks.origin[q.y]);
            ks.fused[q.x] = matmul(rodrigues(axis_w, tors[k]), fp);
            ks.origin[q.x] = mine_w;
        }
        __syncwarp();
    }
    for (int p = lane; p < N; p += kWarp) {
        const int f = frag_of[p];
        float3 w;
        if (mine_of[f] >= 0 && p == mine_of[f]) {
            w = ks.origin[f];
        } else {
            w = add3(mat_apply(ks.fused[f], xyz(c[p])), ks.origin[f]);
        }
        c[p] = make_float4(w.x, w.y, w.z, 0.f);
    }
    __syncwarp();
}

struct LigKinArgs {
    DevLigand L;
    int n_poses;
    const float* xyz_in;   // [N][3] reference pose (atom order)
    const float* centers;  // [P][3]
    const float* rots;     // [P][9]
    const float* tors;     // [P][T]
    float* out;            // [P][N][3]
};

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
        const float* r = a.rots + 9 * static_cast<size_t>(pose);
        Mat3 rot;
        rot.r0 = make_float3(r[0], r[1], r[2]);
        rot.r1 = make_float3(r[3], r[4], r[5]);
        rot.r2 = make_float3(r[6], r[7], r[8]);
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
    LigKinArgs a{L, n_poses, xyz_in, centers, rots, tors, xyz_out};
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
    cudaMemcpyAsync(mem, xyz0.data(), b0, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(static_cast<char*>(mem) + b0, rotor.data(), b1, cudaMemcpyHostToDevice, s);
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

}  // namespace pxd
