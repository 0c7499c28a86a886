// Ligand torsion-tree forward kinematics for one pose held by a warp (shared by the
// kinematics and Monte-Carlo kernels); see kinematics.cu for the algorithm.
#pragma once

#include "device_eval.cuh"

namespace pxd {

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

// Rotation matrix of the quaternion q4 = (w, x, y, z) after normalisation
// (get_rotation_matrix, math.cpp:22-42).
__device__ __forceinline__ Mat3 unit_quat_rotation(const float* q4) {
    const float inv = rsqrtf(q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
    const float a = q4[0] * inv, b = q4[1] * inv, c = q4[2] * inv, d = q4[3] * inv;
    Mat3 m;
    m.r0 = make_float3(a * a + b * b - c * c - d * d, 2.f * (b * c - a * d), 2.f * (a * c + b * d));
    m.r1 = make_float3(2.f * (a * d + b * c), a * a - b * b + c * c - d * d, 2.f * (c * d - a * b));
    m.r2 = make_float3(2.f * (b * d - a * c), 2.f * (a * b + c * d), a * a - b * b - c * c + d * d);
    return m;
}

struct KinShared {
    Mat3 fused[kMaxFrags];
    float3 origin[kMaxFrags];
};

// Applies the torsion tree of L to the pose c (permuted order, smem, float4[N]) in place.
// frag_of[p] is the fragment of position p; mine_of[f] its bond atom (-1 for roots).
static __device__ void ligand_forward(const DevLigand& L, float4* c, const int* frag_of,
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

}  // namespace pxd
