// Gather-bandwidth probe: random 16-byte loads over a device-resident working set, the
// access pattern of the map lookups (grid_lookup: float4 records at data-dependent
// offsets, read through L1 with ld.global.nc). With a working set below the L2 size
// (129 MB on GB300) and well above L1 it measures the L2 gather bandwidth that bounds the
// batched kernels whose maps stay L2-resident; with a larger set, the HBM gather
// bandwidth. Used by the bench to state its roofline against a measured L2 figure.
#include <algorithm>
#include <vector>

#include "pxd_internal.h"

namespace pxd {

namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeLoads = 256;  // loads per thread per launch, 8 in flight

__global__ void probe_fill_kernel(float4* buf, size_t n) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        buf[i] = make_float4(1.f, 0.5f, 0.25f, static_cast<float>(i & 1023));
}

// 32-bit mix (a Murmur3-style finaliser) of the thread's load number: uniform offsets.
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

// Each thread makes kProbeLoads independent 16-byte loads at hashed offsets in
// [0, mask] and folds them into one value so that no load is dead.
__global__ void __launch_bounds__(kProbeThreads) probe_gather_kernel(const float4* __restrict__ buf, uint32_t mask,
                                                                    uint32_t salt, float* out) {
    const uint32_t t = blockIdx.x * kProbeThreads + threadIdx.x;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 8
    for (int k = 0; k < kProbeLoads; ++k) {
        const uint32_t idx = mix32(t * kProbeLoads + k + salt) & mask;
        const float4 v = __ldg(&buf[idx]);
        acc.x += v.x;
        acc.y += v.y;
        acc.z += v.z;
        acc.w += v.w;
    }
    out[t] = acc.x + acc.y + acc.z + acc.w;
}

}  // namespace

}  // namespace pxd

using namespace pxd;

extern "C" int pxd_gather_bandwidth(int32_t device, int64_t working_set_bytes, int32_t reps, double* gbs) {
    if (!gbs || reps < 1 || working_set_bytes < (int64_t(1) << 20)) return PXD_ERR_INVALID;
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || device < 0 || device >= n_dev) return PXD_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return PXD_ERR_CUDA;
    int n_sm = 0;
    if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return PXD_ERR_CUDA;
    // the working set as a power-of-two count of float4 records, at most 2^31
    size_t n = 1;
    while (n * 2 * sizeof(float4) <= static_cast<size_t>(working_set_bytes) && n < (size_t(1) << 31)) n *= 2;
    const int blocks = n_sm * 8;
    const size_t threads = static_cast<size_t>(blocks) * kProbeThreads;
    float4* buf = nullptr;
    float* out = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = PXD_OK;
    auto ok = [&rc](cudaError_t e) {
        if (e != cudaSuccess && rc == PXD_OK) rc = PXD_ERR_CUDA;
        return rc == PXD_OK;
    };
    std::vector<float> ms;
    if (ok(cudaMalloc(&buf, n * sizeof(float4))) && ok(cudaMalloc(&out, threads * sizeof(float))) &&
        ok(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) && ok(cudaEventCreate(&e0)) &&
        ok(cudaEventCreate(&e1))) {
        probe_fill_kernel<<<n_sm * 8, 256, 0, s>>>(buf, n);
        ok(cudaGetLastError());
        const uint32_t mask = static_cast<uint32_t>(n - 1);
        for (int r = 0; r < reps + 2 && rc == PXD_OK; ++r) {  // two warm-up launches
            ok(cudaEventRecord(e0, s));
            probe_gather_kernel<<<blocks, kProbeThreads, 0, s>>>(buf, mask, 0x9e3779b9U * r, out);
            ok(cudaGetLastError());
            ok(cudaEventRecord(e1, s));
            if (ok(cudaEventSynchronize(e1)) && r >= 2) {
                float t = 0.f;
                if (ok(cudaEventElapsedTime(&t, e0, e1))) ms.push_back(t);
            }
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (out) cudaFree(out);
    if (buf) cudaFree(buf);
    if (rc) return rc;
    std::sort(ms.begin(), ms.end());
    const double t = ms[ms.size() / 2] * 1e-3;  // median launch
    *gbs = static_cast<double>(threads) * kProbeLoads * sizeof(float4) / t / 1e9;
    return PXD_OK;
}
