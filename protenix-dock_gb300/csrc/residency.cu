// L2 residency of the receptor maps.
//
// The optimiser and the search gather map records at data-dependent offsets every
// evaluation (receptor_cache::get, grid.cpp:197-303). When the maps of the types a batch
// uses stay L2-resident (the bench's 8 maps, 76 MB, in the 129 MB L2) nothing else is
// needed; when they exceed L2 (a screening batch over many ligand types, or the engine's
// 100 maps), the pose and history traffic of the same launch competes with them for L2.
// pxd_set_l2_residency sets aside part of L2 for persisting lines and marks the map
// records as a persisting access-policy window on every optimiser and search launch of
// the context. The set-aside is a limit of the process's CUDA context on the device; it
// is restored when the last context that asked for one releases it (or is destroyed),
// and it ends with the process.
#include <algorithm>
#include <map>
#include <mutex>

#include "pxd_internal.h"

namespace pxd {

namespace {

struct DeviceShare {
    int users = 0;
    size_t previous = 0;  // the limit before the first user set it
    size_t current = 0;
};

std::mutex g_mu;
std::map<int, DeviceShare> g_devices;

int release_locked(pxd_context* ctx) {
    if (ctx->l2_setaside == 0) return PXD_OK;
    DeviceShare& d = g_devices[ctx->device];
    ctx->l2_setaside = 0;
    if (--d.users > 0) return PXD_OK;
    // the last user: persisting lines back to normal, the limit back to what it was
    int rc = cuda_check(ctx, cudaCtxResetPersistingL2Cache(), "persisting L2 reset");
    if (!rc)
        rc = cuda_check(ctx, cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, d.previous), "persisting L2 limit");
    d.current = d.previous;
    return rc;
}

}  // namespace

cudaLaunchAttribute map_window(const pxd_context* ctx, bool* on) {
    cudaLaunchAttribute attr{};
    *on = false;
    if (ctx->l2_setaside == 0 || !ctx->maps || ctx->n_slots <= 0) return attr;
    const size_t bytes = sizeof(float4) * static_cast<size_t>(ctx->grid.P) * ctx->n_slots;
    const size_t window = std::min(bytes, ctx->l2_max_window);
    if (window == 0) return attr;
    attr.id = cudaLaunchAttributeAccessPolicyWindow;
    attr.val.accessPolicyWindow.base_ptr = ctx->maps;
    attr.val.accessPolicyWindow.num_bytes = window;
    attr.val.accessPolicyWindow.hitRatio =
        static_cast<float>(std::min(1.0, static_cast<double>(ctx->l2_setaside) / static_cast<double>(window)));
    attr.val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr.val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    *on = true;
    return attr;
}

int release_l2_residency(pxd_context* ctx) {
    std::lock_guard<std::mutex> lock(g_mu);
    return release_locked(ctx);
}

}  // namespace pxd

using namespace pxd;

extern "C" int pxd_set_l2_residency(pxd_context* ctx, double fraction) {
    if (!ctx) return PXD_ERR_INVALID;
    if (!(fraction >= 0.0 && fraction <= 1.0))
        return set_error(ctx, PXD_ERR_INVALID, "L2 residency fraction must lie in [0, 1]");
    cudaSetDevice(ctx->device);
    std::lock_guard<std::mutex> lock(g_mu);
    int rc = release_locked(ctx);
    if (rc || fraction == 0.0) return rc;
    int max_persist = 0, max_window = 0;
    rc = cuda_check(ctx, cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, ctx->device),
                    "persisting L2 size");
    if (!rc)
        rc = cuda_check(ctx, cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, ctx->device),
                        "access-policy window size");
    if (rc) return rc;
    if (max_persist <= 0 || max_window <= 0)
        return set_error(ctx, PXD_ERR_STATE, "the device offers no persisting L2 set-aside");
    const size_t want = static_cast<size_t>(fraction * max_persist);
    if (want == 0) return PXD_OK;
    DeviceShare& d = g_devices[ctx->device];
    if (d.users == 0) {
        rc = cuda_check(ctx, cudaDeviceGetLimit(&d.previous, cudaLimitPersistingL2CacheSize), "persisting L2 limit");
        if (rc) return rc;
        d.current = d.previous;
    }
    if (want > d.current) {
        rc = cuda_check(ctx, cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want), "persisting L2 limit");
        if (rc) return rc;
        d.current = want;
    }
    ++d.users;
    ctx->l2_setaside = want;
    ctx->l2_max_window = static_cast<size_t>(max_window);
    return PXD_OK;
}
