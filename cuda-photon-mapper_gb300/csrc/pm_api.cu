// pm_api.cu -- the C ABI (include/pm.h): contexts, status codes, and the
// reference's three exports on an implicit context.
#include "pm.h"
#include "pm_ctx.cuh"

#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <new>
#include <string>

namespace pm {

DeviceGuard::DeviceGuard(int device) {
    cudaGetDevice(&prev_);
    if (prev_ != device) cudaSetDevice(device);
    dev_ = device;
}
DeviceGuard::~DeviceGuard() {
    if (prev_ != dev_) cudaSetDevice(prev_);
}

pm_status fail(pm_ctx *ctx, pm_status s, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return s;
}

pm_status check_cuda(pm_ctx *ctx, cudaError_t e, const char *where) {
    if (e == cudaSuccess) return PM_OK;
    return fail(ctx, e == cudaErrorMemoryAllocation ? PM_ERR_ALLOC : PM_ERR_CUDA,
                std::string(where) + ": " + cudaGetErrorString(e));
}

static pm_status ensure_legacy(pm_ctx *ctx) {
    if (ctx->legacy_ready) return PM_OK;
    pm_status s = check_cuda(ctx, legacy_alloc(ctx->legacy), "legacy allocation");
    if (s == PM_OK) ctx->legacy_ready = true;
    return s;
}

}  // namespace pm

using namespace pm;

extern "C" {

const char *pm_status_string(pm_status s) {
    switch (s) {
        case PM_OK: return "ok";
        case PM_ERR_INVALID: return "invalid argument";
        case PM_ERR_CUDA: return "CUDA error";
        case PM_ERR_ALLOC: return "device allocation failed";
        case PM_ERR_STATE: return "call out of order";
        case PM_ERR_LIMIT: return "size beyond the supported maximum";
        case PM_ERR_TIMEOUT: return "device wait timed out";
    }
    return "unknown status";
}

pm_status pm_create(pm_ctx **out, int device) {
    if (!out) return PM_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return PM_ERR_INVALID;
    }
    pm_ctx *ctx = new (std::nothrow) pm_ctx();
    if (!ctx) return PM_ERR_ALLOC;
    ctx->device = device;
    *out = ctx;
    return PM_OK;
}

void pm_destroy(pm_ctx *ctx) {
    if (!ctx) return;
    {
        DeviceGuard g(ctx->device);
        if (ctx->legacy_ready) legacy_free(ctx->legacy);
        physical_free(ctx);
        cache_free(ctx);
    }
    delete ctx;
}

const char *pm_last_error(const pm_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

pm_status pm_legacy_init_random(pm_ctx *ctx, cudaStream_t stream) {
    if (!ctx) return PM_ERR_INVALID;
    DeviceGuard g(ctx->device);
    pm_status s = ensure_legacy(ctx);
    if (s != PM_OK) return s;
    return check_cuda(ctx, legacy_init_random(ctx->legacy, stream), "init_random");
}

pm_status pm_legacy_emit(pm_ctx *ctx, float anim_time, int flags, cudaStream_t stream) {
    if (!ctx || (flags & ~(PM_LEGACY_INTERPOLATE | PM_LEGACY_MEDIA))) return PM_ERR_INVALID;
    DeviceGuard g(ctx->device);
    pm_status s = ensure_legacy(ctx);
    if (s != PM_OK) return s;
    return check_cuda(ctx, legacy_emit(ctx->legacy, anim_time, flags, stream), "emit");
}

pm_status pm_legacy_render(pm_ctx *ctx, uchar4 *pos, unsigned width, unsigned height,
                           float anim_time, int flags, float *rgb_out, cudaStream_t stream) {
    if (!ctx || (flags & ~(PM_LEGACY_INTERPOLATE | PM_LEGACY_MEDIA))) return PM_ERR_INVALID;
    if ((width != 0 && height != 0) && !pos) return fail(ctx, PM_ERR_INVALID, "null output");
    if ((unsigned long long)width * height > 0xFFFFFFFFull)
        return fail(ctx, PM_ERR_LIMIT, "image larger than 2^32 pixels");
    DeviceGuard g(ctx->device);
    pm_status s = ensure_legacy(ctx);
    if (s != PM_OK) return s;
    return check_cuda(ctx,
                      legacy_render(ctx->legacy, pos, width, height, anim_time, flags, rgb_out, stream),
                      "render");
}

pm_status pm_legacy_get_grid(pm_ctx *ctx, float *host_out) {
    if (!ctx || !host_out) return PM_ERR_INVALID;
    DeviceGuard g(ctx->device);
    pm_status s = ensure_legacy(ctx);
    if (s != PM_OK) return s;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy(host_out, ctx->legacy.grid3, sizeof(float) * 3 * kLegacyVoxels,
                       cudaMemcpyDeviceToHost);
    return check_cuda(ctx, e, "get_grid");
}

pm_status pm_legacy_set_grid(pm_ctx *ctx, const float *host_in) {
    if (!ctx || !host_in) return PM_ERR_INVALID;
    DeviceGuard g(ctx->device);
    pm_status s = ensure_legacy(ctx);
    if (s != PM_OK) return s;
    cudaError_t e = legacy_upload_grid(ctx->legacy, host_in, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return check_cuda(ctx, e, "set_grid");
}

pm_status pm_legacy_get_random_numbers(pm_ctx *ctx, float *host_out) {
    if (!ctx || !host_out) return PM_ERR_INVALID;
    DeviceGuard g(ctx->device);
    pm_status s = ensure_legacy(ctx);
    if (s != PM_OK) return s;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy2D(host_out, 3 * sizeof(float), ctx->legacy.table, sizeof(float4),
                         3 * sizeof(float), kLegacyPhotons, cudaMemcpyDeviceToHost);
    return check_cuda(ctx, e, "get_random_numbers");
}

pm_status pm_legacy_rng_draws(pm_ctx *ctx, unsigned long long *draws) {
    if (!ctx || !draws) return PM_ERR_INVALID;
    *draws = ctx->legacy.rng_draws;
    return PM_OK;
}

// ---- the reference's exports ------------------------------------------------

static std::mutex g_legacy_mu;
static pm_ctx *g_legacy = nullptr;
static int g_exit_on_error = 1;
static int g_last_status = PM_OK;
static std::string g_last_error;

static void legacy_report(pm_status s, const char *what) {
    g_last_status = s;
    if (s == PM_OK) return;
    g_last_error = std::string(what) + " failed!: " + (g_legacy ? g_legacy->err : "no device");
    if (g_exit_on_error) {
        // checkCUDAError (photonMappingKernel.cu:49-55)
        fprintf(stderr, "Cuda error: %s.\n", g_last_error.c_str());
        exit(EXIT_FAILURE);
    }
}

static pm_status legacy_ctx() {
    if (g_legacy) return PM_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    return pm_create(&g_legacy, dev);
}

void pm_legacy_set_exit_on_error(int exit_on_error) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    g_exit_on_error = exit_on_error;
}
int pm_legacy_last_status(void) { return g_last_status; }
const char *pm_legacy_last_error(void) { return g_last_error.c_str(); }

void pm_legacy_release(void) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    pm_destroy(g_legacy);
    g_legacy = nullptr;
}

void launch_init_random_numbers_kernel(void) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    pm_status s = legacy_ctx();
    if (s == PM_OK) s = pm_legacy_init_random(g_legacy, 0);
    if (s == PM_OK) s = check_cuda(g_legacy, cudaDeviceSynchronize(), "synchronize");
    legacy_report(s, "init_random_numbers_kernel");
}

void launch_emit_photons_kernel(uchar4 *pos, unsigned int image_width, unsigned int image_height,
                                float animTime, bool interpolateFlag, bool participatingMediaFlag) {
    (void)pos; (void)image_width; (void)image_height;
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    int flags = (interpolateFlag ? PM_LEGACY_INTERPOLATE : 0) | (participatingMediaFlag ? PM_LEGACY_MEDIA : 0);
    pm_status s = legacy_ctx();
    if (s == PM_OK) s = pm_legacy_emit(g_legacy, animTime, flags, 0);
    if (s == PM_OK) s = check_cuda(g_legacy, cudaDeviceSynchronize(), "synchronize");
    legacy_report(s, "emit_photons_kernel");
}

void launch_photon_mapping_kernel(uchar4 *pos, unsigned int image_width, unsigned int image_height,
                                  float animTime, bool interpolateFlag,
                                  bool participatingMediaFlag) {
    std::lock_guard<std::mutex> lk(g_legacy_mu);
    int flags = (interpolateFlag ? PM_LEGACY_INTERPOLATE : 0) | (participatingMediaFlag ? PM_LEGACY_MEDIA : 0);
    pm_status s = legacy_ctx();
    if (s == PM_OK) s = pm_legacy_render(g_legacy, pos, image_width, image_height, animTime, flags, nullptr, 0);
    if (s == PM_OK) s = check_cuda(g_legacy, cudaDeviceSynchronize(), "synchronize");
    legacy_report(s, "photon_mapping_kernel");
}

}  // extern "C"
