// pm_ctx.cuh -- the context behind a pm_ctx handle, shared by the C ABI
// implementation files.
#pragma once
#include "pm.h"
#include "legacy.cuh"

#include <string>

struct pm_ctx {
    int device = 0;
    std::string err;
    pm::LegacyState legacy;
    bool legacy_ready = false;
    struct PhysicalState *phys = nullptr;
    struct CacheState *cache = nullptr;
};

namespace pm {

// Makes `device` current for the scope and restores the caller's device.
class DeviceGuard {
  public:
    explicit DeviceGuard(int device);
    ~DeviceGuard();

  private:
    int prev_ = 0, dev_ = 0;
};

pm_status fail(pm_ctx *ctx, pm_status s, const std::string &msg);
pm_status check_cuda(pm_ctx *ctx, cudaError_t e, const char *where);
void physical_free(pm_ctx *ctx);
void cache_free(pm_ctx *ctx);

}  // namespace pm
