// physical.cu -- physically based mode (filled in by the physical kernels).
#include "pm_ctx.cuh"

namespace pm {
void physical_free(pm_ctx *ctx) { (void)ctx; }
}  // namespace pm
