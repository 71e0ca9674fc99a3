// gather.cuh -- k-nearest-photon queries and the frame render.
#pragma once
#include "phys_common.cuh"

namespace pm {

// A built photon map as the gather reads it (tree order).
struct MapView {
    const float4 *pos;   // xyz + record index bits
    const float4 *pow;   // rgb flux + octahedral direction bits
    const float4 *lo, *hi;
    uint32_t n;
    int depth;
};

struct RenderParams {
    int width, height;
    float aspect;        // width / height
    int k;
    float r2cap;         // radius^2
    float step;          // volume march step (0: no march)
    float exposure;
    uint64_t seed;
    uint32_t scene_id;
    unsigned long long *counters;  // [0] surface gathers, [1] volume gathers (nullable)
};

cudaError_t knn_query(const MapView &m, const float4 *q, uint32_t nq, int k, float radius,
                      uint32_t *idx, float *d2, cudaStream_t s);
cudaError_t radius_gather(const MapView &m, const float4 *pts, const float4 *nrm, uint32_t nq,
                          float sq_radius, float exposure, float4 *out, cudaStream_t s);
cudaError_t render_frame(const PScene &S, const MapView &surf, const MapView &vol,
                         const RenderParams &R, float4 *rad, uchar4 *rgba, cudaStream_t s);

}  // namespace pm
