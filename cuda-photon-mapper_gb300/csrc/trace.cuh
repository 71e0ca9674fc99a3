// trace.cuh -- photon tracing into per-path slots and compaction into maps.
#pragma once
#include "phys_common.cuh"

namespace pm {

// Bound on tentative collisions per path segment under delta tracking.
constexpr uint32_t kMaxDeltaSteps = 4096;

struct TraceParams {
    uint64_t seed;
    uint32_t scene_id;
    int max_bounces;
    float rr;                     // Russian-roulette survival probability
    uint32_t target_s, target_v;  // map targets: stop issuing paths once both are reached
    uint32_t path_cap;            // slots exist for this many paths
    uint32_t *path_counter;       // next path id
    uint32_t *stored_s, *stored_v;
    float4 *spos, *spow;          // surface slots [path_cap * max_bounces]
    float4 *vpos, *vpow;          // volume slots
    uint32_t *cnt_s, *cnt_v;      // records per path (zeroed before the launch)
};

cudaError_t trace_photons(const PScene &S, const TraceParams &P, int sm_count, cudaStream_t s);

// Scans the per-path counts of the first `issued` paths, finds how many
// paths reach `target` records (extent[0] = records, extent[1] = paths, on
// the device) and copies those records in path order to pos/pw, with the
// record index in pos.w and power scaled by power / paths.
cudaError_t compact_map(uint32_t issued, const uint32_t *cnt, uint32_t *off, uint32_t *total,
                        uint32_t *scan_tmp, uint32_t target, uint32_t *extent, const float4 *spos,
                        const float4 *spow, int mb, float power, float4 *pos, float4 *pw,
                        cudaStream_t s);

}  // namespace pm
