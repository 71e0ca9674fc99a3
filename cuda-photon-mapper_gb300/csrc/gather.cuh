// gather.cuh -- k-nearest-photon queries and the frame render.
#pragma once
#include "phys_common.cuh"

namespace pm {

// A built photon map as the gather reads it (tree order).
struct MapView {
    const float4 *pos;   // xyz + record index bits
    const float4 *pow;   // rgb flux + octahedral direction bits
    const float4 *dir;   // the decoded directions (xyz)
    const float4 *lo, *hi;
    uint32_t n;
    int depth;
    int leaf_shift = 0;  // leaves hold 32 << leaf_shift records
};

// Search knobs that change the speed of a k-NN query but not its result:
// records collected unsorted before the first sort into the k-list, and
// the leaf candidates at or above which insertion is one bulk merge.
struct KnnTune {
    int collect_max = 128;  // 32, 64 or 128
    int merge_min = 16;
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
    KnnTune tune;
};

// One scene of a batched render (device array entry).
struct BatchRenderScene {
    PScene sc;
    MapView surf, vol;
    RenderParams R;
    float4 *rad;        // this scene's pixels (nullable)
    uchar4 *rgba;       // (nullable)
    int slots;          // k-list width: ceil(k / 32)
    int tile;           // pixels per warp per work chunk (the gather tile)
};

// k-list width (registers per lane) the kernels use for k.
int slots_for_k(int k);
// Renders every scene of the batch in one persistent launch; chunk_prefix
// (nscenes + 1 entries) is the exclusive scan of the scenes' chunk counts
// ceil(pixels / (4 * tile)); work is one device word of scratch.
cudaError_t render_batch(const BatchRenderScene *scenes, const uint32_t *chunk_prefix, int nscenes,
                         uint32_t *work, int sm_count, cudaStream_t s);

cudaError_t knn_query(const MapView &m, const float4 *q, uint32_t nq, int k, float radius,
                      uint32_t *idx, float *d2, cudaStream_t s);
cudaError_t radius_gather(const MapView &m, const float4 *pts, const float4 *nrm, uint32_t nq,
                          float sq_radius, float exposure, float4 *out, cudaStream_t s);
cudaError_t render_frame(const PScene &S, const MapView &surf, const MapView &vol,
                         const RenderParams &R, float4 *rad, uchar4 *rgba, cudaStream_t s);

}  // namespace pm
