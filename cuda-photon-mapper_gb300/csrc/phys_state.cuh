// phys_state.cuh -- the physically based mode's per-context state, shared
// by the C ABI implementation files (physical.cu, cache_api.cu).
#pragma once
#include "gather.cuh"
#include "pm.h"

// The frame as a list of radiance queries (every volume march sample and
// every diffuse hit of every eye path, as the render visits them; see
// eye_path.cuh), shared by the k-NN render and the learned cache.
struct QueryList {
    uint32_t npix_cap = 0;
    uint32_t *cnt = nullptr, *off = nullptr;    // per pixel: queries, exclusive scan (+ total)
    uint32_t *scnt = nullptr, *soff = nullptr;  // per pixel: diffuse queries (0 or 1), scan
    uint32_t *slist = nullptr;                  // indices of the diffuse queries
    uint32_t *scan_tmp = nullptr;
    float4 *qa = nullptr, *qd = nullptr;        // query records, 32-pixel blocks sample-major
    float4 *val = nullptr;                      // per-query values of the last pass
    int val_owner = 0;                          // who wrote val: 0 nobody, 1 pm_render, 2 cache
    uint32_t qcap = 0, nq = 0, nsurf = 0;
    uint64_t gen = 0;                           // scene generation the list was built for
    int flags = -1;                             // bit 0: volume queries, bit 1: diffuse
    // spatial order: (map, Morton code) sort of the queries
    uint32_t *key = nullptr, *ord = nullptr, *key_tmp = nullptr, *ord_tmp = nullptr;
    uint32_t *hist = nullptr, *n_dev = nullptr;
    uint32_t *order = nullptr;                  // points at the sorted query indices
    uint32_t sort_cap = 0;
    bool sorted = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float ms_build = 0.0f;
    unsigned long long *gather_stats = nullptr;  // counters of the last estimate pass
    float *anchor_d = nullptr;                   // per warp chunk of the estimate pass
    uint32_t *defer_n = nullptr;
    uint32_t anchor_cap = 0;
};

struct PhysicalState {
    pm_scene scene;
    pm_config cfg;
    pm::PScene dscene;
    float *het = nullptr;
    uint32_t path_cap = 0;
    int mb = 0;
    uint32_t *cnt[2] = {nullptr, nullptr};  // records per path, per map
    uint32_t *off[2] = {nullptr, nullptr};  // exclusive scans of cnt
    uint32_t *scan_tmp = nullptr;
    // the writing pass's work: ids of the paths holding a record of a map,
    // in increasing order, and the per-tile counts and offsets that place them
    uint32_t *need_list = nullptr, *need_tile = nullptr, *need_tile_off = nullptr;
    uint32_t *words = nullptr;  // [0] path counter [1] stored_s [2] stored_v [3] total [4..7] extents [8] needed paths
    struct Map {
        float4 *pos = nullptr, *pow = nullptr, *tpos = nullptr, *tpow = nullptr;
        float4 *tdir = nullptr;  // decoded directions in tree order
        float4 *lo = nullptr, *hi = nullptr;
        uint32_t cap = 0, n = 0, paths = 0;
        int depth = 0;
        int leaf_shift = 0;
        bool built = false;
    } map[2];
    uint64_t *keys = nullptr, *keys_tmp = nullptr;
    uint32_t *vals = nullptr, *vals_tmp = nullptr, *hist = nullptr;
    uint32_t sort_cap = 0;
    unsigned long long *gctr = nullptr;
    cudaEvent_t ev[8] = {};  // emit, build, render, k-NN estimates within the render: start/stop
    pm_frame_stats stats;
    bool emitted = false;
    bool rendered = false;
    bool gathers_on_host = false;    // last render counted its gathers on the host
    uint64_t host_gathers[2] = {0, 0};
    int sm_count = 148;
    uint64_t gen = 0;  // bumped whenever the scene or the camera changes
    QueryList ql;
};

namespace pm {

inline MapView view_of(const PhysicalState::Map &m) {
    MapView v;
    v.pos = m.tpos;
    v.pow = m.tpow;
    v.dir = m.tdir;
    v.lo = m.lo;
    v.hi = m.hi;
    v.n = m.built ? m.n : 0;
    v.depth = m.depth;
    v.leaf_shift = m.leaf_shift;
    return v;
}

// Builds the query list of the installed camera (always when `force`, else
// only when the scene changed since); synchronises the stream once to size
// the list. Resets the spatial order.
cudaError_t query_list_build(PhysicalState *st, bool force, cudaStream_t s);
// Sorts the list by (map, Morton code of the position in the scene box)
// into ql.order, unless already sorted.
cudaError_t query_list_sort(PhysicalState *st, cudaStream_t s);
void query_list_free(QueryList &ql);
// Exact k-NN values of every query, raw (flux sum, squared radius or -1),
// into ql.val: the list in spatial order, warm-started runs of queries.
cudaError_t knn_values_raw(PhysicalState *st, cudaStream_t s);
constexpr int kGatherStats = 7;
// Scratch of knn_values_tiles: anchor_d[tile_chunks(n, groups)], defer[n],
// two defer_n words (deferred count, chunk counter); stats: kGatherStats
// counters added (nullable).
struct TileBuffers {
    float *anchor_d;
    uint32_t *defer;
    uint32_t *defer_n;
    unsigned long long *stats;
};
// One scene of an estimate pass over many scenes (device memory): its
// scene, maps, query records and values, its queries in (map, Morton)
// order, their count, the first of its chunks in the launch's numbering,
// k and the squared gather radius.
struct TileScene {
    const pm::PScene *sc;
    MapView surf, vol;
    const float4 *qa, *qd;
    float4 *val;
    const uint32_t *order;
    uint32_t n;
    uint32_t chunk_begin;
    int k;
    float r2cap;
};
// knn_values_tiles over the scenes of `scenes` (nsc descriptors, chunks
// numbered scene after scene, total_chunks in all), all with k <= 32 *
// slots, in three launches (anchors, one persistent shared-candidate launch,
// deferred queries). buf.anchor_d holds total_chunks words, buf.defer and
// defer_sc the largest possible number of deferred queries.
cudaError_t knn_values_tiles_multi(const TileScene *scenes, int nsc, uint32_t total_chunks, int groups,
                                   int slots, bool raw, const TileBuffers &buf, uint32_t *defer_sc,
                                   int sm_count, cudaStream_t s);
// Warps of an estimate pass over n queries, `groups` groups of 32 per warp.
uint32_t tile_chunks(uint32_t n, int groups);
// k-NN estimates of the queries in spatial order (order[0..n) indexes qa/qd
// and val; with n_dev, the first min(n, *n_dev): n is then a capacity and
// the launch sizes do not depend on the count), one shared candidate set
// per group of 32 neighbours, `groups`
// (1-4) consecutive groups per warp of which the later ones are bounded by
// the earlier (tile_gather.cu; use 1 when the groups are not neighbours): diffuse queries e / (pi r^2) / pi from the surface map,
// volume queries e / (4/3 pi r^3) with the phase function toward wo from
// the volume map; with raw set, the flux sum e and r^2 (-1 when nothing
// was found) instead.
cudaError_t knn_values_tiles(const PScene &S, const MapView &surf, const MapView &vol,
                             const float4 *qa, const float4 *qd, const uint32_t *order, uint32_t n,
                             const uint32_t *n_dev, int groups, int k, float radius, bool raw,
                             float4 *val, const TileBuffers &buf, int sm_count, cudaStream_t s);

// The render parameters pm_render passes for the installed configuration.
inline RenderParams render_params(const PhysicalState *st) {
    RenderParams R;
    R.width = st->cfg.width;
    R.height = st->cfg.height;
    R.aspect = st->cfg.height > 0 ? (float)st->cfg.width / (float)st->cfg.height : 1.0f;
    R.k = st->cfg.k;
    R.r2cap = st->cfg.radius * st->cfg.radius;
    R.step = st->cfg.march_step;
    R.exposure = st->cfg.exposure;
    R.seed = st->cfg.seed;
    R.scene_id = st->cfg.scene_id;
    R.counters = nullptr;
    return R;
}

}  // namespace pm
