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
    uint32_t target_s, target_v;  // map targets: counting stops issuing paths once both are met
    uint32_t path_cap;            // counting pass: most paths that may be issued
    uint32_t *path_counter;       // next path id (zeroed before each pass)
    uint32_t *stored_s, *stored_v;
    uint32_t *cnt_s, *cnt_v;      // records per path (zeroed before the counting pass)
    // Writing pass (store != 0): the paths below max(ext_s[1], ext_v[1])
    // that hold a record of a map (cnt > 0) are traced again, each record
    // written straight to map index off[p] + k when below the map size
    // ext[0], power scaled by power / ext[1].
    int store;
    const uint32_t *off_s, *off_v;
    const uint32_t *ext_s, *ext_v;
    float power;
    float4 *spos, *spow, *vpos, *vpow;
    // Writing pass with a list (nullable): the paths to trace are
    // list[0 .. *list_n), instead of every id below the extents whose
    // counts are nonzero.
    const uint32_t *list, *list_n;
};

// One persistent launch over the photon paths (counting or writing pass).
cudaError_t trace_photons(const PScene &S, const TraceParams &P, int sm_count, cudaStream_t s);

// Scans the per-path counts of the first `issued` paths into off and finds
// how many paths reach `target` records: extent[0] = records, extent[1] =
// paths (device).
cudaError_t map_extent(uint32_t issued, const uint32_t *cnt, uint32_t *off, uint32_t *total,
                       uint32_t *scan_tmp, uint32_t target, uint32_t *extent, cudaStream_t s);
// The same without a host round trip: scans all `cap` counts (zero beyond
// the issued paths) and reads the issued count from issued_dev.
cudaError_t map_extent_dev(uint32_t cap, const uint32_t *issued_dev, const uint32_t *cnt,
                           uint32_t *off, uint32_t *total, uint32_t *scan_tmp, uint32_t target,
                           uint32_t *extent, cudaStream_t s);
// map_extent_dev of many maps in one launch, their counts already scanned
// (off[i] the counts of paths before i, e.g. by a segmented scan of a pool).
struct ExtentJob {
    const uint32_t *cnt, *off;  // the map's per-path counts and their scan, over cap paths
    uint32_t cap, target;
    const uint32_t *issued;     // paths the counting pass issued (device)
    uint32_t *total;            // out: records of all cap paths
    uint32_t *extent;           // out: records, paths
};
cudaError_t map_extents_multi(const ExtentJob *jobs, int n, cudaStream_t s);
// The ids below `issued` of the paths that hold a record of a map (id <
// ext_s[1] with cnt_s > 0, or id < ext_v[1] with cnt_v > 0), in increasing
// order, into list[0 .. *list_n): per-tile counts, a scan of them, then each
// tile's ids placed at its offset. tile_cnt / tile_off hold
// needed_tiles(issued) words; scan_tmp as exclusive_scan_u32_large's.
uint32_t needed_tiles(uint32_t n);
cudaError_t needed_paths(uint32_t issued, const uint32_t *cnt_s, const uint32_t *cnt_v,
                         const uint32_t *ext_s, const uint32_t *ext_v, uint32_t *tile_cnt,
                         uint32_t *tile_off, uint32_t *scan_tmp, uint32_t *list, uint32_t *list_n,
                         cudaStream_t s);
// One persistent launch over the paths of n scenes (scenes and params are
// device arrays; each scene's params carry its own counters and maps).
cudaError_t trace_photons_batch(const PScene *scenes, const TraceParams *params, int n,
                                int sm_count, cudaStream_t s);
// Fills records [*n_dev, cap) of a map with records at infinity (never
// within any radius), so a tree built over `cap` records serves a map of
// *n_dev records.
cudaError_t pad_map(float4 *pos, float4 *pw, const uint32_t *n_dev, uint32_t cap, cudaStream_t s);

}  // namespace pm
