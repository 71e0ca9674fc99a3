// cache_train.cuh -- the pieces of online radiance-cache training shared by
// the single-scene cache (pm_cache_*) and the per-scene caches of a batch
// (pm_batch_cache_*): configuration checks, the hash grid of a scene, one
// network's device arrays, and one frame's picks and k-NN targets.
#pragma once
#include "cache.cuh"
#include "pm.h"

namespace pm {

// One frame's training picks: their queries, keys and records in (map,
// Morton) order, their k-NN targets, and the same in training order (batch
// after batch, each batch every nb-th sorted pick). Networks that train one
// after another on a stream share it.
struct TrainScratch {
    uint32_t ns = 0;                    // picks per frame
    uint32_t *sel = nullptr;            // picked queries
    uint32_t *skey = nullptr, *sval = nullptr, *skey_tmp = nullptr, *sval_tmp = nullptr;
    uint32_t *shist = nullptr, *sn = nullptr;
    uint32_t *run_ctr = nullptr;        // the target launch's run counter
    float4 *pqa = nullptr, *pqd = nullptr, *pval = nullptr;  // sorted picks: records, targets
    uint32_t *pord = nullptr;           // identity order of the sorted picks
    float4 *tqa = nullptr, *tqd = nullptr, *tgt = nullptr;   // training order: records, targets
    uint32_t *tsel = nullptr;           // training order: queries
    float *scale_sum = nullptr;         // one word
};
cudaError_t train_scratch_alloc(uint32_t ns, TrainScratch *t);
void train_scratch_free(TrainScratch &t);

bool cache_config_ok(const pm_cache_config &cfg);
// Levels and resolutions of the configuration; the unit box.
void cache_grid_init(const pm_cache_config &cfg, CacheGrid *g);
// The grid box: the scene box (walls included) with a 1 % margin.
void cache_grid_box(CacheGrid &g, const pm_scene &sc);
size_t cache_table_floats(const pm_cache_config &cfg);
// One network's parameters, moments, gradients, fp16 table, weight image,
// loss and status word, initialised from cfg.seed; with parts_cap > 0 also
// the per-step scratch (weight-gradient rows of parts_cap CTAs, feature
// gradients and tile images of cfg.batch samples).
cudaError_t cache_net_alloc(const pm_cache_config &cfg, const CacheGrid &g, uint64_t seed, int parts_cap,
                            CacheParams *p);
void cache_net_free(CacheParams &p);

// Training batches of a frame of ns picks (every one a spatially
// stratified sample, cache_train_order) and the slots [*o, *o + *n) of
// batch b.
uint32_t cache_batch_count(uint32_t ns, uint32_t batch);
void cache_batch_range(uint32_t ns, uint32_t nb, uint32_t b, uint32_t *o, uint32_t *n);

// A frame's picks (uniform, stratified between diffuse and volume queries;
// frame number `frame`, or *frame_dev when set) of the query list
// qa/qd[0..nq) with diffuse queries slist[0..nsurf), and their k-NN targets,
// into t in training order. The picks are sorted by (map, Morton code),
// their records gathered in that order and estimated in runs of
// warm-started list searches (picks this sparse are too far apart to share
// candidate sets), then batch b takes every nb-th sorted pick.
cudaError_t cache_pick_and_target(const pm_cache_config &cfg, const CacheGrid &grid, uint32_t frame,
                                  const unsigned long long *frame_dev, const PScene &S, const MapView &surf,
                                  const MapView &vol, int k, float radius, const float4 *qa, const float4 *qd,
                                  uint32_t nq, const uint32_t *slist, uint32_t nsurf, TrainScratch &t,
                                  int sm_count, cudaStream_t s);

}  // namespace pm
