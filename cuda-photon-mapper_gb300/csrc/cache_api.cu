// cache_api.cu -- the learned radiance cache behind the pm_cache_* C ABI:
// configuration, the per-camera query list, online training frames, cached
// and k-NN renders through the query list, parameter access and files.
#include "cache.cuh"
#include "cache_train.cuh"
#include "phys_state.cuh"
#include "pm_ctx.cuh"
#include "radix_sort.cuh"
#include "tc.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

struct CacheState {
    pm_cache_config cfg;
    pm::CacheGrid grid;
    pm::CacheParams p;
    size_t table_floats = 0;
    int sm_count = 148;
    // the query list itself lives in the physical state (shared with pm_render);
    // the frame's picks and targets
    pm::TrainScratch ts;
    float target_scale = 0.0f;  // 0: set from the first training frame
    unsigned long long steps = 0, frames = 0;
    cudaEvent_t ev[7] = {};  // queries start/end, values start, values end/composite start, composite end, train mid/end
    cudaEvent_t tev0 = nullptr;
    bool rendered = false, trained = false;
    pm_cache_stats stats;
};

namespace pm {

constexpr int kTargetRun = 8;  // training targets warm-started in runs of this length

namespace {
template <typename T>
cudaError_t talloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, sizeof(T) * count);
}
}  // namespace

cudaError_t train_scratch_alloc(uint32_t ns, TrainScratch *t) {
    cudaError_t e;
#define TS_TRY(x) do { e = (x); if (e != cudaSuccess) { train_scratch_free(*t); return e; } } while (0)
    *t = TrainScratch();
    t->ns = ns;
    TS_TRY(talloc(&t->sel, ns));
    TS_TRY(talloc(&t->skey, ns));
    TS_TRY(talloc(&t->sval, ns));
    TS_TRY(talloc(&t->skey_tmp, ns));
    TS_TRY(talloc(&t->sval_tmp, ns));
    TS_TRY(talloc(&t->shist, radix_sort_hist_words(ns)));
    TS_TRY(talloc(&t->sn, 1));
    TS_TRY(talloc(&t->run_ctr, 1));
    TS_TRY(talloc(&t->pqa, ns));
    TS_TRY(talloc(&t->pqd, ns));
    TS_TRY(talloc(&t->pval, ns));
    TS_TRY(talloc(&t->pord, ns));
    TS_TRY(talloc(&t->tqa, ns));
    TS_TRY(talloc(&t->tqd, ns));
    TS_TRY(talloc(&t->tgt, ns));
    TS_TRY(talloc(&t->tsel, ns));
    TS_TRY(talloc(&t->scale_sum, 1));
    TS_TRY(cudaMemcpy(t->sn, &ns, sizeof(uint32_t), cudaMemcpyHostToDevice));
#undef TS_TRY
    return cudaSuccess;
}

void train_scratch_free(TrainScratch &t) {
    cudaFree(t.sel); cudaFree(t.skey); cudaFree(t.sval); cudaFree(t.skey_tmp); cudaFree(t.sval_tmp);
    cudaFree(t.shist); cudaFree(t.sn); cudaFree(t.run_ctr);
    cudaFree(t.pqa); cudaFree(t.pqd); cudaFree(t.pval); cudaFree(t.pord);
    cudaFree(t.tqa); cudaFree(t.tqd); cudaFree(t.tgt); cudaFree(t.tsel); cudaFree(t.scale_sum);
    t = TrainScratch();
}

bool cache_config_ok(const pm_cache_config &cfg) {
    return !(cfg.levels < 1 || cfg.levels > kCacheMaxLevels || cfg.log2_table < 8 || cfg.log2_table > 22 ||
             cfg.base_res < 2 || cfg.max_res < cfg.base_res || cfg.max_res > 65536 ||
             cfg.train_samples < 1 || cfg.train_samples > (1u << 24) || cfg.batch < 128 ||
             cfg.batch % 128 != 0 || !(cfg.lr > 0.0f) || !(cfg.beta1 >= 0.0f && cfg.beta1 < 1.0f) ||
             !(cfg.beta2 >= 0.0f && cfg.beta2 < 1.0f) || !(cfg.eps >= 0.0f) ||
             !(cfg.lr_min >= 0.0f) || !(cfg.lr_half_life >= 0.0f) || !(cfg.loss_eps > 0.0f) ||
             !(cfg.surface_fraction >= 0.0f && cfg.surface_fraction <= 1.0f));
}

void cache_grid_init(const pm_cache_config &cfg, CacheGrid *g) {
    memset(g, 0, sizeof(*g));
    g->levels = cfg.levels;
    g->log2_t = (uint32_t)cfg.log2_table;
    const double b = cfg.levels > 1 ? std::exp(std::log((double)cfg.max_res / cfg.base_res) / (cfg.levels - 1)) : 1.0;
    for (int l = 0; l < cfg.levels; ++l) g->res[l] = (int)std::floor(cfg.base_res * std::pow(b, l) + 1e-6);
    for (int a = 0; a < 3; ++a) {
        g->lo[a] = 0.0f;
        g->inv_size[a] = 1.0f;
    }
}

void cache_grid_box(CacheGrid &g, const pm_scene &sc) {
    for (int a = 0; a < 3; ++a) {
        const float ext = sc.box_max[a] - sc.box_min[a];
        const float m = 0.01f * (ext > 0.0f ? ext : 1.0f);
        g.lo[a] = sc.box_min[a] - m;
        const float size = ext + 2.0f * m;
        g.inv_size[a] = size > 0.0f ? 1.0f / size : 1.0f;
    }
}

size_t cache_table_floats(const pm_cache_config &cfg) { return (size_t)cfg.levels << (cfg.log2_table + 1); }

cudaError_t cache_net_alloc(const pm_cache_config &cfg, const CacheGrid &g, uint64_t seed, int parts_cap,
                            CacheParams *out) {
    CacheParams p;
    memset(&p, 0, sizeof(p));
    const size_t tf = cache_table_floats(cfg);
    cudaError_t e;
#define NA_TRY(x) do { e = (x); if (e != cudaSuccess) { cache_net_free(p); return e; } } while (0)
    NA_TRY(talloc(&p.w, kCacheWeights));
    NA_TRY(talloc(&p.w_grad, kCacheWeights));
    NA_TRY(talloc(&p.w_m, kCacheWeights));
    NA_TRY(talloc(&p.w_v, kCacheWeights));
    NA_TRY(talloc(&p.table, tf));
    NA_TRY(talloc(&p.table_grad, tf));
    NA_TRY(talloc(&p.table_m, tf));
    NA_TRY(talloc(&p.table_v, tf));
    NA_TRY(talloc(&p.table_h, tf / 2));
    NA_TRY(talloc(&p.w_img, kCacheWImageBytes / 16));
    NA_TRY(talloc(&p.loss, 1));
    NA_TRY(talloc(&p.status, 1));
    NA_TRY(cudaMemset(p.status, 0, sizeof(int)));
    if (parts_cap > 0) {
        p.parts_cap = parts_cap;
        NA_TRY(talloc(&p.w_part, (size_t)parts_cap * kCacheWeights));
        NA_TRY(talloc(&p.loss_part, parts_cap));
        p.dx_cap = cfg.batch;
        NA_TRY(talloc(&p.dx, (size_t)cfg.batch * 8));
        NA_TRY(talloc(&p.xt, (size_t)cfg.batch * 8));
    }
    p.wait_polls = kMbarSpin;
    NA_TRY(cache_init(g, p, seed, 0));
#undef NA_TRY
    *out = p;
    return cudaSuccess;
}

void cache_net_free(CacheParams &p) {
    cudaFree(p.w); cudaFree(p.w_grad); cudaFree(p.w_m); cudaFree(p.w_v);
    cudaFree(p.table); cudaFree(p.table_grad); cudaFree(p.table_m); cudaFree(p.table_v); cudaFree(p.table_h);
    cudaFree(p.w_img); cudaFree(p.loss); cudaFree(p.status);
    if (p.parts_cap > 0) {
        cudaFree(p.w_part); cudaFree(p.loss_part); cudaFree(p.dx); cudaFree(p.xt);
    }
    memset(&p, 0, sizeof(p));
}

uint32_t cache_batch_count(uint32_t ns, uint32_t batch) { return (ns + batch - 1) / batch; }

void cache_batch_range(uint32_t ns, uint32_t nb, uint32_t b, uint32_t *o, uint32_t *n) {
    *o = b * (ns / nb) + std::min(b, ns % nb);
    *n = ns / nb + (b < ns % nb ? 1u : 0u);
}

cudaError_t cache_pick_and_target(const pm_cache_config &cfg, const CacheGrid &grid, uint32_t frame,
                                  const unsigned long long *frame_dev, const PScene &S, const MapView &surf,
                                  const MapView &vol, int k, float radius, const float4 *qa, const float4 *qd,
                                  uint32_t nq, const uint32_t *slist, uint32_t nsurf, TrainScratch &t,
                                  int sm_count, cudaStream_t stream) {
    const uint32_t ns = t.ns;
    cudaError_t e;
#define CT_TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)
    CT_TRY(cache_select(cfg.seed, frame, nq, slist, nsurf, ns, cfg.surface_fraction, t.sel, stream, frame_dev));
    CT_TRY(cache_sample_keys(grid, qa, t.sel, ns, t.skey, t.sval, stream));
    uint32_t *ok_keys = nullptr, *ok_vals = nullptr;
    CT_TRY(radix_sort_pairs_u32(t.skey, t.sval, t.skey_tmp, t.sval_tmp, t.sn, ns, 0, 31, t.shist, stream, &ok_keys,
                                &ok_vals));
    CT_TRY(cache_pick_records(ok_vals, t.sel, qa, qd, ns, t.pqa, t.pqd, t.pord, stream));
    CT_TRY(cache_knn_values_runs(S, surf, vol, t.pqa, t.pqd, nullptr, t.pord, ns, kTargetRun, k, radius, false,
                                 t.pval, t.run_ctr, sm_count, stream));
    CT_TRY(cache_train_order(t.pqa, t.pqd, t.pval, ok_vals, t.sel, ns, cache_batch_count(ns, cfg.batch), t.tqa,
                             t.tqd, t.tgt, t.tsel, stream));
#undef CT_TRY
    return cudaSuccess;
}

namespace {

// The frame's training picks of the installed query list and their k-NN
// targets, in training order (cache_pick_and_target).
cudaError_t pick_and_target(PhysicalState *st, CacheState *c, cudaStream_t stream) {
    return cache_pick_and_target(c->cfg, c->grid, (uint32_t)c->frames, nullptr, st->dscene, view_of(st->map[0]),
                                 view_of(st->map[1]), st->cfg.k, st->cfg.radius, st->ql.qa, st->ql.qd, st->ql.nq,
                                 st->ql.slist, st->ql.nsurf, c->ts, c->sm_count, stream);
}

template <typename T>
cudaError_t dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, sizeof(T) * count);
}

void free_cache(CacheState *c) {
    if (!c) return;
    cache_net_free(c->p);
    train_scratch_free(c->ts);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->tev0) cudaEventDestroy(c->tev0);
    delete c;
}

// Builds the query list of the installed camera unless it is current
// (force: always) and points the cache's grid box at the scene.
pm_status ensure_queries(pm_ctx *ctx, PhysicalState *st, CacheState *c, cudaStream_t stream,
                         bool force = false) {
    cudaError_t e = query_list_build(st, force, stream);
    if (e != cudaSuccess) return check_cuda(ctx, e, "query_list_build");
    c->stats.ms_queries = 0.0f;
    cache_grid_box(c->grid, st->scene);
    return PM_OK;
}

#define PM_TRY(x) do { e = (x); if (e != cudaSuccess) return check_cuda(ctx, e, #x); } while (0)

pm_status need_cache(pm_ctx *ctx, bool need_maps) {
    if (!ctx->cache) return fail(ctx, PM_ERR_STATE, "radiance cache not enabled");
    if (need_maps) {
        PhysicalState *st = ctx->phys;
        if (!st || !st->map[0].built || !st->map[1].built)
            return fail(ctx, PM_ERR_STATE, "photon maps not built");
    }
    return PM_OK;
}

}  // namespace

void cache_free(pm_ctx *ctx) {
    free_cache(ctx->cache);
    ctx->cache = nullptr;
}

}  // namespace pm

using namespace pm;

extern "C" {

void pm_cache_default_config(pm_cache_config *cfg) {
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->levels = 16;
    cfg->log2_table = 19;
    cfg->base_res = 16;
    cfg->max_res = 2048;
    cfg->train_samples = 1u << 20;
    cfg->batch = 1u << 17;  // 8 steps per frame, each filling every SM
    cfg->lr = 5e-2f;
    cfg->beta1 = 0.9f;
    cfg->beta2 = 0.99f;
    cfg->eps = 1e-15f;
    cfg->lr_min = 3e-4f;
    cfg->lr_half_life = 300.0f;
    cfg->loss_eps = 10.0f;
    cfg->surface_fraction = 0.5f;
    cfg->seed = 0x5EED0004ull;
}

pm_status pm_cache_enable(pm_ctx *ctx, const pm_cache_config *cfg_in) {
    if (!ctx) return PM_ERR_INVALID;
    pm_cache_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else pm_cache_default_config(&cfg);
    if (!cache_config_ok(cfg)) return fail(ctx, PM_ERR_INVALID, "invalid radiance-cache configuration");
    DeviceGuard g(ctx->device);
    cache_free(ctx);
    CacheState *c = new CacheState();
    ctx->cache = c;
    c->cfg = cfg;
    memset(&c->stats, 0, sizeof(c->stats));
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
    CacheGrid &gr = c->grid;
    cache_grid_init(cfg, &gr);
    if (ctx->phys) cache_grid_box(gr, ctx->phys->scene);
    c->table_floats = cache_table_floats(cfg);
    cudaError_t e;
#define PM_TRY_FREE(x) do { e = (x); if (e != cudaSuccess) { cache_free(ctx); return check_cuda(ctx, e, #x); } } while (0)
    PM_TRY_FREE(cache_net_alloc(cfg, gr, cfg.seed, c->sm_count, &c->p));
    PM_TRY_FREE(train_scratch_alloc(cfg.train_samples, &c->ts));
    for (auto &ev : c->ev) PM_TRY_FREE(cudaEventCreate(&ev));
    PM_TRY_FREE(cudaEventCreate(&c->tev0));
    PM_TRY_FREE(cudaDeviceSynchronize());
#undef PM_TRY_FREE
    return PM_OK;
}

pm_status pm_cache_disable(pm_ctx *ctx) {
    if (!ctx) return PM_ERR_INVALID;
    DeviceGuard g(ctx->device);
    cudaDeviceSynchronize();
    cache_free(ctx);
    return PM_OK;
}

pm_status pm_cache_train(pm_ctx *ctx, int frames, cudaStream_t stream) {
    if (!ctx || frames < 0) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, true);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    PhysicalState *st = ctx->phys;
    CacheState *c = ctx->cache;
    s = ensure_queries(ctx, st, c, stream);
    if (s != PM_OK) return s;
    if (st->ql.nq == 0 || frames == 0) return PM_OK;
    cudaError_t e;
    const uint32_t ns = c->cfg.train_samples;
    const uint32_t nb = cache_batch_count(ns, c->cfg.batch);
    for (int f = 0; f < frames; ++f) {
        PM_TRY(cudaEventRecord(c->tev0, stream));
        PM_TRY(pick_and_target(st, c, stream));
        PM_TRY(cudaEventRecord(c->ev[5], stream));
        if (!(c->target_scale > 0.0f)) {
            float sum = 0.0f;
            PM_TRY(cudaMemsetAsync(c->ts.scale_sum, 0, sizeof(float), stream));
            PM_TRY(cache_value_sum(c->ts.tgt, ns, c->ts.scale_sum, stream));
            PM_TRY(cudaMemcpyAsync(&sum, c->ts.scale_sum, sizeof(float), cudaMemcpyDeviceToHost, stream));
            PM_TRY(cudaStreamSynchronize(stream));
            const float mean = sum / (float)ns;
            c->target_scale = mean > 0.0f && std::isfinite(mean) ? mean : 1.0f;
        }
        PM_TRY(cudaMemsetAsync(c->p.loss, 0, sizeof(float), stream));
        for (uint32_t b = 0; b < nb; ++b) {
            // batch b: slots [o, o + n) of the training order
            uint32_t o, n;
            cache_batch_range(ns, nb, b, &o, &n);
            PM_TRY(cache_backward(c->grid, c->p, st->dscene, c->ts.tqa + o, c->ts.tqd + o, nullptr, c->ts.tgt + o, n,
                                  1.0f / c->target_scale, 1.0f / (3.0f * (float)n), c->cfg.loss_eps,
                                  nullptr, nullptr, c->sm_count, stream));
            float lr = c->cfg.lr;
            if (c->cfg.lr_half_life > 0.0f)
                lr = c->cfg.lr_min + (c->cfg.lr - c->cfg.lr_min) *
                                         (float)std::exp2(-(double)c->steps / c->cfg.lr_half_life);
            ++c->steps;
            PM_TRY(cache_adam(c->grid, c->p, lr, c->cfg.beta1, c->cfg.beta2, c->cfg.eps,
                              (int)std::min<unsigned long long>(c->steps, 1u << 30), stream));
        }
        PM_TRY(cudaEventRecord(c->ev[6], stream));
        ++c->frames;
    }
    float loss = 0.0f;
    PM_TRY(cudaMemcpyAsync(&loss, c->p.loss, sizeof(float), cudaMemcpyDeviceToHost, stream));
    PM_TRY(cudaStreamSynchronize(stream));
    c->stats.loss = loss / (float)nb;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->tev0, c->ev[5]);
    c->stats.ms_targets = ms;
    cudaEventElapsedTime(&ms, c->ev[5], c->ev[6]);
    c->stats.ms_train = ms;
    c->trained = true;
    return PM_OK;
}

pm_status pm_render_cached(pm_ctx *ctx, float4 *radiance, uchar4 *rgba, int source,
                           cudaStream_t stream) {
    if (!ctx || source < 0 || source > 1) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, true);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    PhysicalState *st = ctx->phys;
    CacheState *c = ctx->cache;
    // the list is rebuilt on every render call, like pm_render's
    s = ensure_queries(ctx, st, c, stream, true);
    if (s != PM_OK) return s;
    cudaError_t e;
    const uint32_t npix = (uint32_t)st->cfg.width * (uint32_t)st->cfg.height;
    PM_TRY(cudaEventRecord(c->ev[2], stream));
    if (source == 0) {
        const float scale = c->target_scale > 0.0f ? c->target_scale : 1.0f;
        // list order: pixel blocks sample-major, neighbouring rays at similar depths
        PM_TRY(cache_infer(c->grid, c->p, st->dscene, st->ql.qa, st->ql.qd, nullptr, st->ql.nq, scale,
                           st->ql.val, c->sm_count, stream));
        PM_TRY(cudaEventRecord(c->ev[3], stream));
        PM_TRY(cache_composite(st->dscene, st->ql.off, st->ql.qa, st->ql.qd, st->ql.val, npix,
                               st->cfg.exposure, radiance, rgba, stream));
    } else {
        // the k-NN render through the list (pm_render's path): raw values,
        // then the exact composite
        PM_TRY(knn_values_raw(st, stream));
        PM_TRY(cudaEventRecord(c->ev[3], stream));
        PM_TRY(render_composite(st->dscene, st->ql.off, st->ql.qa, st->ql.qd, st->ql.val, npix,
                                st->cfg.exposure, radiance, rgba, stream));
    }
    PM_TRY(cudaEventRecord(c->ev[4], stream));
    st->ql.val_owner = 2;
    c->stats.queries = st->ql.nq;
    c->rendered = true;
    return PM_OK;
}

pm_status pm_cache_get_stats(pm_ctx *ctx, pm_cache_stats *out) {
    if (!ctx || !out) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, false);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    CacheState *c = ctx->cache;
    cudaError_t e;
    if (c->rendered) {
        PM_TRY(cudaEventSynchronize(c->ev[4]));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
        c->stats.ms_values = ms;
        cudaEventElapsedTime(&ms, c->ev[3], c->ev[4]);
        c->stats.ms_composite = ms;
    }
    int status = 0;
    PM_TRY(cudaMemcpy(&status, c->p.status, sizeof(int), cudaMemcpyDeviceToHost));
    c->stats.tc_status = status;
    c->stats.train_steps = c->steps;
    c->stats.train_frames = c->frames;
    c->stats.target_scale = c->target_scale;
    *out = c->stats;
    return PM_OK;
}

pm_status pm_cache_set_wait_limit(pm_ctx *ctx, int polls) {
    if (!ctx) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, false);
    if (s != PM_OK) return s;
    ctx->cache->p.wait_polls = polls < 0 ? kMbarSpin : (uint32_t)polls;
    return PM_OK;
}

pm_status pm_cache_clear_status(pm_ctx *ctx) {
    if (!ctx) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, false);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    cudaError_t e;
    PM_TRY(cudaDeviceSynchronize());
    PM_TRY(cudaMemset(ctx->cache->p.status, 0, sizeof(int)));
    return PM_OK;
}

pm_status pm_cache_get_params(pm_ctx *ctx, float *weights, float *table, int *res) {
    if (!ctx) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, false);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    CacheState *c = ctx->cache;
    cudaError_t e;
    PM_TRY(cudaDeviceSynchronize());
    if (weights) PM_TRY(cudaMemcpy(weights, c->p.w, sizeof(float) * kCacheWeights, cudaMemcpyDeviceToHost));
    if (table) PM_TRY(cudaMemcpy(table, c->p.table, sizeof(float) * c->table_floats, cudaMemcpyDeviceToHost));
    if (res)
        for (int l = 0; l < c->grid.levels; ++l) res[l] = c->grid.res[l];
    return PM_OK;
}

pm_status pm_cache_set_params(pm_ctx *ctx, const float *weights, const float *table) {
    if (!ctx) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, false);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    CacheState *c = ctx->cache;
    cudaError_t e;
    PM_TRY(cudaDeviceSynchronize());
    if (weights) {
        PM_TRY(cudaMemcpy(c->p.w, weights, sizeof(float) * kCacheWeights, cudaMemcpyHostToDevice));
        PM_TRY(cudaMemset(c->p.w_m, 0, sizeof(float) * kCacheWeights));
        PM_TRY(cudaMemset(c->p.w_v, 0, sizeof(float) * kCacheWeights));
        PM_TRY(cache_weight_image(c->p, 0));
    }
    if (table) {
        PM_TRY(cudaMemcpy(c->p.table, table, sizeof(float) * c->table_floats, cudaMemcpyHostToDevice));
        PM_TRY(cudaMemset(c->p.table_m, 0, sizeof(float) * c->table_floats));
        PM_TRY(cudaMemset(c->p.table_v, 0, sizeof(float) * c->table_floats));
        PM_TRY(cache_sync_half(c->grid, c->p, 0));
    }
    PM_TRY(cudaDeviceSynchronize());
    return PM_OK;
}

pm_status pm_cache_debug_step(pm_ctx *ctx, const float4 *qa, const float4 *qd, const float4 *target,
                              uint32_t n, float target_scale, float *x, float *y, float *loss,
                              float *w_grad, float *table_grad) {
    if (!ctx || (n && (!qa || !qd || !target)) || !(target_scale > 0.0f)) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, false);
    if (s != PM_OK) return s;
    if (!ctx->phys) return fail(ctx, PM_ERR_STATE, "pm_cache_debug_step before pm_set_scene");
    if (n > (1u << 20)) return fail(ctx, PM_ERR_LIMIT, "debug step above 2^20 samples");
    DeviceGuard g(ctx->device);
    CacheState *c = ctx->cache;
    PhysicalState *st = ctx->phys;
    cache_grid_box(c->grid, st->scene);
    cudaError_t e;
    float4 *dqa = nullptr, *dqd = nullptr, *dt = nullptr;
    float *dx = nullptr, *dy = nullptr, *tg = nullptr;
    float4 *ddx = nullptr;
    uint4 *dxt = nullptr;
    CacheParams dp = c->p;
    std::string where;
#define PM_DBG(x) do { e = (x); if (e != cudaSuccess) { where = #x; goto done; } } while (0)
    PM_DBG(cudaDeviceSynchronize());
    PM_DBG(dalloc(&dqa, n));
    PM_DBG(dalloc(&dqd, n));
    PM_DBG(dalloc(&dt, n));
    PM_DBG(dalloc(&dx, (size_t)n * 64));
    PM_DBG(dalloc(&dy, (size_t)n * 4));
    if (n) {
        PM_DBG(cudaMemcpy(dqa, qa, sizeof(float4) * n, cudaMemcpyHostToDevice));
        PM_DBG(cudaMemcpy(dqd, qd, sizeof(float4) * n, cudaMemcpyHostToDevice));
        PM_DBG(cudaMemcpy(dt, target, sizeof(float4) * n, cudaMemcpyHostToDevice));
    }
    PM_DBG(cudaMemset(c->p.w_grad, 0, sizeof(float) * kCacheWeights));
    PM_DBG(cudaMemset(c->p.table_grad, 0, sizeof(long long) * c->table_floats));
    PM_DBG(cudaMemset(c->p.loss, 0, sizeof(float)));
    // the feature-gradient rows of n samples (n may exceed the batch)
    PM_DBG(dalloc(&ddx, (size_t)(n + 127) / 128 * 128 * 8));
    PM_DBG(dalloc(&dxt, (size_t)(n + 127) / 128 * 128 * 8));
    dp.dx = ddx;
    dp.xt = dxt;
    dp.dx_cap = (n + 127) / 128 * 128;
    PM_DBG(cache_backward(c->grid, dp, st->dscene, dqa, dqd, nullptr, dt, n, 1.0f / target_scale,
                          n ? 1.0f / (3.0f * (float)n) : 0.0f, c->cfg.loss_eps, dx, dy, c->sm_count,
                          0));
    PM_DBG(cudaDeviceSynchronize());
    if (x && n) PM_DBG(cudaMemcpy(x, dx, sizeof(float) * 64 * n, cudaMemcpyDeviceToHost));
    if (y && n) PM_DBG(cudaMemcpy(y, dy, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost));
    if (loss) PM_DBG(cudaMemcpy(loss, c->p.loss, sizeof(float), cudaMemcpyDeviceToHost));
    if (w_grad) PM_DBG(cudaMemcpy(w_grad, c->p.w_grad, sizeof(float) * kCacheWeights, cudaMemcpyDeviceToHost));
    if (table_grad) {
        // the fixed-point sums converted to floats in a scratch buffer
        PM_DBG(dalloc(&tg, c->table_floats));
        PM_DBG(cache_table_grad_float(c->grid, c->p, tg, 0));
        PM_DBG(cudaMemcpy(table_grad, tg, sizeof(float) * c->table_floats, cudaMemcpyDeviceToHost));
    }
    PM_DBG(cudaMemset(c->p.w_grad, 0, sizeof(float) * kCacheWeights));
    PM_DBG(cudaMemset(c->p.table_grad, 0, sizeof(long long) * c->table_floats));
done:
#undef PM_DBG
    cudaFree(dqa); cudaFree(dqd); cudaFree(dt); cudaFree(dx); cudaFree(dy); cudaFree(tg); cudaFree(ddx); cudaFree(dxt);
    if (e != cudaSuccess) return check_cuda(ctx, e, where.c_str());
    return PM_OK;
}

pm_status pm_cache_get_queries(pm_ctx *ctx, float4 *qa, float4 *qd, uint32_t cap, uint32_t *count) {
    if (!ctx) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, true);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    PhysicalState *st = ctx->phys;
    CacheState *c = ctx->cache;
    s = ensure_queries(ctx, st, c, 0);
    if (s != PM_OK) return s;
    if (count) *count = st->ql.nq;
    const uint32_t n = std::min(cap, st->ql.nq);
    cudaError_t e;
    PM_TRY(cudaDeviceSynchronize());
    if (n && qa) PM_TRY(cudaMemcpy(qa, st->ql.qa, sizeof(float4) * n, cudaMemcpyDeviceToHost));
    if (n && qd) PM_TRY(cudaMemcpy(qd, st->ql.qd, sizeof(float4) * n, cudaMemcpyDeviceToHost));
    return PM_OK;
}

pm_status pm_cache_debug_targets(pm_ctx *ctx, float4 *targets, uint32_t *query) {
    if (!ctx) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, true);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    PhysicalState *st = ctx->phys;
    CacheState *c = ctx->cache;
    s = ensure_queries(ctx, st, c, 0);
    if (s != PM_OK) return s;
    const uint32_t ns = c->cfg.train_samples;
    cudaError_t e;
    PM_TRY(pick_and_target(st, c, 0));
    PM_TRY(cudaDeviceSynchronize());
    if (targets) PM_TRY(cudaMemcpy(targets, c->ts.tgt, sizeof(float4) * ns, cudaMemcpyDeviceToHost));
    if (query) PM_TRY(cudaMemcpy(query, c->ts.tsel, sizeof(uint32_t) * ns, cudaMemcpyDeviceToHost));
    return PM_OK;
}

pm_status pm_cache_get_values(pm_ctx *ctx, float4 *val, uint32_t cap, uint32_t *count) {
    if (!ctx) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, false);
    if (s != PM_OK) return s;
    CacheState *c = ctx->cache;
    PhysicalState *st = ctx->phys;
    if (!c->rendered || st->ql.val_owner != 2)
        return fail(ctx, PM_ERR_STATE, "pm_cache_get_values without a pm_render_cached since the last render");
    DeviceGuard g(ctx->device);
    if (count) *count = st->ql.nq;
    const uint32_t n = std::min(cap, st->ql.nq);
    cudaError_t e;
    PM_TRY(cudaDeviceSynchronize());
    if (n && val) PM_TRY(cudaMemcpy(val, st->ql.val, sizeof(float4) * n, cudaMemcpyDeviceToHost));
    return PM_OK;
}

}  // extern "C"

namespace {

const char kCacheMagic[] = "{\"format\": \"pm-radiance-cache\", \"version\": 1";

}  // namespace

extern "C" {

// File = one JSON header line, then fp32 arrays: weights, their two Adam
// moments, the table, its two Adam moments.
pm_status pm_cache_save(pm_ctx *ctx, const char *path) {
    if (!ctx || !path) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, false);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    CacheState *c = ctx->cache;
    const size_t nw = kCacheWeights, nt = c->table_floats;
    std::vector<float> buf(3 * nw + 3 * nt);
    cudaError_t e;
    PM_TRY(cudaDeviceSynchronize());
    const float *src[6] = {c->p.w, c->p.w_m, c->p.w_v, c->p.table, c->p.table_m, c->p.table_v};
    size_t at = 0;
    for (int i = 0; i < 6; ++i) {
        const size_t len = i < 3 ? nw : nt;
        PM_TRY(cudaMemcpy(buf.data() + at, src[i], sizeof(float) * len, cudaMemcpyDeviceToHost));
        at += len;
    }
    FILE *f = fopen(path, "wb");
    if (!f) return fail(ctx, PM_ERR_INVALID, std::string("cannot open ") + path);
    fprintf(f,
            "%s, \"levels\": %d, \"log2_table\": %d, \"base_res\": %d, \"max_res\": %d, "
            "\"target_scale\": %.9g, \"steps\": %llu, \"frames\": %llu, \"weights\": %zu, "
            "\"table_floats\": %zu, \"layout\": \"fp32 weights, m, v; table, m, v\"}\n",
            kCacheMagic, c->cfg.levels, c->cfg.log2_table, c->cfg.base_res, c->cfg.max_res,
            c->target_scale, c->steps, c->frames, nw, nt);
    bool ok = fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
    ok = (fclose(f) == 0) && ok;
    return ok ? PM_OK : fail(ctx, PM_ERR_INVALID, "short write");
}

pm_status pm_cache_load(pm_ctx *ctx, const char *path) {
    if (!ctx || !path) return PM_ERR_INVALID;
    pm_status s = need_cache(ctx, false);
    if (s != PM_OK) return s;
    DeviceGuard g(ctx->device);
    CacheState *c = ctx->cache;
    FILE *f = fopen(path, "rb");
    if (!f) return fail(ctx, PM_ERR_INVALID, std::string("cannot open ") + path);
    char line[1024];
    if (!fgets(line, sizeof(line), f) || strncmp(line, kCacheMagic, strlen(kCacheMagic)) != 0) {
        fclose(f);
        return fail(ctx, PM_ERR_INVALID, "not a radiance-cache file");
    }
    int levels = -1, log2t = -1, base = -1, maxr = -1;
    float scale = 0.0f;
    unsigned long long steps = 0, frames = 0;
    const char *q;
    if ((q = strstr(line, "\"levels\": "))) sscanf(q + 10, "%d", &levels);
    if ((q = strstr(line, "\"log2_table\": "))) sscanf(q + 14, "%d", &log2t);
    if ((q = strstr(line, "\"base_res\": "))) sscanf(q + 12, "%d", &base);
    if ((q = strstr(line, "\"max_res\": "))) sscanf(q + 11, "%d", &maxr);
    if ((q = strstr(line, "\"target_scale\": "))) sscanf(q + 16, "%f", &scale);
    if ((q = strstr(line, "\"steps\": "))) sscanf(q + 9, "%llu", &steps);
    if ((q = strstr(line, "\"frames\": "))) sscanf(q + 10, "%llu", &frames);
    if (levels != c->cfg.levels || log2t != c->cfg.log2_table || base != c->cfg.base_res ||
        maxr != c->cfg.max_res) {
        fclose(f);
        return fail(ctx, PM_ERR_INVALID, "radiance-cache file has another grid configuration");
    }
    const size_t nw = kCacheWeights, nt = c->table_floats;
    std::vector<float> buf(3 * nw + 3 * nt);
    const bool ok = fread(buf.data(), sizeof(float), buf.size(), f) == buf.size();
    fclose(f);
    if (!ok) return fail(ctx, PM_ERR_INVALID, "truncated radiance-cache file");
    cudaError_t e;
    PM_TRY(cudaDeviceSynchronize());
    float *dst[6] = {c->p.w, c->p.w_m, c->p.w_v, c->p.table, c->p.table_m, c->p.table_v};
    size_t at = 0;
    for (int i = 0; i < 6; ++i) {
        const size_t len = i < 3 ? nw : nt;
        PM_TRY(cudaMemcpy(dst[i], buf.data() + at, sizeof(float) * len, cudaMemcpyHostToDevice));
        at += len;
    }
    PM_TRY(cudaMemset(c->p.w_grad, 0, sizeof(float) * nw));
    PM_TRY(cudaMemset(c->p.table_grad, 0, sizeof(long long) * nt));
    PM_TRY(cache_sync_half(c->grid, c->p, 0));
    PM_TRY(cache_weight_image(c->p, 0));
    PM_TRY(cudaDeviceSynchronize());
    c->target_scale = scale;
    c->steps = steps;
    c->frames = frames;
    return PM_OK;
}

#undef PM_TRY
}  // extern "C"
