// physical.cu -- the physically based mode behind the pm_* C ABI: scene
// installation, photon emission, kd-tree build, render and queries.
#include "cache.cuh"
#include "gather.cuh"
#include "kdtree.cuh"
#include "launch_count.cuh"
#include "phys_state.cuh"
#include "pm_ctx.cuh"
#include "radix_sort.cuh"
#include "scene.cuh"
#include "trace.cuh"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <vector>

namespace pm {

namespace {

template <typename T>
cudaError_t dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, sizeof(T) * count);
}

void free_state(PhysicalState *st) {
    if (!st) return;
    query_list_free(st->ql);
    cudaFree(st->het);
    for (auto &p : st->cnt) cudaFree(p);
    for (auto &p : st->off) cudaFree(p);
    cudaFree(st->scan_tmp);
    cudaFree(st->need_list); cudaFree(st->need_tile); cudaFree(st->need_tile_off);
    cudaFree(st->words);
    for (auto &m : st->map) {
        cudaFree(m.pos); cudaFree(m.pow); cudaFree(m.tpos); cudaFree(m.tpow); cudaFree(m.tdir);
        cudaFree(m.lo); cudaFree(m.hi);
    }
    cudaFree(st->keys); cudaFree(st->keys_tmp); cudaFree(st->vals); cudaFree(st->vals_tmp);
    cudaFree(st->hist);
    cudaFree(st->gctr);
    for (auto &e : st->ev)
        if (e) cudaEventDestroy(e);
    delete st;
}


}  // namespace

uint64_t next_scene_gen() {
    static std::atomic<uint64_t> gen{0};
    return ++gen;
}

void physical_free(pm_ctx *ctx) {
    free_state(ctx->phys);
    ctx->phys = nullptr;
}

}  // namespace pm

using namespace pm;

extern "C" {

pm_status pm_set_scene(pm_ctx *ctx, const pm_scene *scene, const pm_config *cfg) {
    if (!ctx || !scene || !cfg) return PM_ERR_INVALID;
    std::string why;
    pm_status s = validate(*scene, *cfg, &why);
    if (s != PM_OK) return fail(ctx, s, why);
    DeviceGuard g(ctx->device);
    physical_free(ctx);
    PhysicalState *st = new PhysicalState();
    ctx->phys = st;
    st->scene = *scene;
    st->cfg = *cfg;
    memset(&st->stats, 0, sizeof(st->stats));
    cudaDeviceGetAttribute(&st->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
    const uint32_t tmax = std::max(cfg->surface_photons, cfg->volume_photons);
    uint64_t cap = cfg->max_paths ? cfg->max_paths : (uint64_t)tmax * 16u;
    cap = std::max<uint64_t>(cap, 1024);
    if (cap > 0xFFFFFFFFull) return fail(ctx, PM_ERR_LIMIT, "path cap above 2^32");
    if (tmax > (1u << 28)) return fail(ctx, PM_ERR_LIMIT, "map target above 2^28 records");
    st->path_cap = (uint32_t)cap;
    st->mb = cfg->max_bounces;
    cudaError_t e = cudaSuccess;
#define PM_TRY(x) do { e = (x); if (e != cudaSuccess) { physical_free(ctx); return check_cuda(ctx, e, #x); } } while (0)
    for (auto &p : st->cnt) PM_TRY(dalloc(&p, st->path_cap));
    for (auto &p : st->off) PM_TRY(dalloc(&p, st->path_cap));
    PM_TRY(dalloc(&st->scan_tmp, scan_tile_count(st->path_cap) + 1));
    PM_TRY(dalloc(&st->need_list, st->path_cap));
    PM_TRY(dalloc(&st->need_tile, needed_tiles(st->path_cap)));
    PM_TRY(dalloc(&st->need_tile_off, needed_tiles(st->path_cap)));
    PM_TRY(dalloc(&st->words, 16));
    PM_TRY(cudaMemset(st->words, 0, 16 * sizeof(uint32_t)));
    const uint32_t targets[2] = {cfg->surface_photons, cfg->volume_photons};
    const int leaf_shift = cfg->leaf_size == 128 ? 2 : (cfg->leaf_size == 64 ? 1 : 0);
    for (int m = 0; m < 2; ++m) {
        auto &mp = st->map[m];
        mp.leaf_shift = leaf_shift;
        mp.cap = targets[m];
        PM_TRY(dalloc(&mp.pos, mp.cap));
        PM_TRY(dalloc(&mp.pow, mp.cap));
        PM_TRY(dalloc(&mp.tpos, mp.cap));
        PM_TRY(dalloc(&mp.tpow, mp.cap));
        PM_TRY(dalloc(&mp.tdir, mp.cap));
        PM_TRY(dalloc(&mp.lo, tree_nodes(mp.cap)));
        PM_TRY(dalloc(&mp.hi, tree_nodes(mp.cap)));
    }
    PM_TRY(dalloc(&st->keys, tmax));
    PM_TRY(dalloc(&st->keys_tmp, tmax));
    PM_TRY(dalloc(&st->vals, tmax));
    PM_TRY(dalloc(&st->vals_tmp, tmax));
    PM_TRY(dalloc(&st->hist, radix_sort_hist_words(std::max<uint32_t>(tmax, 1))));
    st->sort_cap = tmax;
    PM_TRY(dalloc(&st->gctr, 2));
    if (scene->het_res > 0) {
        const size_t nv = (size_t)scene->het_res * scene->het_res * scene->het_res;
        PM_TRY(dalloc(&st->het, nv));
        PM_TRY(make_noise_grid(st->het, scene->het_res, cfg->seed ^ 0x6E6F697365ull, scene->het_min,
                               scene->het_max, 0));
    }
    for (auto &ev : st->ev) PM_TRY(cudaEventCreate(&ev));
    PM_TRY(cudaDeviceSynchronize());
#undef PM_TRY
    st->dscene = to_device_scene(*scene, st->het);
    st->gen = next_scene_gen();
    return PM_OK;
}

pm_status pm_update_scene(pm_ctx *ctx, const pm_scene *scene) {
    if (!ctx || !scene) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st) return fail(ctx, PM_ERR_STATE, "pm_update_scene before pm_set_scene");
    std::string why;
    pm_status s = validate(*scene, st->cfg, &why);
    if (s != PM_OK) return fail(ctx, s, why);
    if (scene->het_res != st->scene.het_res)
        return fail(ctx, PM_ERR_INVALID, "het_res differs from the installed scene");
    DeviceGuard g(ctx->device);
    const bool regen = scene->het_res > 0 &&
                       (scene->het_min != st->scene.het_min || scene->het_max != st->scene.het_max);
    st->scene = *scene;
    if (regen) {
        cudaError_t e = make_noise_grid(st->het, scene->het_res, st->cfg.seed ^ 0x6E6F697365ull,
                                        scene->het_min, scene->het_max, 0);
        if (e != cudaSuccess) return check_cuda(ctx, e, "make_noise_grid");
    }
    st->dscene = to_device_scene(*scene, st->het);
    st->gen = next_scene_gen();
    return PM_OK;
}

pm_status pm_emit(pm_ctx *ctx, cudaStream_t stream) {
    if (!ctx) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st) return fail(ctx, PM_ERR_STATE, "pm_emit before pm_set_scene");
    DeviceGuard g(ctx->device);
    cudaError_t e;
#define PM_TRY(x) do { e = (x); if (e != cudaSuccess) return check_cuda(ctx, e, #x); } while (0)
    PM_TRY(cudaEventRecord(st->ev[0], stream));
    PM_TRY(cudaMemsetAsync(st->words, 0, 16 * sizeof(uint32_t), stream));
    TraceParams P;
    memset(&P, 0, sizeof(P));
    P.seed = st->cfg.seed;
    P.scene_id = st->cfg.scene_id;
    P.max_bounces = st->mb;
    P.rr = st->cfg.rr_survival;
    P.target_s = st->cfg.surface_photons;
    P.target_v = st->cfg.volume_photons;
    P.path_cap = st->path_cap;
    P.path_counter = st->words + 0;
    P.stored_s = st->words + 1;
    P.stored_v = st->words + 2;
    P.cnt_s = st->cnt[0];
    P.cnt_v = st->cnt[1];
    // counting pass: every issued path writes its two counts
    PM_TRY(trace_photons(st->dscene, P, st->sm_count, stream));
    uint32_t counter = 0;
    PM_TRY(cudaMemcpyAsync(&counter, st->words, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    PM_TRY(cudaStreamSynchronize(stream));
    const uint32_t issued = std::min(counter, st->path_cap);
    for (int m = 0; m < 2; ++m) {
        const uint32_t target = m == 0 ? st->cfg.surface_photons : st->cfg.volume_photons;
        PM_TRY(map_extent(issued, st->cnt[m], st->off[m], st->words + 3, st->scan_tmp, target,
                          st->words + 4 + 2 * m, stream));
    }
    // writing pass over the paths the maps need, taken from their list
    PM_TRY(needed_paths(issued, st->cnt[0], st->cnt[1], st->words + 4, st->words + 6, st->need_tile,
                        st->need_tile_off, st->scan_tmp, st->need_list, st->words + 8, stream));
    PM_TRY(cudaMemsetAsync(st->words, 0, sizeof(uint32_t), stream));
    P.store = 1;
    P.list = st->need_list;
    P.list_n = st->words + 8;
    P.off_s = st->off[0];
    P.off_v = st->off[1];
    P.ext_s = st->words + 4;
    P.ext_v = st->words + 6;
    P.power = st->scene.light_power;
    P.spos = st->map[0].pos; P.spow = st->map[0].pow;
    P.vpos = st->map[1].pos; P.vpow = st->map[1].pow;
    PM_TRY(trace_photons(st->dscene, P, st->sm_count, stream));
    uint32_t ext[4];
    PM_TRY(cudaMemcpyAsync(ext, st->words + 4, sizeof(ext), cudaMemcpyDeviceToHost, stream));
    PM_TRY(cudaEventRecord(st->ev[1], stream));
    PM_TRY(cudaStreamSynchronize(stream));
    for (int m = 0; m < 2; ++m) {
        st->map[m].n = ext[2 * m];
        st->map[m].paths = ext[2 * m + 1];
        st->map[m].built = false;
        st->map[m].depth = tree_depth(ext[2 * m], st->map[m].leaf_shift);
        st->stats.map_size[m] = ext[2 * m];
        st->stats.map_paths[m] = ext[2 * m + 1];
    }
    st->stats.paths_traced = issued;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, st->ev[0], st->ev[1]);
    st->stats.ms_emit = ms;
    st->emitted = true;
    return PM_OK;
}

pm_status pm_build(pm_ctx *ctx, cudaStream_t stream) {
    if (!ctx) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st || !st->emitted) return fail(ctx, PM_ERR_STATE, "pm_build before pm_emit");
    DeviceGuard g(ctx->device);
    cudaError_t e;
    PM_TRY(cudaEventRecord(st->ev[2], stream));
    for (int m = 0; m < 2; ++m) {
        auto &mp = st->map[m];
        if (mp.n == 0) { mp.built = true; continue; }
        if (mp.depth > 29) return fail(ctx, PM_ERR_LIMIT, "photon map too large for the tree");
        KdBuildArgs a;
        a.box_dev = nullptr;
        a.n = mp.n;
        a.n_dev = st->words + 4 + 2 * m;
        a.lo = make_float3(st->scene.box_min[0], st->scene.box_min[1], st->scene.box_min[2]);
        a.hi = make_float3(st->scene.box_max[0], st->scene.box_max[1], st->scene.box_max[2]);
        a.pos_in = mp.pos;
        a.pow_in = mp.pow;
        a.pos_out = mp.tpos;
        a.pow_out = mp.tpow;
        a.dir_out = mp.tdir;
        a.node_lo = mp.lo;
        a.node_hi = mp.hi;
        a.keys = st->keys; a.keys_tmp = st->keys_tmp;
        a.vals = st->vals; a.vals_tmp = st->vals_tmp;
        a.hist = st->hist;
        a.order_out = nullptr;
        a.leaf_shift = mp.leaf_shift;
        PM_TRY(build_tree(a, stream));
        mp.built = true;
    }
    PM_TRY(cudaEventRecord(st->ev[3], stream));
    PM_TRY(cudaEventSynchronize(st->ev[3]));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, st->ev[2], st->ev[3]);
    st->stats.ms_build = ms;
    return PM_OK;
}

pm_status pm_render(pm_ctx *ctx, float4 *radiance, uchar4 *rgba, cudaStream_t stream) {
    if (!ctx) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st || !st->map[0].built || !st->map[1].built)
        return fail(ctx, PM_ERR_STATE, "pm_render before pm_build");
    DeviceGuard g(ctx->device);
    cudaError_t e;
    // The frame as its list of radiance queries (rebuilt on every call),
    // estimated in spatial order by warm-started runs, then summed per pixel
    // in march order with the single-kernel render's arithmetic: the image
    // is bit-identical to render_frame's.
    PM_TRY(cudaEventRecord(st->ev[4], stream));
    PM_TRY(query_list_build(st, true, stream));
    PM_TRY(query_list_sort(st, stream));
    PM_TRY(cudaEventRecord(st->ev[6], stream));
    PM_TRY(knn_values_raw(st, stream));
    PM_TRY(cudaEventRecord(st->ev[7], stream));
    const uint32_t npix = (uint32_t)st->cfg.width * (uint32_t)st->cfg.height;
    PM_TRY(render_composite(st->dscene, st->ql.off, st->ql.qa, st->ql.qd, st->ql.val, npix,
                            st->cfg.exposure, radiance, rgba, stream));
    PM_TRY(cudaEventRecord(st->ev[5], stream));
    st->ql.val_owner = 1;
    // one gather per query; the counts are known on the host
    st->host_gathers[0] = st->ql.nsurf;
    st->host_gathers[1] = (uint64_t)st->ql.nq - st->ql.nsurf;
    st->gathers_on_host = true;
    st->rendered = true;
    return PM_OK;
}

pm_status pm_render_single_kernel(pm_ctx *ctx, float4 *radiance, uchar4 *rgba, cudaStream_t stream) {
    if (!ctx) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st || !st->map[0].built || !st->map[1].built)
        return fail(ctx, PM_ERR_STATE, "pm_render_single_kernel before pm_build");
    DeviceGuard g(ctx->device);
    cudaError_t e;
    RenderParams R = render_params(st);
    R.counters = st->gctr;
    PM_TRY(cudaMemsetAsync(st->gctr, 0, 2 * sizeof(unsigned long long), stream));
    PM_TRY(cudaEventRecord(st->ev[4], stream));
    PM_TRY(render_frame(st->dscene, view_of(st->map[0]), view_of(st->map[1]), R, radiance, rgba, stream));
    PM_TRY(cudaEventRecord(st->ev[5], stream));
    st->gathers_on_host = false;
    st->rendered = true;
    return PM_OK;
}

pm_status pm_knn(pm_ctx *ctx, int map, const float4 *queries, uint32_t nq, int k, float radius,
                 uint32_t *idx_out, float *d2_out, cudaStream_t stream) {
    if (!ctx || map < 0 || map > 1 || k < 1 || k > 128 || !(radius > 0.0f)) return PM_ERR_INVALID;
    if (nq && (!queries || !idx_out || !d2_out)) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st || !st->map[map].built) return fail(ctx, PM_ERR_STATE, "pm_knn before pm_build");
    DeviceGuard g(ctx->device);
    cudaError_t e;
    PM_TRY(knn_query(view_of(st->map[map]), queries, nq, k, radius, idx_out, d2_out, stream));
    return PM_OK;
}

pm_status pm_radius_gather(pm_ctx *ctx, int map, const float4 *points, const float4 *normals,
                           uint32_t nq, float sq_radius, float exposure, float4 *out,
                           cudaStream_t stream) {
    if (!ctx || map < 0 || map > 1 || !(sq_radius > 0.0f) || !(exposure != 0.0f)) return PM_ERR_INVALID;
    if (nq && (!points || !normals || !out)) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st || !st->map[map].built) return fail(ctx, PM_ERR_STATE, "pm_radius_gather before pm_build");
    DeviceGuard g(ctx->device);
    cudaError_t e;
    PM_TRY(radius_gather(view_of(st->map[map]), points, normals, nq, sq_radius, exposure, out, stream));
    return PM_OK;
}

pm_status pm_get_photons_soa(pm_ctx *ctx, int map, float4 *pos, float4 *pw, uint32_t cap,
                             uint32_t *count) {
    if (!ctx || map < 0 || map > 1) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st || !st->emitted) return fail(ctx, PM_ERR_STATE, "no photon map yet");
    DeviceGuard g(ctx->device);
    const auto &mp = st->map[map];
    if (count) *count = mp.n;
    uint32_t n = std::min(cap, mp.n);
    cudaError_t e;
    PM_TRY(cudaDeviceSynchronize());
    if (n && pos) PM_TRY(cudaMemcpy(pos, mp.pos, sizeof(float4) * n, cudaMemcpyDeviceToHost));
    if (n && pw) PM_TRY(cudaMemcpy(pw, mp.pow, sizeof(float4) * n, cudaMemcpyDeviceToHost));
    return PM_OK;
}

pm_status pm_get_photons(pm_ctx *ctx, int map, pm_photon_record *out, uint32_t cap,
                         uint32_t *count) {
    if (!ctx || map < 0 || map > 1) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st || !st->emitted) return fail(ctx, PM_ERR_STATE, "no photon map yet");
    uint32_t n = std::min(cap, st->map[map].n);
    std::vector<float4> pos(n), pw(n);
    pm_status s = pm_get_photons_soa(ctx, map, pos.data(), pw.data(), n, count);
    if (s != PM_OK) return s;
    for (uint32_t i = 0; i < n && out; ++i) {
        uint32_t bits;
        memcpy(&bits, &pw[i].w, 4);
        v3 d = oct_decode(bits);
        out[i].location[0] = pos[i].x; out[i].location[1] = pos[i].y; out[i].location[2] = pos[i].z;
        out[i].direction[0] = d.x; out[i].direction[1] = d.y; out[i].direction[2] = d.z;
        out[i].energy[0] = pw[i].x; out[i].energy[1] = pw[i].y; out[i].energy[2] = pw[i].z;
    }
    return PM_OK;
}

pm_status pm_get_gather_stats(pm_ctx *ctx, uint64_t *out, int n) {
    if (!ctx || !out || n < 0 || n > kGatherStats) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st || !st->ql.gather_stats || !st->gathers_on_host)
        return fail(ctx, PM_ERR_STATE, "pm_get_gather_stats before a pm_render");
    DeviceGuard g(ctx->device);
    cudaError_t e;
    unsigned long long c[kGatherStats];
    PM_TRY(cudaEventSynchronize(st->ev[5]));
    PM_TRY(cudaMemcpy(c, st->ql.gather_stats, sizeof(c), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) out[i] = c[i];
    return PM_OK;
}

pm_status pm_get_stats(pm_ctx *ctx, pm_frame_stats *out) {
    if (!ctx || !out) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st) return fail(ctx, PM_ERR_STATE, "no scene");
    DeviceGuard g(ctx->device);
    cudaError_t e;
    if (st->rendered) {
        PM_TRY(cudaEventSynchronize(st->ev[5]));
        float ms = 0.f;
        PM_TRY(cudaEventElapsedTime(&ms, st->ev[4], st->ev[5]));
        st->stats.ms_render = ms;
        if (st->gathers_on_host) {
            st->stats.surface_gathers = st->host_gathers[0];
            st->stats.volume_gathers = st->host_gathers[1];
            PM_TRY(cudaEventElapsedTime(&ms, st->ev[6], st->ev[7]));
            st->stats.ms_gather = ms;
        } else {
            unsigned long long c[2] = {0, 0};
            PM_TRY(cudaMemcpy(c, st->gctr, sizeof(c), cudaMemcpyDeviceToHost));
            st->stats.surface_gathers = c[0];
            st->stats.volume_gathers = c[1];
            st->stats.ms_gather = ms;
        }
    }
    *out = st->stats;
    return PM_OK;
}

pm_status pm_set_photons(pm_ctx *ctx, int map, const float4 *pos, const float4 *pw, uint32_t n) {
    if (!ctx || map < 0 || map > 1 || (n && (!pos || !pw))) return PM_ERR_INVALID;
    PhysicalState *st = ctx->phys;
    if (!st) return fail(ctx, PM_ERR_STATE, "pm_set_photons before pm_set_scene");
    if (n > (1u << 28)) return fail(ctx, PM_ERR_LIMIT, "map above 2^28 records");
    DeviceGuard g(ctx->device);
    cudaError_t e;
    auto &mp = st->map[map];
    PM_TRY(cudaDeviceSynchronize());
    if (n > mp.cap) {
        cudaFree(mp.pos); cudaFree(mp.pow); cudaFree(mp.tpos); cudaFree(mp.tpow); cudaFree(mp.tdir);
        cudaFree(mp.lo); cudaFree(mp.hi);
        const int ls = mp.leaf_shift;
        mp = PhysicalState::Map();
        mp.leaf_shift = ls;
        PM_TRY(dalloc(&mp.pos, n)); PM_TRY(dalloc(&mp.pow, n));
        PM_TRY(dalloc(&mp.tpos, n)); PM_TRY(dalloc(&mp.tpow, n)); PM_TRY(dalloc(&mp.tdir, n));
        PM_TRY(dalloc(&mp.lo, tree_nodes(n))); PM_TRY(dalloc(&mp.hi, tree_nodes(n)));
        mp.cap = n;
        if (n > st->sort_cap) {
            cudaFree(st->keys); cudaFree(st->keys_tmp); cudaFree(st->vals); cudaFree(st->vals_tmp);
            cudaFree(st->hist);
            PM_TRY(dalloc(&st->keys, n)); PM_TRY(dalloc(&st->keys_tmp, n));
            PM_TRY(dalloc(&st->vals, n)); PM_TRY(dalloc(&st->vals_tmp, n));
            PM_TRY(dalloc(&st->hist, radix_sort_hist_words(n)));
            st->sort_cap = n;
        }
    }
    std::vector<float4> tmp(pos, pos + n);
    for (uint32_t i = 0; i < n; ++i) memcpy(&tmp[i].w, &i, 4);
    if (n) {
        PM_TRY(cudaMemcpy(mp.pos, tmp.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
        PM_TRY(cudaMemcpy(mp.pow, pw, sizeof(float4) * n, cudaMemcpyHostToDevice));
    }
    PM_TRY(cudaMemcpy(st->words + 4 + 2 * map, &n, sizeof(uint32_t), cudaMemcpyHostToDevice));
    mp.n = n;
    mp.paths = 0;
    mp.built = false;
    mp.depth = tree_depth(n, mp.leaf_shift);
    st->stats.map_size[map] = n;
    st->stats.map_paths[map] = 0;
    st->emitted = true;
    return PM_OK;
}

unsigned long long pm_kernel_launches(void) { return launch_counter().load(); }

size_t pm_abi_struct_size(int which) {
    switch (which) {
        case 0: return sizeof(pm_scene);
        case 1: return sizeof(pm_config);
        case 2: return sizeof(pm_photon_record);
        case 3: return sizeof(pm_frame_stats);
        case 4: return sizeof(pm_cache_config);
        case 5: return sizeof(pm_cache_stats);
    }
    return 0;
}

#undef PM_TRY
}  // extern "C"
