// batch.cu -- many independent scenes per frame behind the pm_batch_* C ABI:
// persistent multi-scene trace and render launches, the kd-trees of every
// map in shared launches, CUDA-graph capture of the whole frame, and the
// autotuner of the search knobs.
//
// Frame (all on the caller's stream, no host round trip):
//   1. zero the per-scene words, path counts and gather counters
//   2. counting pass: one persistent launch over every scene's paths
//   3. every map's record extent (records, paths): one segmented scan of
//      all maps' path counts (each map a tile-aligned segment over its
//      path cap, zero beyond the issued paths), then one search per map
//   4. writing pass: one persistent launch
//   5. the kd-trees of every map in shared launches (KdMulti): records past
//      each map's size set to infinity, the radix-sorted levels of all
//      maps, then their subtree finishes, permutations and boxes; each tree
//      is built over its map's capacity (so every launch size is a host
//      constant)
//   6. the render: the scenes in per-pixel mode in one persistent launch
//      over their pixels; the query lists of all query-list scenes in one
//      arena sized at creation (a scene's query count depends only on its
//      geometry and camera; each scene's pixel words and query slots are
//      tile-aligned segments of two pools): one count launch, segmented
//      scans, one write launch, one segmented (map, Morton) sort; then one
//      persistent shared-candidate estimate pass over all of them per
//      k-list width and one exact composite launch, every count the
//      launches need kept on the device. The frame's launch count does not
//      grow with the number of scenes.
//   7. with per-scene radiance caches (pm_batch_cache_enable) step 6's
//      estimate pass is replaced, scene by scene after the lists are
//      built: the scene's training picks and their k-NN targets, its
//      network's Adam steps (schedule, target scale and frame counter in
//      device memory, so replayed frames keep training), inference over
//      every query of the list and the composite
// A scene's image equals the single-scene render of the same scene bit for
// bit: the paths, extents and records are the same, and the k-NN sets do
// not depend on the tree (records at infinity are never within a radius).
#include "cache.cuh"
#include "cache_train.cuh"
#include "gather.cuh"
#include "kdtree.cuh"
#include "launch_count.cuh"
#include "phys_state.cuh"
#include "pm_ctx.cuh"
#include "radix_sort.cuh"
#include "scene.cuh"
#include "trace.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace pm {
namespace {

constexpr int kWords = 16;  // device words per scene, all reset every frame
enum {
    W_COUNTER = 0,  // path counter (count pass, then write pass)
    W_STORED_S = 1, W_STORED_V = 2,
    W_TOTAL_S = 3, W_TOTAL_V = 4,   // scan totals
    W_EXT_S = 5,                    // records, paths of the surface map
    W_EXT_V = 7,                    // records, paths of the volume map
    W_ISSUED = 9,                   // paths issued by the counting pass
};
constexpr int kPathCapFactor = 8;

__global__ void reset_counters_kernel(uint32_t *words, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    words[s * kWords + W_ISSUED] = words[s * kWords + W_COUNTER];
    words[s * kWords + W_COUNTER] = 0u;
}

template <typename T>
cudaError_t dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, sizeof(T) * count);
}

int shift_of(int leaf_size) { return leaf_size >= 128 ? 2 : (leaf_size >= 64 ? 1 : 0); }

// A query-list scene's gather counters from its scans: diffuse queries,
// then the rest (volume march samples).
__global__ void query_gathers_kernel(const uint32_t *off_total, const uint32_t *soff_total,
                                     unsigned long long *gathers) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        gathers[0] = *soff_total;
        gathers[1] = (unsigned long long)*off_total - *soff_total;
    }
}

// The same for every scene of the batched list launches.
__global__ void list_gathers_kernel(const ListScene *ls, const int *ids, int n, unsigned long long *gathers) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int s = ids[j];
    const ListScene &d = ls[s];
    const uint32_t all = d.off[d.npix], surf = d.soff[d.npix];
    gathers[2 * s] = surf;
    gathers[2 * s + 1] = (unsigned long long)all - surf;
}

// Segments of whole sort tiles laid out one after another in a pool (a
// scene's path counts of one map, its per-pixel counts, its query slice),
// cut into runs of at most kRunMax items that one segmented scan or sort
// handles. tab holds, per tile of the pool, its segment's first tile
// (counted from the run's first tile) and the segment's tile count.
constexpr size_t kRunMax = (size_t)1 << 31;
struct SegRuns {
    struct Run {
        size_t first;
        uint32_t n;
    };
    std::vector<Run> runs;
    uint2 *tab = nullptr;
    uint32_t *n_dev = nullptr;  // per run: its item count
    uint32_t max_n = 0;
};

void seg_runs_free(SegRuns &r) {
    cudaFree(r.tab);
    cudaFree(r.n_dev);
    r = SegRuns();
}

// Lays out segments of seg_items[i] items, each rounded up to whole tiles:
// first[i] its first item; *total the pool's items.
cudaError_t seg_runs_build(const std::vector<size_t> &seg_items, SegRuns *r, std::vector<size_t> *first,
                           size_t *total) {
    seg_runs_free(*r);
    std::vector<uint2> tab;
    first->assign(seg_items.size(), 0);
    size_t pos = 0, run_first = 0, run_n = 0;
    for (size_t i = 0; i < seg_items.size(); ++i) {
        const size_t tiles = (seg_items[i] + kSortTile - 1) / kSortTile, items = tiles * kSortTile;
        if (items > kRunMax) return cudaErrorInvalidValue;
        if (run_n + items > kRunMax) {
            r->runs.push_back({run_first, (uint32_t)run_n});
            run_first = pos;
            run_n = 0;
        }
        (*first)[i] = pos;
        const uint32_t t0 = (uint32_t)(run_n / kSortTile);
        for (size_t k = 0; k < tiles; ++k) tab.push_back(make_uint2(t0, (uint32_t)tiles));
        run_n += items;
        pos += items;
    }
    if (run_n > 0) r->runs.push_back({run_first, (uint32_t)run_n});
    *total = pos;
    std::vector<uint32_t> ns;
    for (const auto &run : r->runs) {
        ns.push_back(run.n);
        r->max_n = std::max(r->max_n, run.n);
    }
    cudaError_t e = dalloc(&r->tab, tab.size());
    if (e == cudaSuccess && !tab.empty())
        e = cudaMemcpy(r->tab, tab.data(), sizeof(uint2) * tab.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = dalloc(&r->n_dev, ns.size());
    if (e == cudaSuccess && !ns.empty())
        e = cudaMemcpy(r->n_dev, ns.data(), sizeof(uint32_t) * ns.size(), cudaMemcpyHostToDevice);
    return e;
}

// Segmented exclusive scans of every run of a pool: out[i] counts in[]
// from the first item of i's segment.
cudaError_t scan_runs(const SegRuns &r, const uint32_t *in, uint32_t *out, uint32_t *tmp, cudaStream_t st) {
    for (const auto &run : r.runs) {
        cudaError_t e = exclusive_scan_u32_segmented(in + run.first, out + run.first, run.n,
                                                     r.tab + run.first / kSortTile, tmp, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace
}  // namespace pm

using namespace pm;

struct pm_batch {
    pm_ctx *ctx = nullptr;
    int n = 0;
    int sm_count = 148;
    std::vector<pm_scene> scenes;
    std::vector<pm_config> cfgs;
    std::vector<PScene> dsc;
    std::vector<float *> het;
    struct Map {
        float4 *pos = nullptr, *pow = nullptr, *tpos = nullptr, *tpow = nullptr;
        float4 *tdir = nullptr;
        float4 *lo = nullptr, *hi = nullptr;
        uint32_t cap = 0;
    };
    std::vector<Map> maps;             // 2 per scene
    std::vector<uint32_t> path_cap;    // per scene
    std::vector<size_t> cnt_off;       // per map (2 per scene): first word of its counts in the pools
    std::vector<size_t> pix_off;       // offset of scene s's pixels in the image pools
    std::vector<pm_batch_tune> tune;
    // pools: per scene and map the per-path record counts over the path cap
    // and their scan, each map a segment of whole tiles
    uint32_t *cnt = nullptr, *off = nullptr;
    size_t cnt_words = 0;
    SegRuns cnt_runs;
    ExtentJob *ext_jobs = nullptr;     // 2 per scene
    uint32_t *scan_tmp = nullptr;
    uint32_t *words = nullptr;         // kWords per scene
    uint32_t *capn = nullptr;          // 2 per scene: map capacities (device n of the builds)
    unsigned long long *gathers = nullptr;  // 2 per scene
    uint32_t *work = nullptr;
    float4 *rad = nullptr;
    uchar4 *rgba = nullptr;
    PScene *scenes_dev = nullptr;
    TraceParams *count_dev = nullptr, *write_dev = nullptr;
    BatchRenderScene *render_dev = nullptr;
    uint32_t *prefix_dev = nullptr;
    struct Sort {
        uint64_t *keys = nullptr, *keys_tmp = nullptr;
        uint32_t *vals = nullptr, *vals_tmp = nullptr, *hist = nullptr;
    } sort;  // the autotuner's per-scene rebuilds
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long graph_kernels = 0;
    bool ran = false;
    int n_pixel = 0;  // scenes in the persistent per-pixel launch
    // one scene's query list at a time, sized for the largest scene: the
    // autotuner's timed single-scene query-list renders and the creation
    // count of every scene's queries
    struct Queries {
        uint32_t *cnt = nullptr, *off = nullptr, *scnt = nullptr, *soff = nullptr, *slist = nullptr;
        uint32_t *scan_tmp = nullptr;
        float4 *qa = nullptr, *qd = nullptr, *val = nullptr;
        uint32_t *key = nullptr, *ord = nullptr, *key_tmp = nullptr, *ord_tmp = nullptr, *hist = nullptr;
        float *anchor_d = nullptr;
        uint32_t *defer_n = nullptr;
        size_t pix_cap = 0, q_cap = 0;
    } q;
    std::vector<uint32_t> nq;  // queries per scene
    // The query lists of every query-list scene side by side ("arena"): a
    // pool of per-pixel words (counts, scans, diffuse-query lists; npix + 1
    // per scene) and a pool of query slots (records, values, sorted order),
    // each scene a segment of whole sort tiles, so that one launch sequence
    // counts, scans, writes and sorts all scenes' lists. Then one
    // descriptor per scene grouped by k-list width and one persistent
    // estimate launch per width, and one composite launch.
    struct Arena {
        float4 *qa = nullptr, *qd = nullptr, *val = nullptr;
        uint32_t *ord = nullptr, *off = nullptr;
        uint32_t *cnt = nullptr, *scnt = nullptr, *soff = nullptr, *slist = nullptr;  // pixel pool
        uint32_t *defer = nullptr, *defer_sc = nullptr, *defer_n = nullptr;
        float *anchor_d = nullptr;
        TileScene *desc = nullptr;
        std::vector<size_t> q_off, p_off;  // per scene: first query slot, first pixel word
        size_t q_total = 0, p_total = 0;
        SegRuns q_runs, p_runs;
        int *tile_scene = nullptr;         // per tile of the query pool: its scene
        uint32_t *scan_tmp = nullptr, *hist = nullptr;
        // the scenes of the batched list launches: descriptors of every
        // scene, the ids of those in the query-list render and their
        // 128-pixel block prefix
        ListScene *lists = nullptr;
        int *list_ids = nullptr;
        uint32_t *list_blk = nullptr;
        int n_list = 0;
        uint32_t list_blocks = 0;
        int class_first[5] = {}, class_n[5] = {};
        uint32_t class_chunks[5] = {};
        bool on = false;
    } ar;
    std::vector<uint32_t> nsurf;  // diffuse queries per scene
    // the radix-sorted levels of every map's tree in shared launches (one
    // plan per set of leaf sizes; re-planned when a tune changes one)
    KdMulti kd;
    // per-scene radiance caches (pm_batch_cache_enable): one network per
    // scene; the frame's picks and the per-step scratch are shared (scenes
    // train one after another on the frame's stream)
    struct SceneCache {
        CacheGrid grid;
        CacheParams p;                      // scale_dev and sched point into dev
        float *dev = nullptr;               // [0] target scale, [1..3] Adam {lr, c1, c2}
        unsigned long long *ctr = nullptr;  // [0] Adam steps, [1] frames
    };
    std::vector<SceneCache> caches;
    pm_cache_config ccfg;
    bool cache_on = false;
    TrainScratch cts;
    CacheParams cstep;  // the shared step scratch (w_part, loss_part, dx, xt)
};

namespace {

void free_caches(pm_batch *b) {
    for (auto &c : b->caches) {
        CacheParams q = c.p;
        q.parts_cap = 0;  // the step scratch is shared
        cache_net_free(q);
        cudaFree(c.dev);
        cudaFree(c.ctr);
    }
    b->caches.clear();
    train_scratch_free(b->cts);
    cache_net_free(b->cstep);
    b->cache_on = false;
}

void free_batch(pm_batch *b) {
    if (!b) return;
    free_caches(b);
    kd_multi_free(b->kd);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto &m : b->maps) {
        cudaFree(m.pos); cudaFree(m.pow); cudaFree(m.tpos); cudaFree(m.tpow); cudaFree(m.tdir);
        cudaFree(m.lo); cudaFree(m.hi);
    }
    for (float *h : b->het) cudaFree(h);
    cudaFree(b->cnt); cudaFree(b->off); cudaFree(b->scan_tmp); cudaFree(b->words);
    seg_runs_free(b->cnt_runs);
    cudaFree(b->ext_jobs);
    cudaFree(b->capn); cudaFree(b->gathers); cudaFree(b->work); cudaFree(b->rad); cudaFree(b->rgba);
    cudaFree(b->scenes_dev); cudaFree(b->count_dev); cudaFree(b->write_dev);
    cudaFree(b->render_dev); cudaFree(b->prefix_dev);
    cudaFree(b->sort.keys); cudaFree(b->sort.keys_tmp); cudaFree(b->sort.vals); cudaFree(b->sort.vals_tmp);
    cudaFree(b->sort.hist);
    auto &q = b->q;
    cudaFree(q.cnt); cudaFree(q.off); cudaFree(q.scnt); cudaFree(q.soff); cudaFree(q.slist);
    cudaFree(q.scan_tmp); cudaFree(q.qa); cudaFree(q.qd); cudaFree(q.val); cudaFree(q.key);
    cudaFree(q.ord); cudaFree(q.key_tmp); cudaFree(q.ord_tmp); cudaFree(q.hist); cudaFree(q.anchor_d);
    cudaFree(q.defer_n);
    auto &ar = b->ar;
    cudaFree(ar.qa); cudaFree(ar.qd); cudaFree(ar.val); cudaFree(ar.ord); cudaFree(ar.off);
    cudaFree(ar.defer); cudaFree(ar.defer_sc); cudaFree(ar.defer_n); cudaFree(ar.anchor_d);
    cudaFree(ar.desc);
    cudaFree(ar.cnt); cudaFree(ar.scnt); cudaFree(ar.soff); cudaFree(ar.slist);
    seg_runs_free(ar.q_runs);
    seg_runs_free(ar.p_runs);
    cudaFree(ar.tile_scene); cudaFree(ar.scan_tmp); cudaFree(ar.hist);
    cudaFree(ar.lists); cudaFree(ar.list_ids); cudaFree(ar.list_blk);
    delete b;
}

int depth_of(const pm_batch *b, int s, int m) {
    return tree_depth(b->maps[2 * s + m].cap, shift_of(b->tune[s].leaf_size));
}

BatchRenderScene render_desc(const pm_batch *b, int s) {
    BatchRenderScene d;
    memset(&d, 0, sizeof(d));
    d.sc = b->dsc[s];
    const pm_config &c = b->cfgs[s];
    for (int m = 0; m < 2; ++m) {
        const auto &mp = b->maps[2 * s + m];
        MapView v;
        v.pos = mp.tpos;
        v.pow = mp.tpow;
        v.dir = mp.tdir;
        v.lo = mp.lo;
        v.hi = mp.hi;
        v.n = mp.cap;
        v.depth = mp.cap ? depth_of(b, s, m) : 0;
        v.leaf_shift = shift_of(b->tune[s].leaf_size);
        (m == 0 ? d.surf : d.vol) = v;
    }
    RenderParams R;
    R.width = c.width;
    R.height = c.height;
    R.aspect = c.height > 0 ? (float)c.width / (float)c.height : 1.0f;
    R.k = c.k;
    R.r2cap = c.radius * c.radius;
    R.step = c.march_step;
    R.exposure = c.exposure;
    R.seed = c.seed;
    R.scene_id = c.scene_id;
    R.counters = b->gathers + 2 * s;
    R.tune.collect_max = b->tune[s].collect_max;
    R.tune.merge_min = b->tune[s].merge_min;
    d.R = R;
    d.rad = b->rad + b->pix_off[s];
    d.rgba = b->rgba + b->pix_off[s];
    d.slots = slots_for_k(c.k);
    d.tile = b->tune[s].tile;
    return d;
}

// Uploads the render descriptors and chunk prefix of scenes `ids` (all
// scenes when empty) to dst / prefix.
cudaError_t upload_render(const pm_batch *b, const std::vector<int> &ids, BatchRenderScene *dst,
                          uint32_t *prefix) {
    std::vector<BatchRenderScene> d;
    std::vector<uint32_t> pre(1, 0u);
    for (int s : ids) {
        d.push_back(render_desc(b, s));
        const uint64_t npix = (uint64_t)b->cfgs[s].width * (uint64_t)b->cfgs[s].height;
        const uint64_t per = (uint64_t)4 * (uint64_t)b->tune[s].tile;
        pre.push_back(pre.back() + (uint32_t)((npix + per - 1) / per));
    }
    cudaError_t e = cudaMemcpy(dst, d.data(), sizeof(BatchRenderScene) * d.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    return cudaMemcpy(prefix, pre.data(), sizeof(uint32_t) * pre.size(), cudaMemcpyHostToDevice);
}

std::vector<int> all_ids(const pm_batch *b) {
    std::vector<int> v(b->n);
    for (int i = 0; i < b->n; ++i) v[i] = i;
    return v;
}

// The scenes of the persistent per-pixel launch.
std::vector<int> pixel_ids(const pm_batch *b) {
    std::vector<int> v;
    for (int i = 0; i < b->n; ++i)
        if (!b->tune[i].query_list) v.push_back(i);
    return v;
}

cudaError_t upload_tile_scenes(pm_batch *b);

// Uploads the per-pixel launch's scene list and the estimate pass's
// descriptors (both follow the scenes' tunes).
cudaError_t upload_pixel_scenes(pm_batch *b) {
    const std::vector<int> ids = pixel_ids(b);
    b->n_pixel = (int)ids.size();
    if (!ids.empty()) {
        cudaError_t e = upload_render(b, ids, b->render_dev, b->prefix_dev);
        if (e != cudaSuccess) return e;
    }
    return upload_tile_scenes(b);
}

// The scene's surface / volume queries exist when its map has capacity
// (the render's rule: records past a map's size sit at infinity).
void query_flags(const pm_batch *b, int s, bool *vol_on, bool *surf_on) {
    *surf_on = b->maps[2 * s].cap > 0;
    *vol_on = b->maps[2 * s + 1].cap > 0;
}

// Scene s through the single-scene render's pipeline on the query buffers.
cudaError_t enqueue_query_scene(pm_batch *b, int s, cudaStream_t st) {
    auto &q = b->q;
    const BatchRenderScene d = render_desc(b, s);
    const pm_config &c = b->cfgs[s];
    const uint32_t npix = (uint32_t)c.width * (uint32_t)c.height;
    const uint32_t nq = b->nq[s];
    if (npix == 0) return cudaSuccess;
    bool vol_on, surf_on;
    query_flags(b, s, &vol_on, &surf_on);
    cudaError_t e;
#define Q_TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)
    Q_TRY(cache_count_queries(d.sc, d.R, vol_on, surf_on, q.cnt, q.scnt, st));
    Q_TRY(exclusive_scan_u32_large(q.cnt, q.off, npix, q.off + npix, q.scan_tmp, st));
    Q_TRY(exclusive_scan_u32_large(q.scnt, q.soff, npix, q.soff + npix, q.scan_tmp, st));
    Q_TRY(cache_write_queries(d.sc, d.R, vol_on, surf_on, q.off, q.soff, q.qa, q.qd, q.slist, st));
    query_gathers_kernel<<<1, 32, 0, st>>>(q.off + npix, q.soff + npix, b->gathers + 2 * s);
    note_launch();
    Q_TRY(cudaGetLastError());
    if (nq > 0) {
        CacheGrid box;
        box.levels = 0;
        box.log2_t = 0;
        const pm_scene &sc = b->scenes[s];
        for (int a = 0; a < 3; ++a) {
            const float ext = sc.box_max[a] - sc.box_min[a];
            const float m = 0.01f * (ext > 0.0f ? ext : 1.0f);
            box.lo[a] = sc.box_min[a] - m;
            const float size = ext + 2.0f * m;
            box.inv_size[a] = size > 0.0f ? 1.0f / size : 1.0f;
        }
        Q_TRY(cache_sample_keys(box, q.qa, nullptr, nq, q.key, q.ord, st));
        uint32_t *ok_keys = nullptr, *ok_vals = nullptr;
        Q_TRY(radix_sort_pairs_u32(q.key, q.ord, q.key_tmp, q.ord_tmp, q.off + npix, nq, 0, 31, q.hist, st,
                                   &ok_keys, &ok_vals));
        const TileBuffers buf{q.anchor_d, ok_vals == q.ord ? q.ord_tmp : q.ord, q.defer_n, nullptr};
        Q_TRY(knn_values_tiles(d.sc, d.surf, d.vol, q.qa, q.qd, ok_vals, nq, q.off + npix, 4, c.k, c.radius,
                               true, q.val, buf, b->sm_count, st));
    }
    Q_TRY(render_composite(d.sc, q.off, q.qa, q.qd, q.val, npix, c.exposure, d.rad, d.rgba, st));
#undef Q_TRY
    return cudaSuccess;
}

constexpr int kTileGroups = 4;  // groups of 32 queries per chunk of the estimate pass

// The sort box of scene s's queries: the scene box with a 1 % margin.
CacheGrid sort_box(const pm_batch *b, int s) {
    CacheGrid box;
    memset(&box, 0, sizeof(box));
    const pm_scene &sc = b->scenes[s];
    for (int a = 0; a < 3; ++a) {
        const float ext = sc.box_max[a] - sc.box_min[a];
        const float m = 0.01f * (ext > 0.0f ? ext : 1.0f);
        box.lo[a] = sc.box_min[a] - m;
        const float size = ext + 2.0f * m;
        box.inv_size[a] = size > 0.0f ? 1.0f / size : 1.0f;
    }
    return box;
}

// Uploads the list launches' scene descriptors (every scene; on for the
// query-list scenes with pixels, whose ids and block prefix follow) and
// the estimate pass's: the query-list scenes grouped by k-list width,
// chunks numbered scene after scene within a width.
cudaError_t upload_tile_scenes(pm_batch *b) {
    auto &ar = b->ar;
    if (!ar.on) return cudaSuccess;
    {
        std::vector<ListScene> ls(b->n);
        std::vector<int> ids;
        std::vector<uint32_t> blk(1, 0u);
        for (int s = 0; s < b->n; ++s) {
            const BatchRenderScene r = render_desc(b, s);
            ListScene &l = ls[s];
            memset(&l, 0, sizeof(l));
            const pm_config &c = b->cfgs[s];
            l.sc = r.sc;
            l.R = r.R;
            l.npix = (uint32_t)c.width * (uint32_t)c.height;
            bool vol_on, surf_on;
            query_flags(b, s, &vol_on, &surf_on);
            l.vol_on = vol_on;
            l.surf_on = surf_on;
            l.on = b->tune[s].query_list && l.npix > 0;
            l.nq = b->nq[s];
            l.q_first = ar.q_off[s];
            l.box = sort_box(b, s);
            l.cnt = ar.cnt + ar.p_off[s];
            l.scnt = ar.scnt + ar.p_off[s];
            l.off = ar.off + ar.p_off[s];
            l.soff = ar.soff + ar.p_off[s];
            l.qa = ar.qa + ar.q_off[s];
            l.qd = ar.qd + ar.q_off[s];
            l.slist = ar.slist + ar.p_off[s];
            l.raw = ar.val + ar.q_off[s];
            l.exposure = c.exposure;
            l.rad = r.rad;
            l.rgba = r.rgba;
            if (l.on) {
                ids.push_back(s);
                blk.push_back(blk.back() + (l.npix + kListBlock - 1) / kListBlock);
            }
        }
        ar.n_list = (int)ids.size();
        ar.list_blocks = blk.back();
        cudaError_t e = cudaMemcpy(ar.lists, ls.data(), sizeof(ListScene) * ls.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess && !ids.empty())
            e = cudaMemcpy(ar.list_ids, ids.data(), sizeof(int) * ids.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(ar.list_blk, blk.data(), sizeof(uint32_t) * blk.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
    }
    std::vector<TileScene> d;
    for (int c = 1; c <= 4; ++c) {
        ar.class_first[c] = (int)d.size();
        uint32_t chunks = 0;
        for (int s = 0; s < b->n; ++s) {
            if (!b->tune[s].query_list || b->nq[s] == 0 || slots_for_k(b->cfgs[s].k) != c) continue;
            const BatchRenderScene r = render_desc(b, s);
            TileScene t;
            t.sc = b->scenes_dev + s;
            t.surf = r.surf;
            t.vol = r.vol;
            t.qa = ar.qa + ar.q_off[s];
            t.qd = ar.qd + ar.q_off[s];
            t.val = ar.val + ar.q_off[s];
            t.order = ar.ord + ar.q_off[s];
            t.n = b->nq[s];
            t.chunk_begin = chunks;
            t.k = b->cfgs[s].k;
            t.r2cap = b->cfgs[s].radius * b->cfgs[s].radius;
            chunks += tile_chunks(t.n, kTileGroups);
            d.push_back(t);
        }
        ar.class_n[c] = (int)d.size() - ar.class_first[c];
        ar.class_chunks[c] = chunks;
    }
    if (d.empty()) return cudaSuccess;
    return cudaMemcpy(ar.desc, d.data(), sizeof(TileScene) * d.size(), cudaMemcpyHostToDevice);
}

// The query lists of every query-list scene into the arena: per-pixel
// counts, their scans restarted at each scene, the records, the gather
// counters, then each scene's (map, Morton) order by one segmented sort
// (the sort keys and their second buffer live in the value array, the
// second index buffer in the deferred-query list: both are free until the
// estimate pass).
cudaError_t enqueue_lists(pm_batch *b, cudaStream_t st) {
    auto &ar = b->ar;
    cudaError_t e;
#define Q_TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)
    Q_TRY(list_count_multi(ar.lists, ar.list_ids, ar.list_blk, ar.n_list, ar.list_blocks, st));
    Q_TRY(scan_runs(ar.p_runs, ar.cnt, ar.off, ar.scan_tmp, st));
    Q_TRY(scan_runs(ar.p_runs, ar.scnt, ar.soff, ar.scan_tmp, st));
    Q_TRY(list_write_multi(ar.lists, ar.list_ids, ar.list_blk, ar.n_list, ar.list_blocks, st));
    list_gathers_kernel<<<(ar.n_list + 127) / 128, 128, 0, st>>>(ar.lists, ar.list_ids, ar.n_list, b->gathers);
    note_launch();
    Q_TRY(cudaGetLastError());
    uint32_t *keys = reinterpret_cast<uint32_t *>(ar.val), *keys_tmp = keys + ar.q_total;
    for (size_t r = 0; r < ar.q_runs.runs.size(); ++r) {
        const auto &run = ar.q_runs.runs[r];
        Q_TRY(list_keys_multi(ar.lists, ar.tile_scene, run.first, run.n, keys + run.first, ar.ord + run.first, st));
        uint32_t *ok_keys = nullptr, *ok_vals = nullptr;
        Q_TRY(radix_sort_pairs_u32(keys + run.first, ar.ord + run.first, keys_tmp + run.first, ar.defer + run.first,
                                   ar.q_runs.n_dev + r, run.n, 0, 31, ar.hist, st, &ok_keys, &ok_vals, 0,
                                   ar.q_runs.tab + run.first / kSortTile));
        if (ok_vals != ar.ord + run.first)
            Q_TRY(cudaMemcpyAsync(ar.ord + run.first, ok_vals, sizeof(uint32_t) * run.n, cudaMemcpyDeviceToDevice,
                                  st));
    }
#undef Q_TRY
    return cudaSuccess;
}

// The estimate pass of every query-list scene (one persistent launch per
// k-list width), then the composite of all of them.
cudaError_t enqueue_arena_estimates(pm_batch *b, cudaStream_t st) {
    auto &ar = b->ar;
    cudaError_t e;
    for (int c = 1; c <= 4; ++c) {
        if (ar.class_n[c] == 0) continue;
        const TileBuffers buf{ar.anchor_d, ar.defer, ar.defer_n, nullptr};
        e = knn_values_tiles_multi(ar.desc + ar.class_first[c], ar.class_n[c], ar.class_chunks[c], kTileGroups, c,
                                   true, buf, ar.defer_sc, b->sm_count, st);
        if (e != cudaSuccess) return e;
    }
    return list_composite_multi(ar.lists, ar.list_ids, ar.list_blk, ar.n_list, ar.list_blocks, st);
}

// Scene s's cached frame, after the query lists were built into the
// arena: the frame's picks and k-NN targets, the Adam steps of its
// network, inference over every query and the composite.
cudaError_t enqueue_scene_cache(pm_batch *b, int s, cudaStream_t st) {
    auto &ar = b->ar;
    auto &c = b->caches[s];
    const pm_cache_config &cf = b->ccfg;
    const BatchRenderScene d = render_desc(b, s);
    const pm_config &cfg = b->cfgs[s];
    const uint32_t npix = (uint32_t)cfg.width * (uint32_t)cfg.height, nq = b->nq[s];
    if (npix == 0 || nq == 0) return cudaSuccess;
    float4 *qa = ar.qa + ar.q_off[s], *qd = ar.qd + ar.q_off[s], *val = ar.val + ar.q_off[s];
    const uint32_t *off = ar.off + ar.p_off[s];
    TrainScratch &t = b->cts;
    const uint32_t ns = t.ns;
    cudaError_t e;
#define S_TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)
    S_TRY(cache_pick_and_target(cf, c.grid, 0, c.ctr + 1, b->dsc[s], d.surf, d.vol, cfg.k, cfg.radius, qa, qd, nq,
                                ar.slist + ar.p_off[s], b->nsurf[s], t, b->sm_count, st));
    S_TRY(cache_scale_init(t.tgt, ns, t.scale_sum, c.dev, st));
    S_TRY(cudaMemsetAsync(c.p.loss, 0, sizeof(float), st));
    const uint32_t nb = cache_batch_count(ns, cf.batch);
    for (uint32_t i = 0; i < nb; ++i) {
        uint32_t o, n;
        cache_batch_range(ns, nb, i, &o, &n);
        // the scales and the learning rate come from c.dev (the host values are unused)
        S_TRY(cache_backward(c.grid, c.p, b->dsc[s], t.tqa + o, t.tqd + o, nullptr, t.tgt + o, n, 1.0f,
                             1.0f / (3.0f * (float)n), cf.loss_eps, nullptr, nullptr, b->sm_count, st));
        S_TRY(cache_schedule(c.dev + 1, c.ctr, cf.lr, cf.lr_min, cf.lr_half_life, cf.beta1, cf.beta2, st));
        S_TRY(cache_adam(c.grid, c.p, cf.lr, cf.beta1, cf.beta2, cf.eps, 1, st));
    }
    S_TRY(cache_count_up(c.ctr + 1, st));
    S_TRY(cache_infer(c.grid, c.p, b->dsc[s], qa, qd, nullptr, nq, 1.0f, val, b->sm_count, st));
    S_TRY(cache_composite(d.sc, off, qa, qd, val, npix, cfg.exposure, d.rad, d.rgba, st));
#undef S_TRY
    return cudaSuccess;
}

// Counts every scene's queries (they depend on its geometry and camera
// only) and sizes the query buffers for the largest scene.
cudaError_t size_query_buffers(pm_batch *b) {
    auto &q = b->q;
    size_t max_pix = 1;
    for (int s = 0; s < b->n; ++s) max_pix = std::max(max_pix, (size_t)b->cfgs[s].width * b->cfgs[s].height);
    cudaError_t e;
#define Z_TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)
    Z_TRY(dalloc(&q.cnt, max_pix));
    Z_TRY(dalloc(&q.off, max_pix + 1));
    Z_TRY(dalloc(&q.scnt, max_pix));
    Z_TRY(dalloc(&q.soff, max_pix + 1));
    Z_TRY(dalloc(&q.slist, max_pix));
    Z_TRY(dalloc(&q.scan_tmp, scan_tile_count((uint32_t)max_pix) + 1));
    q.pix_cap = max_pix;
    b->nq.assign(b->n, 0u);
    b->nsurf.assign(b->n, 0u);
    size_t max_q = 1;
    for (int s = 0; s < b->n; ++s) {
        const BatchRenderScene d = render_desc(b, s);
        const uint32_t npix = (uint32_t)b->cfgs[s].width * (uint32_t)b->cfgs[s].height;
        if (npix == 0) continue;
        bool vol_on, surf_on;
        query_flags(b, s, &vol_on, &surf_on);
        Z_TRY(cache_count_queries(d.sc, d.R, vol_on, surf_on, q.cnt, q.scnt, 0));
        Z_TRY(exclusive_scan_u32_large(q.cnt, q.off, npix, q.off + npix, q.scan_tmp, 0));
        Z_TRY(cudaMemcpy(&b->nq[s], q.off + npix, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        Z_TRY(exclusive_scan_u32_large(q.scnt, q.soff, npix, q.soff + npix, q.scan_tmp, 0));
        Z_TRY(cudaMemcpy(&b->nsurf[s], q.soff + npix, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        max_q = std::max(max_q, (size_t)b->nq[s]);
    }
    Z_TRY(dalloc(&q.qa, max_q));
    Z_TRY(dalloc(&q.qd, max_q));
    Z_TRY(dalloc(&q.val, max_q));
    Z_TRY(dalloc(&q.key, max_q));
    Z_TRY(dalloc(&q.ord, max_q));
    Z_TRY(dalloc(&q.key_tmp, max_q));
    Z_TRY(dalloc(&q.ord_tmp, max_q));
    Z_TRY(dalloc(&q.hist, radix_sort_hist_words((uint32_t)max_q)));
    Z_TRY(dalloc(&q.anchor_d, tile_chunks((uint32_t)max_q, 4)));
    Z_TRY(dalloc(&q.defer_n, 2));  // deferred count, chunk counter
    q.q_cap = max_q;
    // the arena: every scene's pixel words and query slots, each a
    // segment of whole sort tiles
    auto &ar = b->ar;
    size_t max_chunks = 1;
    std::vector<size_t> q_items(b->n), p_items(b->n);
    for (int s = 0; s < b->n; ++s) {
        q_items[s] = b->nq[s];
        p_items[s] = (size_t)b->cfgs[s].width * b->cfgs[s].height + 1;
        max_chunks += tile_chunks(b->nq[s], kTileGroups);
    }
    Z_TRY(seg_runs_build(q_items, &ar.q_runs, &ar.q_off, &ar.q_total));
    Z_TRY(seg_runs_build(p_items, &ar.p_runs, &ar.p_off, &ar.p_total));
    const size_t q_total = std::max<size_t>(ar.q_total, 1), p_total = ar.p_total;
    Z_TRY(dalloc(&ar.qa, q_total));
    Z_TRY(dalloc(&ar.qd, q_total));
    Z_TRY(dalloc(&ar.val, q_total));
    Z_TRY(dalloc(&ar.ord, q_total));
    Z_TRY(dalloc(&ar.off, p_total));
    Z_TRY(dalloc(&ar.cnt, p_total));
    Z_TRY(dalloc(&ar.scnt, p_total));
    Z_TRY(dalloc(&ar.soff, p_total));
    Z_TRY(dalloc(&ar.slist, p_total));
    // counts past each scene's pixels (and of scenes outside the list
    // render) stay 0
    Z_TRY(cudaMemset(ar.cnt, 0, sizeof(uint32_t) * p_total));
    Z_TRY(cudaMemset(ar.scnt, 0, sizeof(uint32_t) * p_total));
    Z_TRY(dalloc(&ar.defer, q_total));
    Z_TRY(dalloc(&ar.defer_sc, q_total));
    Z_TRY(dalloc(&ar.defer_n, 2));
    Z_TRY(dalloc(&ar.anchor_d, max_chunks));
    Z_TRY(dalloc(&ar.desc, (size_t)b->n));
    Z_TRY(dalloc(&ar.lists, (size_t)b->n));
    Z_TRY(dalloc(&ar.list_ids, (size_t)b->n));
    Z_TRY(dalloc(&ar.list_blk, (size_t)b->n + 1));
    Z_TRY(dalloc(&ar.scan_tmp, scan_tile_count(std::max(ar.p_runs.max_n, 1u)) + 1));
    Z_TRY(dalloc(&ar.hist, radix_sort_hist_words(std::max(ar.q_runs.max_n, 1u))));
    {
        std::vector<int> ts(std::max<size_t>(ar.q_total / kSortTile, 1), -1);
        for (int s = 0; s < b->n; ++s)
            for (size_t t = ar.q_off[s] / kSortTile; t < (ar.q_off[s] + q_items[s] + kSortTile - 1) / kSortTile; ++t)
                ts[t] = s;
        Z_TRY(dalloc(&ar.tile_scene, ts.size()));
        Z_TRY(cudaMemcpy(ar.tile_scene, ts.data(), sizeof(int) * ts.size(), cudaMemcpyHostToDevice));
    }
    ar.on = true;
    Z_TRY(upload_tile_scenes(b));
#undef Z_TRY
    return cudaSuccess;
}

// Pads and builds the two trees of scene s on `st` with sort scratch `so`.
// The build arguments of map m of scene s (sort scratch so; nullable for a
// plan of the shared levels).
KdBuildArgs map_args(const pm_batch *b, int s, int m, const pm_batch::Sort *so) {
    const auto &mp = b->maps[2 * s + m];
    KdBuildArgs a;
    a.n = mp.cap;
    a.n_dev = b->capn + 2 * s + m;
    const pm_scene &sc = b->scenes[s];
    a.lo = make_float3(sc.box_min[0], sc.box_min[1], sc.box_min[2]);
    a.hi = make_float3(sc.box_max[0], sc.box_max[1], sc.box_max[2]);
    a.box_dev = nullptr;
    a.pos_in = mp.pos;
    a.pow_in = mp.pow;
    a.pos_out = mp.tpos;
    a.pow_out = mp.tpow;
    a.dir_out = mp.tdir;
    a.node_lo = mp.lo;
    a.node_hi = mp.hi;
    a.keys = so ? so->keys : nullptr;
    a.keys_tmp = so ? so->keys_tmp : nullptr;
    a.vals = so ? so->vals : nullptr;
    a.vals_tmp = so ? so->vals_tmp : nullptr;
    a.hist = so ? so->hist : nullptr;
    a.order_out = nullptr;
    a.leaf_shift = shift_of(b->tune[s].leaf_size);
    a.pad_count = b->words + s * kWords + (m == 0 ? W_EXT_S : W_EXT_V);
    return a;
}

// Pads and builds the two trees of scene s on `st` with sort scratch `so`.
cudaError_t build_scene(pm_batch *b, int s, cudaStream_t st, const pm_batch::Sort &so) {
    for (int m = 0; m < 2; ++m) {
        auto &mp = b->maps[2 * s + m];
        if (mp.cap == 0) continue;
        cudaError_t e = pad_map(mp.pos, mp.pow, b->words + s * kWords + (m == 0 ? W_EXT_S : W_EXT_V),
                                mp.cap, st);
        if (e != cudaSuccess) return e;
        e = build_tree(map_args(b, s, m, &so), st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The plan of the shared tree levels for the current leaf sizes.
cudaError_t plan_trees(pm_batch *b) {
    kd_multi_free(b->kd);
    std::vector<KdBuildArgs> args;
    for (int s = 0; s < b->n; ++s)
        for (int m = 0; m < 2; ++m) args.push_back(map_args(b, s, m, nullptr));
    return kd_multi_create(args, &b->kd);
}

cudaError_t enqueue_frame(pm_batch *b, cudaStream_t st) {
    cudaError_t e;
#define B_TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)
    B_TRY(cudaMemsetAsync(b->words, 0, sizeof(uint32_t) * kWords * b->n, st));
    B_TRY(cudaMemsetAsync(b->cnt, 0, sizeof(uint32_t) * b->cnt_words, st));
    B_TRY(cudaMemsetAsync(b->gathers, 0, sizeof(unsigned long long) * 2 * b->n, st));
    B_TRY(trace_photons_batch(b->scenes_dev, b->count_dev, b->n, b->sm_count, st));
    // every map's record extent: the scans of all path counts, then one
    // search per map
    B_TRY(scan_runs(b->cnt_runs, b->cnt, b->off, b->scan_tmp, st));
    B_TRY(map_extents_multi(b->ext_jobs, 2 * b->n, st));
    reset_counters_kernel<<<(b->n + 127) / 128, 128, 0, st>>>(b->words, b->n);
    note_launch();
    B_TRY(cudaGetLastError());
    B_TRY(trace_photons_batch(b->scenes_dev, b->write_dev, b->n, b->sm_count, st));
    // the trees of every map in shared launches: records past each map's
    // size to infinity, the radix-sorted levels, then the subtree finishes,
    // the permutations into tree order and the boxes
    uint32_t *order = nullptr;
    B_TRY(kd_multi_levels(b->kd, st, &order));
    B_TRY(kd_multi_finish(b->kd, order, st));
    if (b->n_pixel > 0) B_TRY(render_batch(b->render_dev, b->prefix_dev, b->n_pixel, b->work, b->sm_count, st));
    if (b->ar.n_list > 0) {
        B_TRY(enqueue_lists(b, st));
        if (b->cache_on) {
            for (int s = 0; s < b->n; ++s)
                if (b->tune[s].query_list) B_TRY(enqueue_scene_cache(b, s, st));
        } else {
            B_TRY(enqueue_arena_estimates(b, st));
        }
    }
#undef B_TRY
    return cudaSuccess;
}

void drop_graph(pm_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

}  // namespace

extern "C" {

pm_status pm_batch_create(pm_ctx *ctx, int n, const pm_scene *scenes, const pm_config *cfgs,
                          pm_batch **out) {
    if (!ctx || !out || n < 1 || n > 4096 || !scenes || !cfgs) return PM_ERR_INVALID;
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        std::string why;
        pm_status s = validate(scenes[i], cfgs[i], &why);
        if (s != PM_OK) return fail(ctx, s, "scene " + std::to_string(i) + ": " + why);
        if (std::max(cfgs[i].surface_photons, cfgs[i].volume_photons) > (1u << 26))
            return fail(ctx, PM_ERR_LIMIT, "batched map above 2^26 records");
    }
    DeviceGuard g(ctx->device);
    pm_batch *b = new pm_batch();
    b->ctx = ctx;
    b->n = n;
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
    b->scenes.assign(scenes, scenes + n);
    b->cfgs.assign(cfgs, cfgs + n);
    b->maps.resize(2 * (size_t)n);
    b->het.assign(n, nullptr);
    b->tune.resize(n);
    cudaError_t e = cudaSuccess;
#define C_TRY(x) do { e = (x); if (e != cudaSuccess) { free_batch(b); return check_cuda(ctx, e, #x); } } while (0)
    size_t pix = 0;
    uint32_t max_map = 1;
    std::vector<size_t> map_counts;  // per map: path cap (one segment of the count pools each)
    for (int s = 0; s < n; ++s) {
        const pm_config &c = cfgs[s];
        b->tune[s] = pm_batch_tune{c.leaf_size, 1, 128, 16, 1};
        const uint32_t tmax = std::max(c.surface_photons, c.volume_photons);
        uint64_t cap = c.max_paths ? c.max_paths : (uint64_t)tmax * kPathCapFactor;
        cap = std::max<uint64_t>(cap, 1024);
        if (cap > (1ull << 30)) { free_batch(b); return fail(ctx, PM_ERR_LIMIT, "path cap above 2^30"); }
        b->path_cap.push_back((uint32_t)cap);
        map_counts.push_back(cap);
        map_counts.push_back(cap);
        b->pix_off.push_back(pix);
        pix += (size_t)c.width * (size_t)c.height;
        const uint32_t targets[2] = {c.surface_photons, c.volume_photons};
        for (int m = 0; m < 2; ++m) {
            auto &mp = b->maps[2 * s + m];
            mp.cap = targets[m];
            max_map = std::max(max_map, mp.cap);
            C_TRY(dalloc(&mp.pos, mp.cap));
            C_TRY(dalloc(&mp.pow, mp.cap));
            C_TRY(dalloc(&mp.tpos, mp.cap));
            C_TRY(dalloc(&mp.tpow, mp.cap));
            C_TRY(dalloc(&mp.tdir, mp.cap));
            C_TRY(dalloc(&mp.lo, tree_nodes(mp.cap)));
            C_TRY(dalloc(&mp.hi, tree_nodes(mp.cap)));
        }
        if (scenes[s].het_res > 0) {
            const size_t nv = (size_t)scenes[s].het_res * scenes[s].het_res * scenes[s].het_res;
            C_TRY(dalloc(&b->het[s], nv));
            C_TRY(make_noise_grid(b->het[s], scenes[s].het_res, c.seed ^ 0x6E6F697365ull,
                                  scenes[s].het_min, scenes[s].het_max, 0));
        }
        b->dsc.push_back(to_device_scene(scenes[s], b->het[s]));
    }
    C_TRY(seg_runs_build(map_counts, &b->cnt_runs, &b->cnt_off, &b->cnt_words));
    C_TRY(dalloc(&b->cnt, b->cnt_words));
    C_TRY(dalloc(&b->off, b->cnt_words));
    C_TRY(dalloc(&b->scan_tmp, scan_tile_count(b->cnt_runs.max_n) + 1));
    C_TRY(dalloc(&b->ext_jobs, 2 * (size_t)n));
    C_TRY(dalloc(&b->words, (size_t)kWords * n));
    C_TRY(dalloc(&b->capn, 2 * (size_t)n));
    C_TRY(dalloc(&b->gathers, 2 * (size_t)n));
    C_TRY(dalloc(&b->work, 1));
    C_TRY(dalloc(&b->rad, pix));
    C_TRY(dalloc(&b->rgba, pix));
    C_TRY(dalloc(&b->scenes_dev, n));
    C_TRY(dalloc(&b->count_dev, n));
    C_TRY(dalloc(&b->write_dev, n));
    C_TRY(dalloc(&b->render_dev, n));
    C_TRY(dalloc(&b->prefix_dev, (size_t)n + 1));
    C_TRY(dalloc(&b->sort.keys, max_map));
    C_TRY(dalloc(&b->sort.keys_tmp, max_map));
    C_TRY(dalloc(&b->sort.vals, max_map));
    C_TRY(dalloc(&b->sort.vals_tmp, max_map));
    C_TRY(dalloc(&b->sort.hist, radix_sort_hist_words(max_map)));
    // static per-scene parameters
    std::vector<uint32_t> capn(2 * (size_t)n);
    std::vector<TraceParams> cp(n), wp(n);
    std::vector<ExtentJob> jobs(2 * (size_t)n);
    for (int s = 0; s < n; ++s) {
        const pm_config &c = cfgs[s];
        capn[2 * s] = b->maps[2 * s].cap;
        capn[2 * s + 1] = b->maps[2 * s + 1].cap;
        uint32_t *w = b->words + s * kWords;
        const size_t os = b->cnt_off[2 * s], ov = b->cnt_off[2 * s + 1];
        const uint32_t cap = b->path_cap[s];
        for (int m = 0; m < 2; ++m) {
            ExtentJob &j = jobs[2 * s + m];
            const size_t o = m == 0 ? os : ov;
            j.cnt = b->cnt + o;
            j.off = b->off + o;
            j.cap = cap;
            j.target = m == 0 ? c.surface_photons : c.volume_photons;
            j.issued = w + W_COUNTER;
            j.total = w + (m == 0 ? W_TOTAL_S : W_TOTAL_V);
            j.extent = w + (m == 0 ? W_EXT_S : W_EXT_V);
        }
        TraceParams P;
        memset(&P, 0, sizeof(P));
        P.seed = c.seed;
        P.scene_id = c.scene_id;
        P.max_bounces = c.max_bounces;
        P.rr = c.rr_survival;
        P.target_s = c.surface_photons;
        P.target_v = c.volume_photons;
        P.path_cap = cap;
        P.path_counter = w + W_COUNTER;
        P.stored_s = w + W_STORED_S;
        P.stored_v = w + W_STORED_V;
        P.cnt_s = b->cnt + os;
        P.cnt_v = b->cnt + ov;
        cp[s] = P;
        P.store = 1;
        P.off_s = b->off + os;
        P.off_v = b->off + ov;
        P.ext_s = w + W_EXT_S;
        P.ext_v = w + W_EXT_V;
        P.power = scenes[s].light_power;
        P.spos = b->maps[2 * s].pos; P.spow = b->maps[2 * s].pow;
        P.vpos = b->maps[2 * s + 1].pos; P.vpow = b->maps[2 * s + 1].pow;
        wp[s] = P;
    }
    C_TRY(cudaMemcpy(b->capn, capn.data(), sizeof(uint32_t) * capn.size(), cudaMemcpyHostToDevice));
    C_TRY(cudaMemcpy(b->scenes_dev, b->dsc.data(), sizeof(PScene) * n, cudaMemcpyHostToDevice));
    C_TRY(cudaMemcpy(b->count_dev, cp.data(), sizeof(TraceParams) * n, cudaMemcpyHostToDevice));
    C_TRY(cudaMemcpy(b->write_dev, wp.data(), sizeof(TraceParams) * n, cudaMemcpyHostToDevice));
    C_TRY(cudaMemcpy(b->ext_jobs, jobs.data(), sizeof(ExtentJob) * jobs.size(), cudaMemcpyHostToDevice));
    C_TRY(upload_pixel_scenes(b));
    C_TRY(size_query_buffers(b));
    C_TRY(plan_trees(b));
    C_TRY(cudaDeviceSynchronize());
#undef C_TRY
    *out = b;
    return PM_OK;
}

void pm_batch_destroy(pm_batch *b) {
    if (!b) return;
    DeviceGuard g(b->ctx->device);
    cudaDeviceSynchronize();
    free_batch(b);
}

pm_status pm_batch_frame(pm_batch *b, cudaStream_t stream) {
    if (!b) return PM_ERR_INVALID;
    DeviceGuard g(b->ctx->device);
    cudaError_t e = enqueue_frame(b, stream);
    if (e != cudaSuccess) return check_cuda(b->ctx, e, "pm_batch_frame");
    b->ran = true;
    return PM_OK;
}

pm_status pm_batch_capture(pm_batch *b, cudaStream_t stream) {
    if (!b) return PM_ERR_INVALID;
    DeviceGuard g(b->ctx->device);
    drop_graph(b);
    cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return check_cuda(b->ctx, e, "cudaStreamBeginCapture");
    const unsigned long long l0 = launch_counter().load();
    cudaError_t fe = enqueue_frame(b, stream);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(stream, &graph);
    if (fe != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return check_cuda(b->ctx, fe, "pm_batch_capture (frame)");
    }
    if (e != cudaSuccess) return check_cuda(b->ctx, e, "cudaStreamEndCapture");
    b->graph = graph;
    b->graph_kernels = launch_counter().load() - l0;
    // the captured launches ran nowhere: take them off the launch count
    launch_counter().fetch_sub(b->graph_kernels);
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    if (e != cudaSuccess) {
        drop_graph(b);
        return check_cuda(b->ctx, e, "cudaGraphInstantiate");
    }
    return PM_OK;
}

pm_status pm_batch_launch(pm_batch *b, cudaStream_t stream) {
    if (!b) return PM_ERR_INVALID;
    if (!b->exec) return fail(b->ctx, PM_ERR_STATE, "pm_batch_launch before pm_batch_capture");
    DeviceGuard g(b->ctx->device);
    cudaError_t e = cudaGraphLaunch(b->exec, stream);
    if (e != cudaSuccess) return check_cuda(b->ctx, e, "cudaGraphLaunch");
    note_launches(b->graph_kernels);
    b->ran = true;
    return PM_OK;
}

pm_status pm_batch_image(pm_batch *b, int scene, float4 **radiance, uchar4 **rgba) {
    if (!b || scene < 0 || scene >= b->n) return PM_ERR_INVALID;
    if (radiance) *radiance = b->rad + b->pix_off[scene];
    if (rgba) *rgba = b->rgba + b->pix_off[scene];
    return PM_OK;
}

pm_status pm_batch_read(pm_batch *b, int scene, float4 *radiance, uchar4 *rgba) {
    if (!b || scene < 0 || scene >= b->n) return PM_ERR_INVALID;
    DeviceGuard g(b->ctx->device);
    const size_t npix = (size_t)b->cfgs[scene].width * (size_t)b->cfgs[scene].height;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess && radiance && npix)
        e = cudaMemcpy(radiance, b->rad + b->pix_off[scene], sizeof(float4) * npix, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && rgba && npix)
        e = cudaMemcpy(rgba, b->rgba + b->pix_off[scene], sizeof(uchar4) * npix, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return check_cuda(b->ctx, e, "pm_batch_read");
    return PM_OK;
}

pm_status pm_batch_stats(pm_batch *b, int scene, pm_frame_stats *out) {
    if (!b || !out || scene < 0 || scene >= b->n) return PM_ERR_INVALID;
    DeviceGuard g(b->ctx->device);
    cudaError_t e = cudaDeviceSynchronize();
    uint32_t w[kWords];
    unsigned long long gc[2];
    if (e == cudaSuccess)
        e = cudaMemcpy(w, b->words + scene * kWords, sizeof(w), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(gc, b->gathers + 2 * scene, sizeof(gc), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return check_cuda(b->ctx, e, "pm_batch_stats");
    memset(out, 0, sizeof(*out));
    out->paths_traced = std::min(w[W_ISSUED], b->path_cap[scene]);
    out->map_size[0] = w[W_EXT_S];
    out->map_paths[0] = w[W_EXT_S + 1];
    out->map_size[1] = w[W_EXT_V];
    out->map_paths[1] = w[W_EXT_V + 1];
    out->surface_gathers = gc[0];
    out->volume_gathers = gc[1];
    return PM_OK;
}

pm_status pm_batch_set_tune(pm_batch *b, int scene, const pm_batch_tune *t) {
    if (!b || !t || scene < 0 || scene >= b->n) return PM_ERR_INVALID;
    if ((t->leaf_size != 32 && t->leaf_size != 64 && t->leaf_size != 128) || t->tile < 1 ||
        t->tile > 64 || (t->collect_max != 32 && t->collect_max != 64 && t->collect_max != 128) ||
        t->merge_min < 1 || t->merge_min > 33 || (t->query_list != 0 && t->query_list != 1))
        return fail(b->ctx, PM_ERR_INVALID, "invalid batch tune");
    if (b->cache_on && !t->query_list)
        return fail(b->ctx, PM_ERR_STATE, "per-scene radiance caches need the query-list render");
    DeviceGuard g(b->ctx->device);
    cudaDeviceSynchronize();
    b->tune[scene] = *t;
    drop_graph(b);
    cudaError_t e = upload_pixel_scenes(b);
    if (e == cudaSuccess) e = plan_trees(b);
    if (e != cudaSuccess) return check_cuda(b->ctx, e, "pm_batch_set_tune");
    return PM_OK;
}

pm_status pm_batch_get_tune(pm_batch *b, int scene, pm_batch_tune *t) {
    if (!b || !t || scene < 0 || scene >= b->n) return PM_ERR_INVALID;
    *t = b->tune[scene];
    return PM_OK;
}

pm_status pm_batch_cache_enable(pm_batch *b, const pm_cache_config *cfg_in) {
    if (!b) return PM_ERR_INVALID;
    pm_cache_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else pm_cache_default_config(&cfg);
    if (!cache_config_ok(cfg)) return fail(b->ctx, PM_ERR_INVALID, "invalid radiance-cache configuration");
    DeviceGuard g(b->ctx->device);
    cudaDeviceSynchronize();
    drop_graph(b);
    free_caches(b);
    cudaError_t e;
#define E_TRY(x) do { e = (x); if (e != cudaSuccess) { free_caches(b); return check_cuda(b->ctx, e, #x); } } while (0)
    b->ccfg = cfg;
    E_TRY(train_scratch_alloc(cfg.train_samples, &b->cts));
    // the shared step scratch: a network without table or weights of its own
    {
        CacheParams &q = b->cstep;
        memset(&q, 0, sizeof(q));
        q.parts_cap = b->sm_count;
        E_TRY(dalloc(&q.w_part, (size_t)q.parts_cap * kCacheWeights));
        E_TRY(dalloc(&q.loss_part, q.parts_cap));
        q.dx_cap = cfg.batch;
        E_TRY(dalloc(&q.dx, (size_t)cfg.batch * 8));
        E_TRY(dalloc(&q.xt, (size_t)cfg.batch * 8));
    }
    b->caches.resize(b->n);
    for (int s = 0; s < b->n; ++s) {
        auto &c = b->caches[s];
        cache_grid_init(cfg, &c.grid);
        cache_grid_box(c.grid, b->scenes[s]);
        E_TRY(cache_net_alloc(cfg, c.grid, cfg.seed + (uint64_t)s, 0, &c.p));
        E_TRY(dalloc(&c.dev, 4));
        E_TRY(dalloc(&c.ctr, 2));
        E_TRY(cudaMemset(c.dev, 0, sizeof(float) * 4));
        E_TRY(cudaMemset(c.ctr, 0, sizeof(unsigned long long) * 2));
        c.p.scale_dev = c.dev;
        c.p.sched = c.dev + 1;
        c.p.parts_cap = b->cstep.parts_cap;
        c.p.w_part = b->cstep.w_part;
        c.p.loss_part = b->cstep.loss_part;
        c.p.dx_cap = b->cstep.dx_cap;
        c.p.dx = b->cstep.dx;
        c.p.xt = b->cstep.xt;
        // the cache renders through the query list
        b->tune[s].query_list = 1;
    }
    E_TRY(upload_pixel_scenes(b));
    E_TRY(cudaDeviceSynchronize());
#undef E_TRY
    b->cache_on = true;
    return PM_OK;
}

pm_status pm_batch_cache_disable(pm_batch *b) {
    if (!b) return PM_ERR_INVALID;
    DeviceGuard g(b->ctx->device);
    cudaDeviceSynchronize();
    drop_graph(b);
    free_caches(b);
    return PM_OK;
}

pm_status pm_batch_autotune(pm_batch *b, const char *json_path, cudaStream_t stream) {
    if (!b) return PM_ERR_INVALID;
    if (b->cache_on) return fail(b->ctx, PM_ERR_STATE, "pm_batch_autotune with per-scene radiance caches on");
    DeviceGuard g(b->ctx->device);
    pm_ctx *ctx = b->ctx;
    cudaError_t e;
#define A_TRY(x) do { e = (x); if (e != cudaSuccess) return check_cuda(ctx, e, #x); } while (0)
    if (!b->ran) {
        A_TRY(enqueue_frame(b, stream));
        b->ran = true;
    }
    A_TRY(cudaStreamSynchronize(stream));
    drop_graph(b);
    BatchRenderScene *one = nullptr;
    uint32_t *one_prefix = nullptr;
    A_TRY(dalloc(&one, 1));
    A_TRY(dalloc(&one_prefix, 2));
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    std::string js = "{\"format\": \"pm-batch-autotune\", \"version\": 1, \"classes\": [";
    bool first_class = true;
    const int leaves[3] = {32, 64, 128}, tiles[4] = {1, 2, 4, 8}, collects[3] = {32, 64, 128},
              merges[3] = {8, 16, 32};
    auto time_scene = [&](int s, float *ms_out) -> cudaError_t {
        const bool ql = b->tune[s].query_list != 0;
        cudaError_t ee = ql ? cudaSuccess : upload_render(b, {s}, one, one_prefix);
        if (ee != cudaSuccess) return ee;
        float best = 3.0e38f;
        for (int rep = 0; rep < 3; ++rep) {
            ee = cudaEventRecord(t0, stream);
            if (ee == cudaSuccess)
                ee = ql ? enqueue_query_scene(b, s, stream)
                        : render_batch(one, one_prefix, 1, b->work, b->sm_count, stream);
            if (ee == cudaSuccess) ee = cudaEventRecord(t1, stream);
            if (ee == cudaSuccess) ee = cudaEventSynchronize(t1);
            if (ee != cudaSuccess) return ee;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (rep > 0) best = std::min(best, ms);  // first repetition warms the caches
        }
        *ms_out = best;
        return cudaSuccess;
    };
    for (int kc = 32; kc <= 128; kc <<= 1) {
        int rep = -1;
        uint64_t most = 0;
        for (int s = 0; s < b->n; ++s) {
            const uint64_t px = (uint64_t)b->cfgs[s].width * b->cfgs[s].height;
            if (b->cfgs[s].k == kc && px > most) { most = px; rep = s; }
        }
        if (rep < 0) continue;
        std::string trials;
        pm_batch_tune best = b->tune[rep];
        float best_ms = 3.0e38f;
        for (int li = 0; li < 3; ++li) {
            b->tune[rep].leaf_size = leaves[li];
            b->tune[rep].query_list = 0;
            A_TRY(build_scene(b, rep, stream, b->sort));
            for (int ti = 0; ti < 4; ++ti) {
                b->tune[rep].tile = tiles[ti];
                b->tune[rep].collect_max = 128;
                b->tune[rep].merge_min = 16;
                float ms;
                A_TRY(time_scene(rep, &ms));
                char buf[160];
                snprintf(buf, sizeof(buf), "%s{\"leaf_size\": %d, \"tile\": %d, \"collect_max\": 128, "
                         "\"merge_min\": 16, \"query_list\": 0, \"ms\": %.4f}", trials.empty() ? "" : ", ",
                         leaves[li], tiles[ti], ms);
                trials += buf;
                if (ms < best_ms) { best_ms = ms; best = b->tune[rep]; }
            }
        }
        b->tune[rep] = best;
        A_TRY(build_scene(b, rep, stream, b->sort));
        for (int ci = 0; ci < 3; ++ci)
            for (int mi = 0; mi < 3; ++mi) {
                b->tune[rep].collect_max = collects[ci];
                b->tune[rep].merge_min = merges[mi];
                float ms;
                A_TRY(time_scene(rep, &ms));
                char buf[160];
                snprintf(buf, sizeof(buf), ", {\"leaf_size\": %d, \"tile\": %d, \"collect_max\": %d, "
                         "\"merge_min\": %d, \"query_list\": 0, \"ms\": %.4f}", best.leaf_size, best.tile,
                         collects[ci], merges[mi], ms);
                trials += buf;
                if (ms < best_ms) { best_ms = ms; best = b->tune[rep]; }
            }
        // the query-list render at each leaf size (its other knobs do not apply)
        const pm_batch_tune pixel_best = best;
        for (int li = 0; li < 3; ++li) {
            b->tune[rep] = pixel_best;
            b->tune[rep].leaf_size = leaves[li];
            b->tune[rep].query_list = 1;
            A_TRY(build_scene(b, rep, stream, b->sort));
            float ms;
            A_TRY(time_scene(rep, &ms));
            char buf[160];
            snprintf(buf, sizeof(buf), ", {\"leaf_size\": %d, \"tile\": %d, \"collect_max\": %d, "
                     "\"merge_min\": %d, \"query_list\": 1, \"ms\": %.4f}", leaves[li], pixel_best.tile,
                     pixel_best.collect_max, pixel_best.merge_min, ms);
            trials += buf;
            if (ms < best_ms) { best_ms = ms; best = b->tune[rep]; }
        }
        b->tune[rep] = best;
        int members = 0;
        for (int s = 0; s < b->n; ++s)
            if (b->cfgs[s].k == kc) { b->tune[s] = best; ++members; }
        A_TRY(build_scene(b, rep, stream, b->sort));
        char head[400];
        snprintf(head, sizeof(head), "%s{\"k\": %d, \"scenes\": %d, \"probe_scene\": %d, \"pixels\": %llu, "
                 "\"choice\": {\"leaf_size\": %d, \"tile\": %d, \"collect_max\": %d, \"merge_min\": %d, "
                 "\"query_list\": %d, \"ms\": %.4f}, \"trials\": [", first_class ? "" : ", ", kc, members,
                 rep, (unsigned long long)most, best.leaf_size, best.tile, best.collect_max, best.merge_min,
                 best.query_list, best_ms);
        js += head + trials + "]}";
        first_class = false;
    }
    js += "]}\n";
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFree(one);
    cudaFree(one_prefix);
    A_TRY(upload_pixel_scenes(b));
    // every scene's trees follow the new leaf sizes from the next frame on
    A_TRY(plan_trees(b));
    A_TRY(enqueue_frame(b, stream));
    A_TRY(cudaStreamSynchronize(stream));
#undef A_TRY
    if (json_path) {
        FILE *f = fopen(json_path, "w");
        if (!f) return fail(ctx, PM_ERR_INVALID, std::string("cannot open ") + json_path);
        const bool ok = fputs(js.c_str(), f) >= 0;
        if (fclose(f) != 0 || !ok) return fail(ctx, PM_ERR_INVALID, "short write");
    }
    return PM_OK;
}

}  // extern "C"
