// query_list.cu -- the frame's radiance queries: build (count, scan, write
// per pixel) and spatial order (map, Morton code), shared by the k-NN render
// (pm_render) and the learned radiance cache.
#include "cache.cuh"
#include "phys_state.cuh"
#include "radix_sort.cuh"

#include <algorithm>

namespace pm {
namespace {

template <typename T>
cudaError_t dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, sizeof(T) * count);
}

}  // namespace

void query_list_free(QueryList &ql) {
    cudaFree(ql.cnt); cudaFree(ql.off); cudaFree(ql.scnt); cudaFree(ql.soff); cudaFree(ql.slist);
    cudaFree(ql.scan_tmp); cudaFree(ql.qa); cudaFree(ql.qd); cudaFree(ql.val);
    cudaFree(ql.key); cudaFree(ql.ord); cudaFree(ql.key_tmp); cudaFree(ql.ord_tmp);
    cudaFree(ql.hist); cudaFree(ql.n_dev); cudaFree(ql.gather_stats);
    cudaFree(ql.anchor_d); cudaFree(ql.defer_n);
    if (ql.ev0) cudaEventDestroy(ql.ev0);
    if (ql.ev1) cudaEventDestroy(ql.ev1);
    ql = QueryList();
}

cudaError_t query_list_build(PhysicalState *st, bool force, cudaStream_t s) {
    QueryList &ql = st->ql;
    const MapView surf = view_of(st->map[0]), vol = view_of(st->map[1]);
    const int flags = (vol.n > 0 ? 1 : 0) | (surf.n > 0 ? 2 : 0);
    if (!force && ql.gen == st->gen && ql.flags == flags && ql.qa) return cudaSuccess;
    cudaError_t e;
#define QL_TRY(x) do { e = (x); if (e != cudaSuccess) return e; } while (0)
    if (!ql.ev0) {
        QL_TRY(cudaEventCreate(&ql.ev0));
        QL_TRY(cudaEventCreate(&ql.ev1));
    }
    const uint32_t npix = (uint32_t)st->cfg.width * (uint32_t)st->cfg.height;
    if (npix > ql.npix_cap) {
        cudaFree(ql.cnt); cudaFree(ql.off); cudaFree(ql.scan_tmp);
        cudaFree(ql.scnt); cudaFree(ql.soff); cudaFree(ql.slist);
        ql.cnt = ql.off = ql.scan_tmp = ql.scnt = ql.soff = ql.slist = nullptr;
        ql.npix_cap = 0;
        QL_TRY(dalloc(&ql.cnt, npix));
        QL_TRY(dalloc(&ql.off, (size_t)npix + 1));
        QL_TRY(dalloc(&ql.scnt, npix));
        QL_TRY(dalloc(&ql.soff, (size_t)npix + 1));
        QL_TRY(dalloc(&ql.slist, npix));
        QL_TRY(dalloc(&ql.scan_tmp, scan_tile_count(npix) + 1));
        ql.npix_cap = npix;
    }
    const RenderParams R = render_params(st);
    QL_TRY(cudaEventRecord(ql.ev0, s));
    QL_TRY(cache_count_queries(st->dscene, R, flags & 1, flags & 2, ql.cnt, ql.scnt, s));
    QL_TRY(exclusive_scan_u32_large(ql.cnt, ql.off, npix, ql.off + npix, ql.scan_tmp, s));
    QL_TRY(exclusive_scan_u32_large(ql.scnt, ql.soff, npix, ql.soff + npix, ql.scan_tmp, s));
    uint32_t totals[2] = {0, 0};
    QL_TRY(cudaMemcpyAsync(&totals[0], ql.off + npix, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    QL_TRY(cudaMemcpyAsync(&totals[1], ql.soff + npix, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    QL_TRY(cudaStreamSynchronize(s));
    const uint32_t total = totals[0];
    if (total > ql.qcap) {
        cudaFree(ql.qa); cudaFree(ql.qd); cudaFree(ql.val);
        ql.qa = ql.qd = ql.val = nullptr;
        ql.qcap = 0;
        const uint32_t cap = total + total / 8;
        QL_TRY(dalloc(&ql.qa, cap));
        QL_TRY(dalloc(&ql.qd, cap));
        QL_TRY(dalloc(&ql.val, cap));
        ql.qcap = cap;
    }
    QL_TRY(cache_write_queries(st->dscene, R, flags & 1, flags & 2, ql.off, ql.soff, ql.qa, ql.qd,
                               ql.slist, s));
    QL_TRY(cudaEventRecord(ql.ev1, s));
    ql.nq = total;
    ql.nsurf = totals[1];
    ql.gen = st->gen;
    ql.flags = flags;
    ql.sorted = false;
    return cudaSuccess;
}

cudaError_t query_list_sort(PhysicalState *st, cudaStream_t s) {
    QueryList &ql = st->ql;
    if (ql.sorted) return cudaSuccess;
    cudaError_t e;
    const uint32_t nq = ql.nq;
    if (nq > ql.sort_cap) {
        cudaFree(ql.key); cudaFree(ql.ord); cudaFree(ql.key_tmp); cudaFree(ql.ord_tmp);
        cudaFree(ql.hist); cudaFree(ql.n_dev);
        ql.key = ql.ord = ql.key_tmp = ql.ord_tmp = ql.hist = ql.n_dev = nullptr;
        ql.sort_cap = 0;
        const uint32_t cap = ql.qcap;
        QL_TRY(dalloc(&ql.key, cap));
        QL_TRY(dalloc(&ql.ord, cap));
        QL_TRY(dalloc(&ql.key_tmp, cap));
        QL_TRY(dalloc(&ql.ord_tmp, cap));
        QL_TRY(dalloc(&ql.hist, radix_sort_hist_words(cap)));
        QL_TRY(dalloc(&ql.n_dev, 1));
        ql.sort_cap = cap;
    }
    CacheGrid box;
    box.levels = 0;
    box.log2_t = 0;
    for (int a = 0; a < 3; ++a) {
        const float ext = st->scene.box_max[a] - st->scene.box_min[a];
        const float m = 0.01f * (ext > 0.0f ? ext : 1.0f);
        box.lo[a] = st->scene.box_min[a] - m;
        const float size = ext + 2.0f * m;
        box.inv_size[a] = size > 0.0f ? 1.0f / size : 1.0f;
    }
    QL_TRY(cudaMemcpyAsync(ql.n_dev, &ql.nq, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    QL_TRY(cache_sample_keys(box, ql.qa, nullptr, nq, ql.key, ql.ord, s));
    uint32_t *ok_keys = nullptr, *ok_vals = nullptr;
    QL_TRY(radix_sort_pairs_u32(ql.key, ql.ord, ql.key_tmp, ql.ord_tmp, ql.n_dev, nq, 0, 31, ql.hist, s,
                                &ok_keys, &ok_vals));
    ql.order = ok_vals;
    ql.sorted = true;
    return cudaSuccess;
}

cudaError_t knn_values_raw(PhysicalState *st, cudaStream_t s) {
    QueryList &ql = st->ql;
    cudaError_t e;
    QL_TRY(query_list_sort(st, s));
    if (!ql.gather_stats) {
        QL_TRY(dalloc(&ql.gather_stats, kGatherStats));
        QL_TRY(dalloc(&ql.defer_n, 2));  // deferred count, chunk counter
    }
    if (tile_chunks(ql.nq, 4) > ql.anchor_cap) {
        cudaFree(ql.anchor_d);
        ql.anchor_d = nullptr;
        ql.anchor_cap = 0;
        QL_TRY(dalloc(&ql.anchor_d, tile_chunks(ql.qcap, 4)));
        ql.anchor_cap = tile_chunks(ql.qcap, 4);
    }
    QL_TRY(cudaMemsetAsync(ql.gather_stats, 0, sizeof(unsigned long long) * kGatherStats, s));
    // the sort's other index array is free again: the deferred-query list
    const TileBuffers buf{ql.anchor_d, ql.order == ql.ord ? ql.ord_tmp : ql.ord, ql.defer_n, ql.gather_stats};
    QL_TRY(knn_values_tiles(st->dscene, view_of(st->map[0]), view_of(st->map[1]), ql.qa, ql.qd, ql.order,
                            ql.nq, nullptr, 4, st->cfg.k, st->cfg.radius, true, ql.val, buf, st->sm_count,
                            s));
#undef QL_TRY
    return cudaSuccess;
}

}  // namespace pm
