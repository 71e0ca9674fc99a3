// radix_sort.cu -- stable LSD radix sort and single-CTA exclusive scan.
#include "launch_count.cuh"
#include "radix_sort.cuh"

namespace pm {
namespace {

constexpr int kScanThreads = 1024;

__device__ __forceinline__ uint32_t lanemask_lt() {
    return (1u << (threadIdx.x & 31)) - 1u;
}

// Block-wide exclusive scan of one value per thread; returns this thread's
// prefix and writes the block total to *total. blockDim.x is a multiple of 32.
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_sums, uint32_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nwarps ? warp_sums[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nwarps) warp_sums[lane] = wi - w;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    uint32_t r = warp_sums[warp] + incl - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) scan_kernel(const uint32_t *in, uint32_t *out,
                                                            uint32_t n, uint32_t *total_out) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t total;
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t lo = threadIdx.x * per;
    const uint32_t hi = min(n, lo + per);
    uint32_t s = 0;
    for (uint32_t i = lo; i < hi; ++i) s += in[i];
    uint32_t run = block_exclusive_scan(s, warp_sums, &total);
    for (uint32_t i = lo; i < hi; ++i) {
        uint32_t v = in[i];
        out[i] = run;
        run += v;
    }
    if (threadIdx.x == 0 && total_out) *total_out = total;
}

// Per-tile sums for the large scan (tile = kSortTile elements).
__global__ void __launch_bounds__(kSortThreads) tile_sum_kernel(const uint32_t *in, uint32_t n,
                                                                uint32_t *sums) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t total;
    const uint32_t base = blockIdx.x * kSortTile + threadIdx.x * kSortItems;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = base + i;
        if (idx < n) s += in[idx];
    }
    block_exclusive_scan(s, warp_sums, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// With seg_tab (per tile: the first tile of its segment, the segment's
// tiles) each segment's scan starts at 0: the tile's offset less that of
// its segment's first tile.
__global__ void __launch_bounds__(kSortThreads) tile_scan_kernel(const uint32_t *in, uint32_t *out,
                                                                 uint32_t n,
                                                                 const uint32_t *offs,
                                                                 const uint2 *seg_tab) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t total;
    const uint32_t base = blockIdx.x * kSortTile + threadIdx.x * kSortItems;
    uint32_t v[kSortItems];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = base + i;
        v[i] = idx < n ? in[idx] : 0u;
        s += v[i];
    }
    uint32_t run = block_exclusive_scan(s, warp_sums, &total) + offs[blockIdx.x];
    if (seg_tab) run -= offs[seg_tab[blockIdx.x].x];
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        uint32_t idx = base + i;
        if (idx < n) out[idx] = run;
        run += v[i];
    }
}

// Position of the (digit d, tile t) count in the scanned array: segments of
// seg consecutive tiles one after another, digit-major inside a segment, so
// that the scan keeps every segment's items inside the segment (seg >=
// ntiles: one segment, the plain digit-major order).
__device__ __forceinline__ uint32_t count_at(uint32_t d, uint32_t t, uint32_t ntiles, uint32_t seg,
                                             const uint2 *seg_tab) {
    if (seg_tab) {  // per tile: (the segment's first tile, its tiles)
        const uint2 e = seg_tab[t];
        return e.x * 256u + d * e.y + (t - e.x);
    }
    const uint32_t t0 = t / seg * seg;
    return t0 * 256u + d * min(seg, ntiles - t0) + (t - t0);
}

template <typename K>
__global__ void __launch_bounds__(kSortThreads) hist_kernel(const K *keys, const uint32_t *n_dev,
                                                            int shift, uint32_t *hist,
                                                            uint32_t ntiles, uint32_t seg,
                                                            const uint2 *seg_tab) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t n = *n_dev;
    const uint32_t base = blockIdx.x * kSortTile;
    for (uint32_t i = threadIdx.x; i < kSortTile; i += kSortThreads) {
        uint32_t idx = base + i;
        if (idx < n) atomicAdd(&h[(uint32_t)(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[count_at(threadIdx.x, blockIdx.x, ntiles, seg, seg_tab)] = h[threadIdx.x];
}

template <typename K>
__global__ void __launch_bounds__(kSortThreads) scatter_kernel(
    const K *keys_in, const uint32_t *vals_in, K *keys_out, uint32_t *vals_out,
    const uint32_t *n_dev, int shift, const uint32_t *offs, uint32_t ntiles, uint32_t seg,
    const uint2 *seg_tab) {
    constexpr int kWarps = kSortThreads / 32;
    __shared__ uint32_t run[256];
    __shared__ uint32_t wcnt[kWarps][256];
    const int warp = threadIdx.x >> 5;
    const uint32_t n = *n_dev;
    const uint32_t base = blockIdx.x * kSortTile;
    run[threadIdx.x] = offs[count_at(threadIdx.x, blockIdx.x, ntiles, seg, seg_tab)];
    for (int r = 0; r < kSortItems; ++r) {
        const uint32_t idx = base + r * kSortThreads + threadIdx.x;
        if (base + r * kSortThreads >= n) break;  // uniform across the block
#pragma unroll
        for (int w = 0; w < kWarps; ++w) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const bool valid = idx < n;
        K k = valid ? keys_in[idx] : K(0);
        uint32_t d = valid ? ((uint32_t)(k >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lanemask_lt());
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pos = run[d] + rank;
            for (int w = 0; w < warp; ++w) pos += wcnt[w][d];
            keys_out[pos] = k;
            vals_out[pos] = vals_in[idx];
        }
        __syncthreads();
        uint32_t add = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) add += wcnt[w][threadIdx.x];
        run[threadIdx.x] += add;
        __syncthreads();
    }
}

template <typename K>
cudaError_t sort_pairs(K *keys, uint32_t *vals, K *keys_tmp, uint32_t *vals_tmp,
                       const uint32_t *n_dev, uint32_t max_n, int begin_bit, int end_bit,
                       uint32_t *hist, cudaStream_t stream, K **out_keys, uint32_t **out_vals,
                       uint32_t seg_tiles, const uint2 *seg_tab) {
    K *kin = keys, *kout = keys_tmp;
    uint32_t *vin = vals, *vout = vals_tmp;
    uint32_t ntiles = (max_n + kSortTile - 1) / kSortTile;
    if (ntiles == 0) ntiles = 1;
    const uint32_t seg = seg_tiles ? seg_tiles : ntiles;
    // The digit-count scan runs in three multi-CTA steps once the histogram
    // outgrows a few tiles (always for pooled segments, so that a pool's
    // launch sequence does not depend on its size); its tile partials live
    // past the histogram.
    const uint32_t hn = 256u * ntiles;
    uint32_t *partials = hist + hn;
    for (int shift = begin_bit; shift < end_bit; shift += 8) {
        hist_kernel<K><<<ntiles, kSortThreads, 0, stream>>>(kin, n_dev, shift, hist, ntiles, seg,
                                                                        seg_tab); note_launch();
        if (hn <= kSortTile && !seg_tab) {
            scan_kernel<<<1, kScanThreads, 0, stream>>>(hist, hist, hn, nullptr); note_launch();
        } else {
            const uint32_t tiles = scan_tile_count(hn);
            tile_sum_kernel<<<tiles, kSortThreads, 0, stream>>>(hist, hn, partials); note_launch();
            scan_kernel<<<1, kScanThreads, 0, stream>>>(partials, partials, tiles, nullptr); note_launch();
            tile_scan_kernel<<<tiles, kSortThreads, 0, stream>>>(hist, hist, hn, partials, nullptr); note_launch();
        }
        scatter_kernel<K><<<ntiles, kSortThreads, 0, stream>>>(kin, vin, kout, vout, n_dev, shift,
                                                               hist, ntiles, seg, seg_tab); note_launch();
        K *tk = kin; kin = kout; kout = tk;
        uint32_t *tv = vin; vin = vout; vout = tv;
    }
    *out_keys = kin;
    *out_vals = vin;
    return cudaGetLastError();
}

}  // namespace

cudaError_t radix_sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint32_t *keys_tmp,
                                 uint32_t *vals_tmp, const uint32_t *n_dev, uint32_t max_n,
                                 int begin_bit, int end_bit, uint32_t *hist, cudaStream_t stream,
                                 uint32_t **out_keys, uint32_t **out_vals, uint32_t seg_tiles,
                                 const uint2 *seg_tab) {
    return sort_pairs<uint32_t>(keys, vals, keys_tmp, vals_tmp, n_dev, max_n, begin_bit, end_bit,
                                hist, stream, out_keys, out_vals, seg_tiles, seg_tab);
}

cudaError_t radix_sort_pairs_u64(uint64_t *keys, uint32_t *vals, uint64_t *keys_tmp,
                                 uint32_t *vals_tmp, const uint32_t *n_dev, uint32_t max_n,
                                 int begin_bit, int end_bit, uint32_t *hist, cudaStream_t stream,
                                 uint64_t **out_keys, uint32_t **out_vals, uint32_t seg_tiles,
                                 const uint2 *seg_tab) {
    return sort_pairs<uint64_t>(keys, vals, keys_tmp, vals_tmp, n_dev, max_n, begin_bit, end_bit,
                                hist, stream, out_keys, out_vals, seg_tiles, seg_tab);
}

uint32_t scan_tile_count(uint32_t n) {
    uint32_t t = (n + kSortTile - 1) / kSortTile;
    return t == 0 ? 1 : t;
}

cudaError_t exclusive_scan_u32_large(const uint32_t *in, uint32_t *out, uint32_t n,
                                     uint32_t *total, uint32_t *tmp, cudaStream_t stream) {
    if (n <= 65536) return exclusive_scan_u32(in, out, n, total, stream);
    uint32_t tiles = scan_tile_count(n);
    tile_sum_kernel<<<tiles, kSortThreads, 0, stream>>>(in, n, tmp); note_launch();
    scan_kernel<<<1, kScanThreads, 0, stream>>>(tmp, tmp, tiles, total); note_launch();
    tile_scan_kernel<<<tiles, kSortThreads, 0, stream>>>(in, out, n, tmp, nullptr); note_launch();
    return cudaGetLastError();
}

cudaError_t exclusive_scan_u32_segmented(const uint32_t *in, uint32_t *out, uint32_t n, const uint2 *seg_tab,
                                         uint32_t *tmp, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const uint32_t tiles = scan_tile_count(n);
    tile_sum_kernel<<<tiles, kSortThreads, 0, stream>>>(in, n, tmp); note_launch();
    scan_kernel<<<1, kScanThreads, 0, stream>>>(tmp, tmp, tiles, nullptr); note_launch();
    tile_scan_kernel<<<tiles, kSortThreads, 0, stream>>>(in, out, n, tmp, seg_tab); note_launch();
    return cudaGetLastError();
}

cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total,
                               cudaStream_t stream) {
    scan_kernel<<<1, kScanThreads, 0, stream>>>(in, out, n, total); note_launch();
    return cudaGetLastError();
}

}  // namespace pm
