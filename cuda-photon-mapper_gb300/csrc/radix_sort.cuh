// radix_sort.cuh -- stable LSD radix sort of (key, uint32 value) pairs and
// the exclusive scan it is built on.
//
// The element count is read from device memory, so a whole pipeline
// (count -> scan -> sort -> reduce) runs without a host round trip; max_n
// only sizes the grids. Each 8-bit pass is reduce-then-scan: a per-tile
// digit histogram, one exclusive scan over all (digit, tile) counts, and a
// scatter in which every tile ranks its items with warp match masks, so
// equal keys keep their input order.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

namespace pm {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;

// Number of uint32 words of scratch the sort needs for max_n elements: the
// digit counts of every tile plus the partial sums of their scan.
inline size_t radix_sort_hist_words(uint32_t max_n) {
    uint32_t tiles = (max_n + kSortTile - 1) / kSortTile;
    if (tiles == 0) tiles = 1;
    const size_t hn = (size_t)256 * tiles;
    return hn + (hn + kSortTile - 1) / kSortTile + 1;
}

// Sorts keys[0..n) with their values by bits [begin_bit, end_bit), n read
// from n_dev. Ping-pongs between (keys, vals) and (keys_tmp, vals_tmp);
// *out_keys / *out_vals receive whichever pair holds the result.
// hist must hold radix_sort_hist_words(max_n) words.
cudaError_t radix_sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint32_t *keys_tmp,
                                 uint32_t *vals_tmp, const uint32_t *n_dev, uint32_t max_n,
                                 int begin_bit, int end_bit, uint32_t *hist, cudaStream_t stream,
                                 uint32_t **out_keys, uint32_t **out_vals, uint32_t seg_tiles = 0,
                                 const uint2 *seg_tab = nullptr);
// With seg_tiles > 0 the items are sorted within segments of seg_tiles x
// kSortTile consecutive items (each segment keeps its place): a segmented
// sort in the passes of the segment's own bits. With seg_tab (device, one
// entry per tile: the first tile of the tile's segment and the segment's
// tile count) the segments are any runs of whole tiles.
cudaError_t radix_sort_pairs_u64(uint64_t *keys, uint32_t *vals, uint64_t *keys_tmp,
                                 uint32_t *vals_tmp, const uint32_t *n_dev, uint32_t max_n,
                                 int begin_bit, int end_bit, uint32_t *hist, cudaStream_t stream,
                                 uint64_t **out_keys, uint32_t **out_vals, uint32_t seg_tiles = 0,
                                 const uint2 *seg_tab = nullptr);

// Exclusive prefix sum of in[0..n) into out[0..n) with one CTA; the total
// goes to *total (device). n is a host value here.
cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total,
                               cudaStream_t stream);

// Exclusive prefix sum of in[0..n) for large n: per-tile sums, one scan of
// the tile sums, then per-tile scans. tmp must hold scan_tile_count(n) + 1
// words. *total (device) receives the sum.
uint32_t scan_tile_count(uint32_t n);
cudaError_t exclusive_scan_u32_large(const uint32_t *in, uint32_t *out, uint32_t n,
                                     uint32_t *total, uint32_t *tmp, cudaStream_t stream);
// The same scan restarted at every segment: the segments are runs of whole
// tiles of kSortTile items, seg_tab (device) gives per tile its segment's
// first tile and tile count, and out[i] sums in[] from the segment's first
// item up to i (exclusive). tmp: scan_tile_count(n) words. Three launches
// for any number of segments.
cudaError_t exclusive_scan_u32_segmented(const uint32_t *in, uint32_t *out, uint32_t n, const uint2 *seg_tab,
                                         uint32_t *tmp, cudaStream_t stream);

}  // namespace pm
