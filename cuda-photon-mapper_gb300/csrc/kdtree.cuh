// kdtree.cuh -- implicit median-split kd-tree over a photon map.
#pragma once
#include "phys_common.cuh"

#include <vector>

namespace pm {

// Depth D of the tree over n records (leaves of 32 << leaf_shift records at
// depth D, 2^D leaf slots).
int tree_depth(uint32_t n, int leaf_shift = 0);
// Node array length (index 0 unused, root at 1): 2^(D+1).
size_t tree_nodes(uint32_t n, int leaf_shift = 0);

struct KdBuildArgs {
    uint32_t n;                 // records
    const uint32_t *n_dev;      // the same count in device memory
    float3 lo, hi;              // root cell (the scene box)
    const float *box_dev;       // nullable: root cell read from device memory (6 floats)
    const float4 *pos_in, *pow_in;   // records in index order (pow_in nullable)
    float4 *pos_out, *pow_out;       // records in tree order (pow_out nullable)
    float4 *dir_out = nullptr;       // nullable: decoded directions (xyz) in tree order
    float4 *node_lo, *node_hi;       // tree_nodes(n) boxes
    uint64_t *keys, *keys_tmp;       // n each
    uint32_t *vals, *vals_tmp;       // n each
    uint32_t *hist;                  // radix_sort_hist_words(n)
    uint32_t *order_out;             // nullable: tree position -> record index
    int leaf_shift = 0;              // leaves of 32 << leaf_shift records
    // multi build only (nullable): the records from *pad_count to n are set
    // to infinity (position) and zero (power) before the build
    const uint32_t *pad_count = nullptr;
};

cudaError_t build_tree(const KdBuildArgs &a, cudaStream_t s);
// The part of build_tree below the radix-sorted levels -- the subtree
// finish, the permutation into tree order and the boxes -- for a tree whose
// record order after those levels is order[0..a.n).
cudaError_t build_tree_finish(const KdBuildArgs &a, uint32_t *order, cudaStream_t s);

// Several trees built together (a batch's maps): the radix-sorted levels of
// every map in shared launches over one pooled order, then each map's
// finish (build_tree_finish). Each tree comes out as build_tree makes it.
struct KdMultiMap {           // one map, device copy
    const float4 *pos;        // records in index order
    float4 *pad_pos, *pad_pow;     // the same arrays, written by the padding
    const float4 *pow;
    float4 *pos_out, *pow_out, *dir_out;  // tree order
    const uint32_t *pad_count;     // nullable
    float4 *cell_lo, *cell_hi;
    float4 root_lo, root_hi;  // the root cell
    uint32_t n;               // records
    uint32_t base;            // first pooled position (a multiple of the sort tile)
    int depth, lf, leaf_shift;
};
struct KdMulti {
    int nmaps = 0, levels = 0;          // levels: the most radix-sorted levels of any map
    std::vector<KdMultiMap> maps;       // in build order: the most sorted levels first
    std::vector<int> index;             // build order -> the caller's map index
    KdMultiMap *desc = nullptr;
    uint32_t *tile_map = nullptr;       // per pooled tile: its map (build order)
    uint2 *seg_tab = nullptr;           // per level and pooled tile: (node's first tile, node's tiles)
    uint32_t *node_prefix = nullptr;    // per level: nmaps + 1 scanned node counts of the sorted maps
    uint32_t *level_n = nullptr;        // per level: pooled positions of the maps sorted at that level
    std::vector<uint32_t> level_tiles, level_nodes, level_maps;
    // the finish of every map at once: scanned per-map counts of subtrees,
    // leaf slots and (per level from 10 up) inner nodes
    uint32_t *fin_prefix = nullptr;     // subtrees, leaves, then one row per inner level
    uint32_t subtrees = 0, leaves = 0;
    int max_depth = 0;
    std::vector<uint32_t> inner_nodes;  // per level 10 .. max_depth - 1
    bool pad = false;                   // some map pads its records
    uint32_t total = 0;                 // pooled positions
    uint64_t *keys = nullptr, *keys_tmp = nullptr;
    uint32_t *vals = nullptr, *vals_tmp = nullptr, *hist = nullptr;
};
// Plans the build of the maps args[i] (n, pos_in, node_lo/hi, leaf_shift, lo/hi) and allocates
// its tables and pooled scratch. Maps with no records are left out.
cudaError_t kd_multi_create(const std::vector<KdBuildArgs> &args, KdMulti *k);
void kd_multi_free(KdMulti &k);
// The padding and the shared levels of every map; *order receives the
// pooled order (map i of the build order at *order + maps[i].base).
cudaError_t kd_multi_levels(KdMulti &k, cudaStream_t s, uint32_t **order);
// Every map's finish (build_tree_finish) in shared launches.
cudaError_t kd_multi_finish(KdMulti &k, uint32_t *order, cudaStream_t s);

}  // namespace pm
