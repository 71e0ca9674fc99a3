// kdtree.cuh -- implicit median-split kd-tree over a photon map.
#pragma once
#include "phys_common.cuh"

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
};

cudaError_t build_tree(const KdBuildArgs &a, cudaStream_t s);

}  // namespace pm
