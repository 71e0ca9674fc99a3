// kdtree.cu -- photon-map kd-tree build.
//
// 1. 63-bit Morton code of every record (21 bits per axis over the box).
// 2. Stable LSD radix sort of (code, record index): equal codes keep
//    emission order, so the layout is deterministic.
// 3. Records permuted into sorted order (SoA float4 pos / pow).
// 4. Implicit balanced tree over the sorted sequence: every node splits its
//    range at the median, leaves hold 32 consecutive records (one warp's
//    load), node i has children 2i and 2i+1 and leaves sit at depth D. Each
//    node stores the bounding box of its records (lo, hi), built bottom-up,
//    so a query can bound the distance to everything below a node.
#include "launch_count.cuh"
#include "kdtree.cuh"
#include "radix_sort.cuh"

namespace pm {
namespace {

__global__ void morton_kernel(const float4 *__restrict__ pos, uint32_t n, float3 lo, float3 hi,
                              const float *box_dev, uint64_t *keys, uint32_t *vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (box_dev) {
        lo = make_float3(box_dev[0], box_dev[1], box_dev[2]);
        hi = make_float3(box_dev[3], box_dev[4], box_dev[5]);
    }
    float4 p = pos[i];
    uint64_t c = spread21(quantize21(p.x, lo.x, hi.x)) |
                 (spread21(quantize21(p.y, lo.y, hi.y)) << 1) |
                 (spread21(quantize21(p.z, lo.z, hi.z)) << 2);
    keys[i] = c;
    vals[i] = i;
}

__global__ void permute_kernel(const uint32_t *__restrict__ order, uint32_t n,
                               const float4 *__restrict__ pos_in, const float4 *__restrict__ pow_in,
                               float4 *pos_out, float4 *pow_out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = order[i];
    pos_out[i] = pos_in[s];
    if (pow_in) pow_out[i] = pow_in[s];
}

// One warp per leaf slot: box of its (up to) 32 records.
__global__ void leaf_box_kernel(const float4 *__restrict__ pos, uint32_t n, uint32_t first_leaf,
                                uint32_t leaf_slots, float4 *node_lo, float4 *node_hi) {
    uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (warp >= leaf_slots) return;
    uint32_t r = warp * 32u + lane;
    const float inf = __int_as_float(0x7f800000);
    float lx = inf, ly = inf, lz = inf, hx = -inf, hy = -inf, hz = -inf;
    if (r < n) {
        float4 p = pos[r];
        lx = hx = p.x; ly = hy = p.y; lz = hz = p.z;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
        ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
        lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
        hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
        hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
        hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
    }
    if (lane == 0) {
        node_lo[first_leaf + warp] = make_float4(lx, ly, lz, 0.0f);
        node_hi[first_leaf + warp] = make_float4(hx, hy, hz, 0.0f);
    }
}

__global__ void inner_box_kernel(uint32_t first, uint32_t count, float4 *node_lo, float4 *node_hi) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint32_t nd = first + i;
    float4 a = node_lo[2 * nd], b = node_lo[2 * nd + 1];
    float4 c = node_hi[2 * nd], d = node_hi[2 * nd + 1];
    node_lo[nd] = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
    node_hi[nd] = make_float4(fmaxf(c.x, d.x), fmaxf(c.y, d.y), fmaxf(c.z, d.z), 0.0f);
}

// Small levels: one CTA walks the top of the tree level by level.
__global__ void top_box_kernel(uint32_t levels, float4 *node_lo, float4 *node_hi) {
    for (int l = (int)levels - 1; l >= 0; --l) {
        uint32_t first = 1u << l;
        for (uint32_t i = threadIdx.x; i < first; i += blockDim.x) {
            uint32_t nd = first + i;
            float4 a = node_lo[2 * nd], b = node_lo[2 * nd + 1];
            float4 c = node_hi[2 * nd], d = node_hi[2 * nd + 1];
            node_lo[nd] = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
            node_hi[nd] = make_float4(fmaxf(c.x, d.x), fmaxf(c.y, d.y), fmaxf(c.z, d.z), 0.0f);
        }
        __syncthreads();
    }
}

}  // namespace

int tree_depth(uint32_t n) {
    uint32_t leaves = (n + 31) / 32;
    int d = 0;
    while ((1u << d) < leaves) ++d;
    return d;
}

size_t tree_nodes(uint32_t n) { return (size_t)2 << tree_depth(n); }

cudaError_t build_tree(const KdBuildArgs &a, cudaStream_t s) {
    const uint32_t n = a.n;
    if (n == 0) return cudaSuccess;
    morton_kernel<<<(n + 255) / 256, 256, 0, s>>>(a.pos_in, n, a.lo, a.hi, a.box_dev, a.keys,
                                                   a.vals); note_launch();
    uint64_t *sk = nullptr;
    uint32_t *sv = nullptr;
    cudaError_t e = radix_sort_pairs_u64(a.keys, a.vals, a.keys_tmp, a.vals_tmp, a.n_dev, n, 0, 64,
                                         a.hist, s, &sk, &sv);
    if (e != cudaSuccess) return e;
    permute_kernel<<<(n + 255) / 256, 256, 0, s>>>(sv, n, a.pos_in, a.pow_in, a.pos_out, a.pow_out); note_launch();
    const int D = tree_depth(n);
    const uint32_t first_leaf = 1u << D;
    leaf_box_kernel<<<(first_leaf * 32 + 255) / 256, 256, 0, s>>>(a.pos_out, n, first_leaf, first_leaf,
                                                                 a.node_lo, a.node_hi); note_launch();
    // Wide levels one launch each; the top 10 levels in a single CTA.
    int l = D - 1;
    for (; l >= 10; --l) {
        uint32_t first = 1u << l;
        inner_box_kernel<<<(first + 255) / 256, 256, 0, s>>>(first, first, a.node_lo, a.node_hi); note_launch();
    }
    if (l >= 0) {
        top_box_kernel<<<1, 1024, 0, s>>>((uint32_t)(l + 1), a.node_lo, a.node_hi);
        note_launch();
    }
    if (a.order_out) {
        e = cudaMemcpyAsync(a.order_out, sv, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

}  // namespace pm
