// kdtree.cu -- photon-map kd-tree build.
//
// Implicit left-balanced kd-tree: node i has children 2i and 2i+1, leaves
// hold L = 32 << leaf_shift consecutive records (one or more warp-wide
// loads) at depth D, and the node at level l covers records
// [j*L*2^(D-l), (j+1)*L*2^(D-l)) of the final order (j = its index within
// the level), so no child pointers or ranges are stored.
//
// Top-down, one level at a time, all nodes of the level in parallel: every
// record gets the key (node within the level, coordinate along the longest
// axis of its node's cell, quantised to 16 bits of the cell), a stable LSD
// radix sort orders the records by it -- which leaves each node's records
// sorted along that axis, so the node's first half (the left child) is the
// lower half: a median split -- and each child's cell is its parent's cell
// cut at the coordinate of the right child's first record. Equal keys keep their previous order, so the layout is
// deterministic. The records are then permuted into that order (SoA float4
// pos / pow) and every node gets the tight bounding box of its records,
// bottom-up, which is what a query tests. The cells live in the node box
// arrays until the boxes overwrite them.
#include "launch_count.cuh"
#include "kdtree.cuh"
#include "radix_sort.cuh"

#include <algorithm>
#include <cstring>

namespace pm {
namespace {

__device__ __forceinline__ int longest_axis(float4 lo, float4 hi) {
    const float ex = hi.x - lo.x, ey = hi.y - lo.y, ez = hi.z - lo.z;
    return (ex >= ey && ex >= ez) ? 0 : (ey >= ez ? 1 : 2);
}

__global__ void root_cell_kernel(float3 lo, float3 hi, const float *box_dev, float4 *cell_lo,
                                 float4 *cell_hi) {
    if (box_dev) {
        lo = make_float3(box_dev[0], box_dev[1], box_dev[2]);
        hi = make_float3(box_dev[3], box_dev[4], box_dev[5]);
    }
    cell_lo[1] = make_float4(lo.x, lo.y, lo.z, 0.0f);
    cell_hi[1] = make_float4(hi.x, hi.y, hi.z, 0.0f);
}

// Key of record position i at level l: (node within the level, coordinate
// along the longest axis of the node's cell, quantised to 16 bits of the
// cell's extent). Records that quantise alike keep their previous order.
__global__ void split_key_kernel(const float4 *__restrict__ pos, const uint32_t *__restrict__ order,
                                 uint32_t n, int level, uint32_t span,
                                 const float4 *__restrict__ cell_lo,
                                 const float4 *__restrict__ cell_hi, uint64_t *keys,
                                 uint32_t *vals_init) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t node = i / span;
    const uint32_t g = (1u << level) + node;
    const float4 lo = cell_lo[g], hi = cell_hi[g];
    const int ax = longest_axis(lo, hi);
    uint32_t src = i;
    if (order) src = order[i];
    else vals_init[i] = i;
    const float4 p = pos[src];
    const float c = ax == 0 ? p.x : (ax == 1 ? p.y : p.z);
    const float l0 = ax == 0 ? lo.x : (ax == 1 ? lo.y : lo.z);
    const float l1 = ax == 0 ? hi.x : (ax == 1 ? hi.y : hi.z);
    const float f = (c - l0) / (l1 - l0) * 65536.0f;
    const uint32_t qc = !(f > 0.0f) ? 0u : (f >= 65535.0f ? 65535u : (uint32_t)f);
    keys[i] = ((uint64_t)node << 16) | qc;
}

// Children cells of every node at `level`: the parent's cell cut at the
// coordinate of the right child's first record.
__global__ void split_cell_kernel(const float4 *__restrict__ pos, const uint32_t *__restrict__ order,
                                  uint32_t n, int level, uint32_t span, uint32_t nodes,
                                  float4 *cell_lo, float4 *cell_hi) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nodes) return;
    const uint32_t g = (1u << level) + j;
    const float4 lo = cell_lo[g], hi = cell_hi[g];
    const uint32_t start = j * span, half = span >> 1;
    const uint32_t cnt = min(span, n - start);
    float4 llo = lo, lhi = hi, rlo = lo, rhi = hi;
    if (cnt > half) {
        const int ax = longest_axis(lo, hi);
        const float4 p = pos[order[start + half]];
        const float m = ax == 0 ? p.x : (ax == 1 ? p.y : p.z);
        if (ax == 0) { lhi.x = m; rlo.x = m; }
        else if (ax == 1) { lhi.y = m; rlo.y = m; }
        else { lhi.z = m; rlo.z = m; }
    }
    cell_lo[2 * g] = llo;
    cell_hi[2 * g] = lhi;
    cell_lo[2 * g + 1] = rlo;
    cell_hi[2 * g + 1] = rhi;
}

// The levels below a node of at most kSubtreeMax records are finished by
// one CTA in shared memory: per level, a bitonic sort of the composite keys
// (node within the subtree, the same 16-bit quantised coordinate as
// split_key_kernel, position before the level) -- exactly the order of the
// global stable sort by (node, coordinate) -- then the children's cells cut
// at the coordinate of each node's right half's first record, as
// split_cell_kernel does. The tree comes out identical; the deep levels,
// whose global sorts carry the most node bits, cost one pass over the
// records instead of several per level.
constexpr int kSubtreeMax = 2048;
constexpr int kSubtreeThreads = 512;
constexpr int kSubtreeNodes = kSubtreeMax / 32;  // nodes of a subtree level (leaves of >= 32)

struct SubtreeScratch {
    uint64_t key[kSubtreeMax];
    float4 p[kSubtreeMax];
    uint32_t idx[kSubtreeMax];
    float4 clo[2][2 * kSubtreeNodes], chi[2][2 * kSubtreeNodes];
};

extern __shared__ __align__(16) unsigned char subtree_smem[];

// Subtree j of a tree (the node j at level l0); one CTA.
__device__ __forceinline__ void subtree_finish(const float4 *__restrict__ pos, uint32_t *order, uint32_t n, int l0,
                                               int D, uint32_t span0, const float4 *__restrict__ cell_lo,
                                               const float4 *__restrict__ cell_hi, uint32_t j) {
    SubtreeScratch &ss = *reinterpret_cast<SubtreeScratch *>(subtree_smem);
    const uint32_t start = j * span0;
    if (start >= n) return;
    const int cnt = (int)min(span0, n - start);
    const int tid = threadIdx.x;
    for (int t = tid; t < cnt; t += blockDim.x) {
        const uint32_t r = order[start + t];
        ss.idx[t] = r;
        ss.p[t] = pos[r];
    }
    if (tid == 0) {
        ss.clo[0][0] = cell_lo[(1u << l0) + j];
        ss.chi[0][0] = cell_hi[(1u << l0) + j];
    }
    int P = 2;
    while (P < cnt) P <<= 1;
    int cur = 0;
    __syncthreads();
    for (int l = l0; l < D; ++l) {
        const int nspan = (int)(span0 >> (l - l0));  // records per node at this level
        // keys
        for (int t = tid; t < P; t += blockDim.x) {
            uint64_t key = ~0ull;
            if (t < cnt) {
                const int node = t / nspan;
                const float4 lo = ss.clo[cur][node], hi = ss.chi[cur][node];
                const int ax = longest_axis(lo, hi);
                const float4 q = ss.p[t];
                const float c = ax == 0 ? q.x : (ax == 1 ? q.y : q.z);
                const float c0 = ax == 0 ? lo.x : (ax == 1 ? lo.y : lo.z);
                const float c1 = ax == 0 ? hi.x : (ax == 1 ? hi.y : hi.z);
                const float f = (c - c0) / (c1 - c0) * 65536.0f;
                const uint32_t qc = !(f > 0.0f) ? 0u : (f >= 65535.0f ? 65535u : (uint32_t)f);
                key = ((uint64_t)node << 48) | ((uint64_t)qc << 32) | (uint32_t)t;
            }
            ss.key[t] = key;
        }
        __syncthreads();
        for (int size = 2; size <= P; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int t = tid; t < (P >> 1); t += blockDim.x) {
                    const int i = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
                    const int k = i + stride;
                    const bool up = (i & size) == 0;
                    const uint64_t a = ss.key[i], b = ss.key[k];
                    if ((a > b) == up) {
                        ss.key[i] = b;
                        ss.key[k] = a;
                    }
                }
                __syncthreads();
            }
        }
        // the records in the new order
        float4 np[kSubtreeMax / kSubtreeThreads];
        uint32_t ni[kSubtreeMax / kSubtreeThreads];
#pragma unroll
        for (int u = 0; u < kSubtreeMax / kSubtreeThreads; ++u) {
            const int t = tid + u * kSubtreeThreads;
            if (t < cnt) {
                const uint32_t old = (uint32_t)ss.key[t];
                np[u] = ss.p[old];
                ni[u] = ss.idx[old];
            }
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < kSubtreeMax / kSubtreeThreads; ++u) {
            const int t = tid + u * kSubtreeThreads;
            if (t < cnt) {
                ss.p[t] = np[u];
                ss.idx[t] = ni[u];
            }
        }
        __syncthreads();
        // the children's cells
        const int nodes = (cnt + nspan - 1) / nspan, half = nspan >> 1;
        for (int node = tid; node < nodes; node += blockDim.x) {
            const float4 lo = ss.clo[cur][node], hi = ss.chi[cur][node];
            float4 llo = lo, lhi = hi, rlo = lo, rhi = hi;
            const int ncnt = min(nspan, cnt - node * nspan);
            if (ncnt > half) {
                const int ax = longest_axis(lo, hi);
                const float4 q = ss.p[node * nspan + half];
                const float m = ax == 0 ? q.x : (ax == 1 ? q.y : q.z);
                if (ax == 0) { lhi.x = m; rlo.x = m; }
                else if (ax == 1) { lhi.y = m; rlo.y = m; }
                else { lhi.z = m; rlo.z = m; }
            }
            ss.clo[cur ^ 1][2 * node] = llo;
            ss.chi[cur ^ 1][2 * node] = lhi;
            ss.clo[cur ^ 1][2 * node + 1] = rlo;
            ss.chi[cur ^ 1][2 * node + 1] = rhi;
        }
        __syncthreads();
        cur ^= 1;
    }
    for (int t = tid; t < cnt; t += blockDim.x) order[start + t] = ss.idx[t];
}

__global__ void __launch_bounds__(kSubtreeThreads)
    subtree_finish_kernel(const float4 *__restrict__ pos, uint32_t *order, uint32_t n, int l0, int D,
                          uint32_t span0, const float4 *__restrict__ cell_lo,
                          const float4 *__restrict__ cell_hi) {
    subtree_finish(pos, order, n, l0, D, span0, cell_lo, cell_hi, blockIdx.x);
}

__global__ void iota_kernel(uint32_t *v, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

__device__ __forceinline__ void permute_one(const uint32_t *__restrict__ order, uint32_t i,
                                            const float4 *__restrict__ pos_in, const float4 *__restrict__ pow_in,
                                            float4 *pos_out, float4 *pow_out, float4 *dir_out) {
    uint32_t s = order[i];
    pos_out[i] = pos_in[s];
    if (pow_in) {
        const float4 pw = pow_in[s];
        pow_out[i] = pw;
        if (dir_out) {
            const v3 d = oct_decode(__float_as_uint(pw.w));
            dir_out[i] = make_float4(d.x, d.y, d.z, 0.0f);
        }
    }
}

__global__ void permute_kernel(const uint32_t *__restrict__ order, uint32_t n,
                               const float4 *__restrict__ pos_in, const float4 *__restrict__ pow_in,
                               float4 *pos_out, float4 *pow_out, float4 *dir_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) permute_one(order, i, pos_in, pow_in, pos_out, pow_out, dir_out);
}

// One warp per leaf slot: box of its (up to) 32 << leaf_shift records.
// Leaf slot `warp` of a tree: one warp.
__device__ __forceinline__ void leaf_box(const float4 *__restrict__ pos, uint32_t n, uint32_t first_leaf,
                                         int leaf_shift, float4 *node_lo, float4 *node_hi, uint32_t warp) {
    int lane = threadIdx.x & 31;
    const float inf = __int_as_float(0x7f800000);
    float lx = inf, ly = inf, lz = inf, hx = -inf, hy = -inf, hz = -inf;
    for (int c = 0; c < (1 << leaf_shift); ++c) {
        const uint32_t r = (warp << (5 + leaf_shift)) + ((uint32_t)c << 5) + lane;
        if (r < n) {
            float4 p = pos[r];
            lx = fminf(lx, p.x); ly = fminf(ly, p.y); lz = fminf(lz, p.z);
            hx = fmaxf(hx, p.x); hy = fmaxf(hy, p.y); hz = fmaxf(hz, p.z);
        }
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

__global__ void leaf_box_kernel(const float4 *__restrict__ pos, uint32_t n, uint32_t first_leaf,
                                uint32_t leaf_slots, int leaf_shift, float4 *node_lo,
                                float4 *node_hi) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp < leaf_slots) leaf_box(pos, n, first_leaf, leaf_shift, node_lo, node_hi, warp);
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
__device__ __forceinline__ void top_box(uint32_t levels, float4 *node_lo, float4 *node_hi) {
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

__global__ void top_box_kernel(uint32_t levels, float4 *node_lo, float4 *node_hi) {
    top_box(levels, node_lo, node_hi);
}


// ---- several maps at once (KdMulti) ----

// Pooled position i: the map (build order) and the position within it.
__device__ __forceinline__ int multi_map(const uint32_t *tile_map, uint32_t i) { return (int)tile_map[i / kSortTile]; }

__global__ void multi_init_kernel(const KdMultiMap *maps, const uint32_t *tile_map, uint32_t total,
                                  uint32_t *vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    vals[i] = i - maps[multi_map(tile_map, i)].base;
}

__global__ void multi_root_kernel(const KdMultiMap *maps, int nmaps) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmaps || maps[m].depth == 0) return;
    maps[m].cell_lo[1] = maps[m].root_lo;
    maps[m].cell_hi[1] = maps[m].root_hi;
}

// split_key_kernel over the pooled positions of the maps sorted at `level`;
// positions past a map's records (the padding of its last tile) get the
// largest key, so the stable sort keeps them at the end of their node.
__global__ void split_key_multi_kernel(const KdMultiMap *maps, const uint32_t *tile_map, uint32_t total,
                                       int level, const uint32_t *order, uint64_t *keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const KdMultiMap &m = maps[multi_map(tile_map, i)];
    const uint32_t j = i - m.base;
    if (j >= m.n) {
        keys[i] = 0xffffu;
        return;
    }
    const uint32_t span = (32u << m.leaf_shift) << (m.depth - level);
    const uint32_t node = j / span;
    const uint32_t g = (1u << level) + node;
    const float4 lo = m.cell_lo[g], hi = m.cell_hi[g];
    const int ax = longest_axis(lo, hi);
    const float4 p = m.pos[order[i]];
    const float c = ax == 0 ? p.x : (ax == 1 ? p.y : p.z);
    const float l0 = ax == 0 ? lo.x : (ax == 1 ? lo.y : lo.z);
    const float l1 = ax == 0 ? hi.x : (ax == 1 ? hi.y : hi.z);
    const float f = (c - l0) / (l1 - l0) * 65536.0f;
    const uint32_t qc = !(f > 0.0f) ? 0u : (f >= 65535.0f ? 65535u : (uint32_t)f);
    keys[i] = ((uint64_t)node << 16) | qc;
}

// split_cell_kernel over the nodes of every map sorted at `level`
// (prefix: nmaps + 1 scanned node counts).
__global__ void split_cell_multi_kernel(const KdMultiMap *maps, int nmaps, const uint32_t *prefix,
                                        int level, const uint32_t *order) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= prefix[nmaps]) return;
    int lo_m = 0, hi_m = nmaps - 1;  // the last map whose prefix <= u
    while (lo_m < hi_m) {
        const int mid = (lo_m + hi_m + 1) >> 1;
        if (prefix[mid] <= u) lo_m = mid; else hi_m = mid - 1;
    }
    const KdMultiMap &m = maps[lo_m];
    const uint32_t j = u - prefix[lo_m];
    const uint32_t span = (32u << m.leaf_shift) << (m.depth - level);
    const uint32_t g = (1u << level) + j;
    const float4 lo = m.cell_lo[g], hi = m.cell_hi[g];
    const uint32_t start = j * span, half = span >> 1;
    const uint32_t cnt = min(span, m.n - start);
    float4 llo = lo, lhi = hi, rlo = lo, rhi = hi;
    if (cnt > half) {
        const int ax = longest_axis(lo, hi);
        const float4 p = m.pos[order[m.base + start + half]];
        const float c = ax == 0 ? p.x : (ax == 1 ? p.y : p.z);
        if (ax == 0) { lhi.x = c; rlo.x = c; }
        else if (ax == 1) { lhi.y = c; rlo.y = c; }
        else { lhi.z = c; rlo.z = c; }
    }
    m.cell_lo[2 * g] = llo;
    m.cell_hi[2 * g] = lhi;
    m.cell_lo[2 * g + 1] = rlo;
    m.cell_hi[2 * g + 1] = rhi;
}


// The last map m with prefix[m] <= u (prefix: nmaps + 1 scanned counts).
__device__ __forceinline__ int map_at(const uint32_t *prefix, int nmaps, uint32_t u) {
    int lo = 0, hi = nmaps - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= u) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void multi_pad_kernel(const KdMultiMap *maps, const uint32_t *tile_map, uint32_t total) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const KdMultiMap &m = maps[multi_map(tile_map, i)];
    const uint32_t j = i - m.base;
    if (!m.pad_count || j >= m.n || j < *m.pad_count) return;
    const float inf = __int_as_float(0x7f800000);
    m.pad_pos[j] = make_float4(inf, inf, inf, __uint_as_float(j));
    m.pad_pow[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void __launch_bounds__(kSubtreeThreads)
    multi_subtree_kernel(const KdMultiMap *maps, int nmaps, const uint32_t *prefix, uint32_t *order) {
    const KdMultiMap &m = maps[map_at(prefix, nmaps, blockIdx.x)];
    const uint32_t span0 = (32u << m.leaf_shift) << (m.depth - m.lf);
    subtree_finish(m.pos, order + m.base, m.n, m.lf, m.depth, span0, m.cell_lo, m.cell_hi,
                   blockIdx.x - prefix[map_at(prefix, nmaps, blockIdx.x)]);
}

__global__ void multi_permute_kernel(const KdMultiMap *maps, const uint32_t *tile_map, uint32_t total,
                                     const uint32_t *order) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const KdMultiMap &m = maps[multi_map(tile_map, i)];
    const uint32_t j = i - m.base;
    if (j < m.n) permute_one(order + m.base, j, m.pos, m.pow, m.pos_out, m.pow_out, m.dir_out);
}

__global__ void multi_leaf_kernel(const KdMultiMap *maps, int nmaps, const uint32_t *prefix) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= prefix[nmaps]) return;  // whole warps
    const int mi = map_at(prefix, nmaps, w);
    const KdMultiMap &m = maps[mi];
    leaf_box(m.pos_out, m.n, 1u << m.depth, m.leaf_shift, m.cell_lo, m.cell_hi, w - prefix[mi]);
}

__global__ void multi_inner_kernel(const KdMultiMap *maps, int nmaps, const uint32_t *prefix, int level) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= prefix[nmaps]) return;
    const int mi = map_at(prefix, nmaps, u);
    const KdMultiMap &m = maps[mi];
    const uint32_t nd = (1u << level) + (u - prefix[mi]);
    const float4 a = m.cell_lo[2 * nd], b = m.cell_lo[2 * nd + 1];
    const float4 c = m.cell_hi[2 * nd], d = m.cell_hi[2 * nd + 1];
    m.cell_lo[nd] = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
    m.cell_hi[nd] = make_float4(fmaxf(c.x, d.x), fmaxf(c.y, d.y), fmaxf(c.z, d.z), 0.0f);
}

__global__ void multi_top_kernel(const KdMultiMap *maps) {
    const KdMultiMap &m = maps[blockIdx.x];
    top_box((uint32_t)min(m.depth, 10), m.cell_lo, m.cell_hi);
}
}  // namespace

int tree_depth(uint32_t n, int leaf_shift) {
    const uint32_t leaf = 32u << leaf_shift;
    uint32_t leaves = (uint32_t)(((uint64_t)n + leaf - 1) / leaf);
    int d = 0;
    while ((1u << d) < leaves) ++d;
    return d;
}

size_t tree_nodes(uint32_t n, int leaf_shift) { return (size_t)2 << tree_depth(n, leaf_shift); }

// The first level finished per subtree in shared memory: nodes of at most
// kSubtreeMax records.
int first_finish_level(int D, uint32_t leaf) {
    int lf = D;
    while (lf > 0 && ((uint64_t)leaf << (D - (lf - 1))) <= (uint64_t)kSubtreeMax) --lf;
    return lf;
}

cudaError_t build_tree(const KdBuildArgs &a, cudaStream_t s) {
    const uint32_t n = a.n;
    if (n == 0) return cudaSuccess;
    const int D = tree_depth(n, a.leaf_shift);
    const uint32_t blocks = (n + 255) / 256;
    // Top-down median splits; the current order ping-pongs between the two
    // (keys, vals) buffer pairs of the sort.
    uint64_t *ka = a.keys, *kb = a.keys_tmp;
    uint32_t *va = a.vals, *vb = a.vals_tmp;
    cudaError_t e;
    if (D == 0) {
        iota_kernel<<<blocks, 256, 0, s>>>(va, n); note_launch();
    } else {
        root_cell_kernel<<<1, 1, 0, s>>>(a.lo, a.hi, a.box_dev, a.node_lo, a.node_hi); note_launch();
    }
    // levels [lf, D) are finished per subtree in shared memory
    const uint32_t leaf = 32u << a.leaf_shift;
    const int lf = first_finish_level(D, leaf);
    if (lf == 0 && D > 0) {
        iota_kernel<<<blocks, 256, 0, s>>>(va, n);
        note_launch();
    }
    for (int l = 0; l < lf; ++l) {
        const uint32_t span = (32u << a.leaf_shift) << (D - l);
        const uint32_t nodes = (n + span - 1) / span;
        split_key_kernel<<<blocks, 256, 0, s>>>(a.pos_in, l == 0 ? nullptr : va, n, l, span,
                                                a.node_lo, a.node_hi, ka, va); note_launch();
        int node_bits = 0;
        while ((1u << node_bits) < nodes) ++node_bits;
        uint64_t *ko = nullptr;
        uint32_t *vo = nullptr;
        // the records are grouped by node already (a node is a fixed range of
        // positions, a whole number of sort tiles at these levels): sort each
        // node's range by its 16-bit coordinate alone
        e = span % kSortTile == 0
                ? radix_sort_pairs_u64(ka, va, kb, vb, a.n_dev, n, 0, 16, a.hist, s, &ko, &vo, span / kSortTile)
                : radix_sort_pairs_u64(ka, va, kb, vb, a.n_dev, n, 0, 16 + node_bits, a.hist, s, &ko, &vo);
        if (e != cudaSuccess) return e;
        if (vo != va) {
            uint64_t *tk = ka; ka = kb; kb = tk;
            uint32_t *tv = va; va = vb; vb = tv;
        }
        split_cell_kernel<<<(nodes + 255) / 256, 256, 0, s>>>(a.pos_in, va, n, l, span, nodes,
                                                               a.node_lo, a.node_hi); note_launch();
    }
    return build_tree_finish(a, va, s);
}

cudaError_t build_tree_finish(const KdBuildArgs &a, uint32_t *va, cudaStream_t s) {
    const uint32_t n = a.n;
    if (n == 0) return cudaSuccess;
    const int D = tree_depth(n, a.leaf_shift);
    const uint32_t blocks = (n + 255) / 256;
    const uint32_t leaf = 32u << a.leaf_shift;
    const int lf = first_finish_level(D, leaf);
    cudaError_t e;
    if (lf < D) {
        const uint32_t span = leaf << (D - lf);
        const uint32_t nodes = (n + span - 1) / span;
        const int smem = (int)sizeof(SubtreeScratch);
        e = cudaFuncSetAttribute(subtree_finish_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        subtree_finish_kernel<<<nodes, kSubtreeThreads, smem, s>>>(a.pos_in, va, n, lf, D, span, a.node_lo,
                                                                   a.node_hi);
        note_launch();
    }
    permute_kernel<<<blocks, 256, 0, s>>>(va, n, a.pos_in, a.pow_in, a.pos_out, a.pow_out, a.dir_out);
    note_launch();
    const uint32_t first_leaf = 1u << D;
    leaf_box_kernel<<<(first_leaf * 32 + 255) / 256, 256, 0, s>>>(a.pos_out, n, first_leaf, first_leaf,
                                                                 a.leaf_shift, a.node_lo, a.node_hi);
    note_launch();
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
        e = cudaMemcpyAsync(a.order_out, va, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

namespace {
template <typename T>
cudaError_t kd_alloc(T **p, size_t count) {
    *p = nullptr;
    return cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
}
}  // namespace

cudaError_t kd_multi_create(const std::vector<KdBuildArgs> &args, KdMulti *k) {
    *k = KdMulti();
    std::vector<int> idx;
    for (int i = 0; i < (int)args.size(); ++i)
        if (args[i].n > 0) idx.push_back(i);
    auto lf_of = [&](int i) {
        const int D = tree_depth(args[i].n, args[i].leaf_shift);
        return first_finish_level(D, 32u << args[i].leaf_shift);
    };
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return lf_of(a) > lf_of(b); });
    uint32_t tiles = 0;
    for (int i : idx) {
        const KdBuildArgs &a = args[i];
        KdMultiMap m;
        memset(&m, 0, sizeof(m));
        m.pos = a.pos_in;
        m.cell_lo = a.node_lo;
        m.cell_hi = a.node_hi;
        m.root_lo = make_float4(a.lo.x, a.lo.y, a.lo.z, 0.0f);
        m.root_hi = make_float4(a.hi.x, a.hi.y, a.hi.z, 0.0f);
        m.n = a.n;
        m.base = tiles * kSortTile;
        m.depth = tree_depth(a.n, a.leaf_shift);
        m.lf = lf_of(i);
        m.leaf_shift = a.leaf_shift;
        m.pad_pos = const_cast<float4 *>(a.pos_in);
        m.pad_pow = const_cast<float4 *>(a.pow_in);
        m.pow = a.pow_in;
        m.pos_out = a.pos_out;
        m.pow_out = a.pow_out;
        m.dir_out = a.dir_out;
        m.pad_count = a.pad_count;
        if (a.pad_count) k->pad = true;
        tiles += (a.n + kSortTile - 1) / kSortTile;
        k->levels = std::max(k->levels, m.lf);
        k->maps.push_back(m);
        k->index.push_back(i);
    }
    k->nmaps = (int)k->maps.size();
    k->total = tiles * kSortTile;
    const int L = std::max(k->levels, 1);
    std::vector<uint32_t> tile_map(std::max<uint32_t>(tiles, 1), 0);
    std::vector<uint2> seg((size_t)L * std::max<uint32_t>(tiles, 1), make_uint2(0, 1));
    std::vector<uint32_t> prefix((size_t)L * (k->nmaps + 1), 0);
    std::vector<uint32_t> level_n(L, 0);
    for (int mi = 0; mi < k->nmaps; ++mi) {
        const KdMultiMap &m = k->maps[mi];
        const uint32_t t0 = m.base / kSortTile, nt = (m.n + kSortTile - 1) / kSortTile;
        for (uint32_t t = 0; t < nt; ++t) tile_map[t0 + t] = (uint32_t)mi;
    }
    k->level_tiles.assign(L, 0);
    k->level_nodes.assign(L, 0);
    k->level_maps.assign(L, 0);
    for (int l = 0; l < k->levels; ++l) {
        uint32_t nodes = 0;
        for (int mi = 0; mi < k->nmaps; ++mi) {
            const KdMultiMap &m = k->maps[mi];
            prefix[(size_t)l * (k->nmaps + 1) + mi] = nodes;
            if (l >= m.lf) continue;  // maps sorted by lf: the rest are finished
            const uint32_t span = (32u << m.leaf_shift) << (m.depth - l);
            const uint32_t t0 = m.base / kSortTile, nt = (m.n + kSortTile - 1) / kSortTile;
            const uint32_t st = span / kSortTile;  // whole tiles at the sorted levels
            for (uint32_t t = 0; t < nt; ++t) {
                const uint32_t first = t / st * st;
                seg[(size_t)l * tiles + t0 + t] = make_uint2(t0 + first, std::min(st, nt - first));
            }
            nodes += (m.n + span - 1) / span;
            k->level_tiles[l] = t0 + nt;
            k->level_maps[l] = (uint32_t)(mi + 1);
        }
        prefix[(size_t)l * (k->nmaps + 1) + k->nmaps] = nodes;
        k->level_nodes[l] = nodes;
        level_n[l] = k->level_tiles[l] * kSortTile;
    }
    // the finish tables: subtrees, leaf slots, inner nodes of levels 10 ..
    const int nm1 = k->nmaps + 1;
    for (const KdMultiMap &m : k->maps) k->max_depth = std::max(k->max_depth, m.depth);
    const int inner_levels = std::max(k->max_depth - 10, 0);
    std::vector<uint32_t> fin((size_t)(2 + inner_levels) * nm1, 0);
    k->inner_nodes.assign(inner_levels, 0);
    uint32_t subs = 0, leaves = 0;
    std::vector<uint32_t> inner(inner_levels, 0);
    for (int mi = 0; mi < k->nmaps; ++mi) {
        const KdMultiMap &m = k->maps[mi];
        fin[mi] = subs;
        fin[nm1 + mi] = leaves;
        if (m.lf < m.depth) {
            const uint32_t span0 = (32u << m.leaf_shift) << (m.depth - m.lf);
            subs += (m.n + span0 - 1) / span0;
        }
        leaves += 1u << m.depth;
        for (int l = 10; l < m.depth; ++l) {
            fin[(size_t)(2 + l - 10) * nm1 + mi] = inner[l - 10];
            inner[l - 10] += 1u << l;
        }
        for (int l = std::max(m.depth, 10); l < k->max_depth; ++l) fin[(size_t)(2 + l - 10) * nm1 + mi] = inner[l - 10];
    }
    fin[k->nmaps] = subs;
    fin[nm1 + k->nmaps] = leaves;
    for (int l = 0; l < inner_levels; ++l) {
        fin[(size_t)(2 + l) * nm1 + k->nmaps] = inner[l];
        k->inner_nodes[l] = inner[l];
    }
    k->subtrees = subs;
    k->leaves = leaves;
    cudaError_t e;
#define KM_TRY(x) do { e = (x); if (e != cudaSuccess) { kd_multi_free(*k); return e; } } while (0)
    KM_TRY(kd_alloc(&k->fin_prefix, fin.size()));
    KM_TRY(cudaMemcpy(k->fin_prefix, fin.data(), sizeof(uint32_t) * fin.size(), cudaMemcpyHostToDevice));
    KM_TRY(kd_alloc(&k->desc, k->nmaps));
    KM_TRY(kd_alloc(&k->tile_map, tile_map.size()));
    KM_TRY(kd_alloc(&k->seg_tab, seg.size()));
    KM_TRY(kd_alloc(&k->node_prefix, prefix.size()));
    KM_TRY(kd_alloc(&k->level_n, level_n.size()));
    KM_TRY(kd_alloc(&k->keys, k->total));
    KM_TRY(kd_alloc(&k->keys_tmp, k->total));
    KM_TRY(kd_alloc(&k->vals, k->total));
    KM_TRY(kd_alloc(&k->vals_tmp, k->total));
    KM_TRY(kd_alloc(&k->hist, radix_sort_hist_words(k->total)));
    if (k->nmaps)
        KM_TRY(cudaMemcpy(k->desc, k->maps.data(), sizeof(KdMultiMap) * k->nmaps, cudaMemcpyHostToDevice));
    KM_TRY(cudaMemcpy(k->tile_map, tile_map.data(), sizeof(uint32_t) * tile_map.size(), cudaMemcpyHostToDevice));
    KM_TRY(cudaMemcpy(k->seg_tab, seg.data(), sizeof(uint2) * seg.size(), cudaMemcpyHostToDevice));
    KM_TRY(cudaMemcpy(k->node_prefix, prefix.data(), sizeof(uint32_t) * prefix.size(), cudaMemcpyHostToDevice));
    KM_TRY(cudaMemcpy(k->level_n, level_n.data(), sizeof(uint32_t) * level_n.size(), cudaMemcpyHostToDevice));
#undef KM_TRY
    return cudaSuccess;
}

void kd_multi_free(KdMulti &k) {
    cudaFree(k.desc); cudaFree(k.tile_map); cudaFree(k.seg_tab); cudaFree(k.node_prefix); cudaFree(k.level_n);
    cudaFree(k.keys); cudaFree(k.keys_tmp); cudaFree(k.vals); cudaFree(k.vals_tmp); cudaFree(k.hist);
    cudaFree(k.fin_prefix);
    k = KdMulti();
}

cudaError_t kd_multi_levels(KdMulti &k, cudaStream_t s, uint32_t **order) {
    uint64_t *ka = k.keys, *kb = k.keys_tmp;
    uint32_t *va = k.vals, *vb = k.vals_tmp;
    *order = va;
    if (k.nmaps == 0) return cudaSuccess;
    if (k.pad) {
        multi_pad_kernel<<<(k.total + 255) / 256, 256, 0, s>>>(k.desc, k.tile_map, k.total);
        note_launch();
    }
    multi_init_kernel<<<(k.total + 255) / 256, 256, 0, s>>>(k.desc, k.tile_map, k.total, va);
    note_launch();
    multi_root_kernel<<<(k.nmaps + 127) / 128, 128, 0, s>>>(k.desc, k.nmaps);
    note_launch();
    const uint32_t tiles = k.total / kSortTile;
    for (int l = 0; l < k.levels; ++l) {
        const uint32_t n = k.level_tiles[l] * kSortTile;
        split_key_multi_kernel<<<(n + 255) / 256, 256, 0, s>>>(k.desc, k.tile_map, n, l, va, ka);
        note_launch();
        uint64_t *ko = nullptr;
        uint32_t *vo = nullptr;
        cudaError_t e = radix_sort_pairs_u64(ka, va, kb, vb, k.level_n + l, n, 0, 16, k.hist, s, &ko, &vo, 0,
                                             k.seg_tab + (size_t)l * tiles);
        if (e != cudaSuccess) return e;
        if (vo != va) {
            uint64_t *tk = ka; ka = kb; kb = tk;
            uint32_t *tv = va; va = vb; vb = tv;
        }
        split_cell_multi_kernel<<<(k.level_nodes[l] + 255) / 256, 256, 0, s>>>(
            k.desc, (int)k.level_maps[l], k.node_prefix + (size_t)l * (k.nmaps + 1), l, va);
        note_launch();
    }
    *order = va;
    return cudaGetLastError();
}

cudaError_t kd_multi_finish(KdMulti &k, uint32_t *order, cudaStream_t s) {
    if (k.nmaps == 0) return cudaSuccess;
    const int nm1 = k.nmaps + 1;
    cudaError_t e;
    if (k.subtrees > 0) {
        const int smem = (int)sizeof(SubtreeScratch);
        e = cudaFuncSetAttribute(multi_subtree_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        multi_subtree_kernel<<<k.subtrees, kSubtreeThreads, smem, s>>>(k.desc, k.nmaps, k.fin_prefix, order);
        note_launch();
    }
    multi_permute_kernel<<<(k.total + 255) / 256, 256, 0, s>>>(k.desc, k.tile_map, k.total, order);
    note_launch();
    multi_leaf_kernel<<<(uint32_t)(((uint64_t)k.leaves * 32 + 255) / 256), 256, 0, s>>>(k.desc, k.nmaps,
                                                                                          k.fin_prefix + nm1);
    note_launch();
    for (int l = k.max_depth - 1; l >= 10; --l) {
        const uint32_t cnt = k.inner_nodes[l - 10];
        if (cnt == 0) continue;
        multi_inner_kernel<<<(cnt + 255) / 256, 256, 0, s>>>(k.desc, k.nmaps, k.fin_prefix + (size_t)(2 + l - 10) * nm1,
                                                             l);
        note_launch();
    }
    multi_top_kernel<<<k.nmaps, 1024, 0, s>>>(k.desc);
    note_launch();
    return cudaGetLastError();
}

}  // namespace pm
