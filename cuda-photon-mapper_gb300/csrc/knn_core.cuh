// knn_core.cuh -- the warp-cooperative exact k-nearest-record search over
// a map's kd-tree and the order-independent radiance-estimate sum, shared by
// the render kernels (gather.cu) and the shared-candidate gather
// (tile_gather.cu).
//
// One warp answers one query. The k best candidates so far live in
// registers as a list sorted by (squared distance, photon index), spread
// across the warp: lane l holds list positions l*S .. l*S+S-1 (S = k/32
// rounded up). Inserting a candidate is one shuffle from the previous lane
// plus S compare-selects per lane. The tree is walked 32 children at a time:
// the implicit layout puts the descendants five levels below node n at
// n*32 .. n*32+31, so each lane tests one child box with one coalesced
// load; surviving children are pushed far-to-near onto a per-warp stack in
// shared memory. Leaves are 32 consecutive records, one per lane.
//
// A node is skipped only when its box is strictly farther than the current
// k-th candidate, so a photon at exactly that distance with a smaller index
// is still found: the result equals a brute-force sort by (distance, index).
#pragma once
#include "gather.cuh"

namespace pm {
namespace wknn {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kStackCap = 192;     // 32 entries per wide level, 6 levels: depth <= 29


// Per-warp shared memory: the traversal stack and the staging areas of the
// bulk merge (the k-list and the sorted leaf candidates).
struct WarpScratch {
    uint32_t st_node[kStackCap];
    float st_d2[kStackCap];
    uint64_t lk[128];
    uint32_t la[128];
    uint64_t ck[32];
    uint32_t ca[32];
};


__device__ __forceinline__ uint64_t make_key(float d2, uint32_t idx) {
    return ((uint64_t)__float_as_uint(d2) << 32) | idx;
}
__device__ __forceinline__ float key_d2(uint64_t k) { return __uint_as_float((uint32_t)(k >> 32)); }

template <int S>
struct Knn {
    uint64_t key[S];
    uint32_t at[S];  // tree position of the record
    uint64_t worst;
    int k;

    __device__ __forceinline__ void reset(uint64_t cap, int kk) {
        k = kk;
#pragma unroll
        for (int s = 0; s < S; ++s) { key[s] = cap; at[s] = 0xffffffffu; }
        worst = cap;
    }
    __device__ __forceinline__ void update_worst() {
        const int kl = (k - 1) / S, ks = (k - 1) % S;
        uint64_t w = key[0];
#pragma unroll
        for (int s = 1; s < S; ++s)
            if (s == ks) w = key[s];
        worst = __shfl_sync(kFull, w, kl);
    }
    // Inserts x (< worst) keeping the list sorted.
    __device__ __forceinline__ void insert(uint64_t x, uint32_t xa, int lane) {
        uint64_t pk = __shfl_up_sync(kFull, key[S - 1], 1);
        uint32_t pa = __shfl_up_sync(kFull, at[S - 1], 1);
#pragma unroll
        for (int s = S - 1; s >= 0; --s) {
            uint64_t below = s > 0 ? key[s - 1] : pk;
            uint32_t below_at = s > 0 ? at[s - 1] : pa;
            bool first = (s == 0) && (lane == 0);
            if (key[s] >= x) {
                if (first || below < x) { key[s] = x; at[s] = xa; }
                else { key[s] = below; at[s] = below_at; }
            }
        }
        update_worst();
    }
    // Merges the candidates of the lanes in `mask` (each lane's `x` / `xa`,
    // all below worst) into the list at once: every list entry moves up by
    // the number of candidates below it, every candidate lands at its rank
    // among the candidates plus the number of list entries below it. Keys
    // are unique (photon indices), so the new positions are a permutation.
    __device__ __forceinline__ void merge(uint64_t x, uint32_t xa, unsigned mask, int lane,
                                          WarpScratch &w) {
        constexpr int K = 32 * S;
#pragma unroll
        for (int s = 0; s < S; ++s) {
            w.lk[lane * S + s] = key[s];
            w.la[lane * S + s] = at[s];
        }
        const int n = __popc(mask);
        int rc = 0;
        for (unsigned mm = mask; mm; mm &= mm - 1) {
            const int j = __ffs(mm) - 1;
            rc += __shfl_sync(kFull, x, j) < x ? 1 : 0;
        }
        if ((mask >> lane) & 1u) {
            w.ck[rc] = x;
            w.ca[rc] = xa;
        }
        __syncwarp();
        int lpos[S];
#pragma unroll
        for (int s = 0; s < S; ++s) {
            int lo = 0, hi = n;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (w.ck[mid] < key[s]) lo = mid + 1; else hi = mid;
            }
            lpos[s] = lane * S + s + lo;
        }
        int cpos = K;
        uint64_t cv = 0;
        uint32_t cav = 0;
        if (lane < n) {
            cv = w.ck[lane];
            cav = w.ca[lane];
            int lo = 0, hi = K;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (w.lk[mid] < cv) lo = mid + 1; else hi = mid;
            }
            cpos = lane + lo;
        }
        __syncwarp();
#pragma unroll
        for (int s = 0; s < S; ++s)
            if (lpos[s] < K) {
                w.lk[lpos[s]] = key[s];
                w.la[lpos[s]] = at[s];
            }
        if (cpos < K) {
            w.lk[cpos] = cv;
            w.la[cpos] = cav;
        }
        __syncwarp();
#pragma unroll
        for (int s = 0; s < S; ++s) {
            key[s] = w.lk[lane * S + s];
            at[s] = w.la[lane * S + s];
        }
        __syncwarp();
        update_worst();
    }
};

__device__ __forceinline__ float box_d2(float4 lo, float4 hi, v3 q) {
    float dx = fmaxf(fmaxf(lo.x - q.x, q.x - hi.x), 0.0f);
    float dy = fmaxf(fmaxf(lo.y - q.y, q.y - hi.y), 0.0f);
    float dz = fmaxf(fmaxf(lo.z - q.z, q.z - hi.z), 0.0f);
    return dx * dx + dy * dy + dz * dz;
}

// Sorts lk/la[0..P) ascending by key (bitonic network over shared memory);
// P is a power of two in [32, 128].
__device__ __forceinline__ void warp_sort_smem(WarpScratch &w, int P, int lane) {
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = lane; t < (P >> 1); t += 32) {
                // pair (i, i + stride) of the t-th compare-exchange (stride is
                // a power of two: no division)
                const int i = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
                const int j = i + stride;
                const bool up = (i & size) == 0;
                const uint64_t a = w.lk[i], b = w.lk[j];
                if ((a > b) == up) {
                    w.lk[i] = b;
                    w.lk[j] = a;
                    const uint32_t x = w.la[i];
                    w.la[i] = w.la[j];
                    w.la[j] = x;
                }
            }
            __syncwarp();
        }
    }
}

// Sorts the `count` collected candidates (count <= 128) in lk/la and loads
// the first 32*S of them into the k-list; empty slots hold cap.
template <int S>
__device__ __forceinline__ void load_sorted(Knn<S> &kn, WarpScratch &w, int count, uint64_t cap,
                                            int lane) {
    int P = 32;
    while (P < count) P <<= 1;
    for (int i = count + lane; i < P; i += 32) {
        w.lk[i] = cap;
        w.la[i] = 0xffffffffu;
    }
    __syncwarp();
    warp_sort_smem(w, P, lane);
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int j = lane * S + s;
        kn.key[s] = j < P ? w.lk[j] : cap;
        kn.at[s] = j < P ? w.la[j] : 0xffffffffu;
    }
    __syncwarp();
    kn.update_worst();
}

// k nearest records of q, sorted by (squared distance, index), within the
// radius cap held in kn.worst at entry. The walk starts in collect mode:
// every record within the cap is appended to a shared buffer, children are
// pushed in any order and nothing is kept sorted. If more than 128 records
// turn up, the buffer is sorted into the k-list and the walk continues in
// list mode, pruning with the current k-th distance and inserting (bulk
// merge or one at a time). A walk that stays in collect mode sorts its
// buffer once at the end. A warm walk (the next sample of a march) starts
// in list mode from the re-scored previous list and skips the records the
// list already holds. All modes produce the same exact list.
template <int S>
__device__ void knn_search(const MapView &m, v3 q, Knn<S> &kn, WarpScratch &ws, int lane,
                           uint64_t cap, bool warm = false, KnnTune tune = KnnTune()) {
    if (m.n == 0) return;
    const int collect_max = tune.collect_max;
    uint32_t *st_node = ws.st_node;
    float *st_d2 = ws.st_d2;
    const uint32_t first_leaf = 1u << m.depth;
    const int chunks = 1 << m.leaf_shift;
    bool collect = !warm;
    int count = 0;
    int top = 1;
    if (lane == 0) { st_node[0] = 1u; st_d2[0] = 0.0f; }
    __syncwarp();
    while (top > 0) {
        --top;
        const uint32_t node = st_node[top];
        const float nd2 = st_d2[top];
        __syncwarp();
        const float wd2 = key_d2(kn.worst);
        if (nd2 > wd2) continue;
        const int dn = 31 - __clz(node);
        if (dn == m.depth) {
            // a leaf: 32 << leaf_shift records, 32 at a time
            for (int c = 0; c < chunks; ++c) {
                const uint32_t base = ((node - first_leaf) << (5 + m.leaf_shift)) + ((uint32_t)c << 5);
                const uint32_t r = base + lane;
                uint64_t key = ~0ull;
                if (r < m.n) {
                    float4 p = __ldg(&m.pos[r]);
                    float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
                    key = make_key(dx * dx + dy * dy + dz * dz, __float_as_uint(p.w));
                }
                unsigned mask = __ballot_sync(kFull, key < kn.worst);
                if (!mask) continue;
                if (warm) {
                    // drop records the list already holds: list entries carry
                    // their tree positions, so the chunk's duplicates are one
                    // OR over the warp of the entries that fall in it
                    unsigned held = 0u;
#pragma unroll
                    for (int t = 0; t < S; ++t)
                        if ((kn.at[t] >> 5) == (base >> 5)) held |= 1u << (kn.at[t] & 31u);
                    mask &= ~__reduce_or_sync(kFull, held);
                    if (!mask) continue;
                }
                if (collect) {
                    const int add = __popc(mask);
                    if (count + add <= collect_max) {
                        if ((mask >> lane) & 1u) {
                            const int at = count + __popc(mask & ((1u << lane) - 1u));
                            ws.lk[at] = key;
                            ws.la[at] = r;
                        }
                        count += add;
                        __syncwarp();
                        continue;
                    }
                    load_sorted<S>(kn, ws, count, cap, lane);
                    collect = false;
                    mask = __ballot_sync(kFull, key < kn.worst);
                }
                if (__popc(mask) >= tune.merge_min) {
                    kn.merge(key, r, mask, lane, ws);
                } else {
                    while (mask) {
                        const int src = __ffs(mask) - 1;
                        uint64_t x = __shfl_sync(kFull, key, src);
                        kn.insert(x, base + src, lane);
                        mask &= mask - 1;
                        mask &= __ballot_sync(kFull, key < kn.worst);
                    }
                }
            }
        } else {
            int w = (m.depth - dn) % 5;
            if (w == 0) w = 5;
            const int nc = 1 << w;
            const uint32_t child = (node << w) + lane;
            float bd2 = __int_as_float(0x7f800000);
            if (lane < nc) bd2 = box_d2(__ldg(&m.lo[child]), __ldg(&m.hi[child]), q);
            const bool ok = (lane < nc) && (bd2 <= wd2);
            const unsigned mask = __ballot_sync(kFull, ok);
            int rank;
            if (collect || warm) {
                // any order: collect mode sorts at the end, and a warm start
                // already holds a tight k-th distance
                rank = __popc(mask & ((1u << lane) - 1u));
            } else {
                // far-to-near: survivors farther than this lane (ties: higher lane farther)
                rank = 0;
                for (unsigned mm = mask; mm; mm &= mm - 1) {
                    const int j = __ffs(mm) - 1;
                    float o = __shfl_sync(kFull, bd2, j);
                    rank += (o > bd2 || (o == bd2 && j > lane)) ? 1 : 0;
                }
            }
            if (ok && top + rank < kStackCap) {
                st_node[top + rank] = child;
                st_d2[top + rank] = bd2;
            }
            top = min(top + __popc(mask), kStackCap);
            __syncwarp();
        }
    }
    if (collect) load_sorted<S>(kn, ws, count, cap, lane);
}

// Warm start for the next sample of a march: the list of the previous
// sample, re-scored at q (entries beyond the cap dropped) and sorted. The
// search that follows only has to find records closer than its k-th entry.
template <int S>
__device__ void rescore(const MapView &m, v3 q, Knn<S> &kn, WarpScratch &ws, uint64_t cap,
                        int lane) {
    constexpr int K = 32 * S;
    constexpr int P = K <= 32 ? 32 : (K <= 64 ? 64 : 128);
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int j = lane * S + s;
        uint64_t nk = cap;
        uint32_t na = 0xffffffffu;
        if (kn.at[s] != 0xffffffffu) {
            const float4 p = __ldg(&m.pos[kn.at[s]]);
            const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
            const uint64_t k2 = make_key(dx * dx + dy * dy + dz * dz, __float_as_uint(p.w));
            if (k2 < cap) {
                nk = k2;
                na = kn.at[s];
            }
        }
        ws.lk[j] = nk;
        ws.la[j] = na;
    }
    for (int i = K + lane; i < P; i += 32) {
        ws.lk[i] = cap;
        ws.la[i] = 0xffffffffu;
    }
    __syncwarp();
    warp_sort_smem(ws, P, lane);
#pragma unroll
    for (int s = 0; s < S; ++s) {
        kn.key[s] = ws.lk[lane * S + s];
        kn.at[s] = ws.la[lane * S + s];
    }
    __syncwarp();
    kn.update_worst();
}

// Order-independent sum of non-negative float terms over a warp (T terms
// per lane, zeros allowed). With E the largest exponent field of all the
// terms (at least 1), each term becomes the integer floor(t * 2^(182 - E)):
// its 24-bit significand shifted left by 32 - (E - e) bits, or right
// (truncating) when that is negative. The integers add exactly in 64 bits
// (each below 2^56, at most 128 of them), and the total times 2^(E - 182)
// is rounded to float once, to nearest even. Any order of the terms and any
// split over lanes gives the same bits, within one rounding of the exact
// sum; this is what makes a k-NN estimate independent of the search that
// found its records.
__device__ __forceinline__ float scale_pow2(float f, int n) {
    if (n < -126) {  // f is 0 or >= 1: the first step is exact
        f *= __uint_as_float((uint32_t)(127 - 64) << 23);
        n += 64;
    }
    return f * __uint_as_float((uint32_t)(n + 127) << 23);
}

// 2^n as a float, n in [-126, 127].
__device__ __forceinline__ float pow2f(int n) { return __uint_as_float((uint32_t)(n + 127) << 23); }

template <int T>
__device__ __forceinline__ float warp_fixed_sum(const float (&t)[T]) {
    uint32_t emax = 1;
#pragma unroll
    for (int i = 0; i < T; ++i) emax = max(emax, __float_as_uint(t[i]) >> 23);
    emax = __reduce_max_sync(kFull, emax);
    // t * 2^(182 - E) is a power-of-two scale of a value below 2^(E - 126):
    // exact in float, below 2^56, and its truncation is the term's integer
    // (the significand shifted as described above)
    const int sh = 182 - (int)emax;  // [-72, 181]
    const float s1 = pow2f(min(sh, 127)), s2 = pow2f(max(sh - 127, 0));
    uint64_t acc = 0;
#pragma unroll
    for (int i = 0; i < T; ++i) {
        float x = t[i] * s1;
        if (sh > 127) x *= s2;
        acc += __float2ull_rz(x);
    }
    // three 20-bit slices: 32 lanes of each sum below 2^25 in 32 bits
    const uint64_t a0 = __reduce_add_sync(kFull, (uint32_t)(acc & 0xfffffu));
    const uint64_t a1 = __reduce_add_sync(kFull, (uint32_t)((acc >> 20) & 0xfffffu));
    const uint64_t a2 = __reduce_add_sync(kFull, (uint32_t)(acc >> 40));
    return scale_pow2(__ull2float_rn(a0 + (a1 << 20) + (a2 << 40)), (int)emax - 182);
}

// One record's contribution to an estimate's numerator: its flux times the
// weight toward the query. mode 0: surface (1 for photons arriving on the
// side dirv faces, else 0); mode 1: volume (HG phase toward dirv = wo).
__device__ __forceinline__ v3 flux_term(const MapView &m, uint32_t at, int mode, v3 dirv, float g) {
    const float4 pw = __ldg(&m.pow[at]);
    const float4 dv = __ldg(&m.dir[at]);
    const v3 dir = mk3(dv.x, dv.y, dv.z);
    float w;
    if (mode == 0) w = dot(dirv, dir) < 0.0f ? 1.0f : 0.0f;
    else w = hg_phase(g, dot(dir, dirv));
    return mk3(pw.x * w, pw.y * w, pw.z * w);
}

// Radiance-estimate numerator over the k-NN list: the fixed-point sum of
// the records' flux terms. Returns the found count and the squared radius
// in *r2 (the k-th distance, or the cap when fewer than k were found).
template <int S>
__device__ v3 flux_sum(const Knn<S> &kn, const MapView &m, int lane, int mode, v3 dirv, float g,
                       uint64_t cap, float r2cap, int *found, float *r2) {
    float tx[S], ty[S], tz[S];
    int cnt = 0;
#pragma unroll
    for (int s = 0; s < S; ++s) {
        tx[s] = ty[s] = tz[s] = 0.0f;
        const int j = lane * S + s;
        if (j < kn.k && kn.key[s] != cap) {
            ++cnt;
            const v3 t = flux_term(m, kn.at[s], mode, dirv, g);
            tx[s] = t.x;
            ty[s] = t.y;
            tz[s] = t.z;
        }
    }
    cnt = (int)__reduce_add_sync(kFull, (uint32_t)cnt);
    *found = cnt;
    *r2 = cnt == kn.k ? key_d2(kn.worst) : r2cap;
    return mk3(warp_fixed_sum<S>(tx), warp_fixed_sum<S>(ty), warp_fixed_sum<S>(tz));
}

}  // namespace wknn
}  // namespace pm
