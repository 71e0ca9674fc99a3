// tile_gather.cu -- k-NN radiance estimates of a query list in spatial
// order, one candidate set per group of neighbouring queries.
//
// A warp takes 1 to 4 consecutive groups of 32 queries of the (map, Morton
// code) order. The k-th-neighbour distance d(x) (capped at the gather radius) is
// 1-Lipschitz in the query position, so exact distances d_j at points x_j
// bound it everywhere:
//     max_j (d_j - |x - x_j|)  <=  d(x)  <=  min_j (d_j + |x - x_j|).
// The warp's first group is bounded by one anchor (an exact list search at
// one of its queries, done by a separate launch before), every later group
// by the exact results of the group before it. A group's records are
// collected once from the kd-tree -- every record within the largest upper
// bound of the group's bounding box -- into shared memory, and each query
// selects its k nearest from that set: records closer than its lower bound
// are in, records beyond its upper bound are out, and only the band between
// the bounds is ranked (the previous query of the group tightens both
// bounds the same way).
//
// A group whose set does not fit in shared memory is processed in segments:
// halves, down to single queries, each finished segment tightening the
// bounds of the queries after it. A single query whose set still does not
// fit, queries of the other map in a mixed group, and any result that
// contradicts its own upper bound, are deferred to a list-search launch
// after the pass. The selected set is exactly the list search's (ties
// broken by photon index) and the estimate's sum is order-independent
// (knn_core.cuh), so every value is bit-identical to the list search's.
#include <algorithm>

#include "cache.cuh"
#include "eye_path.cuh"
#include "knn_core.cuh"
#include "launch_count.cuh"
#include "phys_state.cuh"

namespace pm {
namespace {

using namespace wknn;

constexpr int kTileWarps = 4;
constexpr int kAnchorAt = 15;                // the anchor: query 15 of a warp's chunk
// Residency before capacity: 7 blocks of 4 warps per SM (the registers capped
// at 72, a few spilled) with candidate sets of 272 records measured faster
// than 5 blocks with 400 (more groups halve, but more warps hide the
// latency of every phase).
constexpr int kTileBlocks = 7;
constexpr int kTileCap = 272;                // candidate records per warp (fits 7 blocks' shared memory)
constexpr int kScanSlots = 2;   // candidates per lane per step of the selection scan
constexpr int kPickSlots = 1;   // band entries per lane per step of the final selection
constexpr float kRel = 2e-4f;                // relative and absolute margins of the distance bounds
constexpr float kAbs = 1e-6f;

// per-launch counters (pm_get_gather_stats)
enum TileStat { kStTiled, kStList, kStShrunk, kStViolations, kStGroups, kStCandidates, kStHalvings, kStCount };

struct TileScratch {
    float4 cpos[kTileCap];   // candidate positions (+ photon index bits)
    uint32_t cat[kTileCap];  // their tree positions
    union {
        uint32_t stack[kStackCap];  // the collection's node stack
        struct {
            float bd2[kTileCap];       // band: squared distances
            uint16_t bslot[kTileCap];  // band: candidate slots
            uint16_t sel[128];         // the k selected candidates
            uint64_t win[32];          // ranking window keys
        } b;
    };
    unsigned long long st[kStCount];  // counters, lane 0
};

// The parameters of the scene a warp is working on (per warp: in a launch
// over many scenes the warps of one block may serve different scenes).
struct TileArgs {
    MapView map[2];  // surface, volume
    float4 *out;
    uint32_t *defer;     // deferred query indices
    uint32_t *defer_sc;  // their scenes (launches over many scenes; nullable)
    uint32_t *defer_n;   // their count
    uint32_t scene;      // the scene's index in such a launch
    uint64_t cap;        // key bound of the gather radius
    float r2cap, rcap, g;
    int k;
    bool raw;
};

extern __shared__ __align__(16) unsigned char tile_smem[];
__shared__ __align__(16) unsigned char tile_args[kTileWarps * sizeof(TileArgs)];

__device__ __forceinline__ TileArgs &targs() {
    return reinterpret_cast<TileArgs *>(tile_args)[threadIdx.x >> 5];
}

// Lane 0 fills the warp's arguments; the warp then synchronises.
__device__ __forceinline__ void set_targs(const MapView &surf, const MapView &vol, float4 *out,
                                          uint32_t *defer, uint32_t *defer_sc, uint32_t *defer_n,
                                          uint32_t scene, float r2cap, float g, int k, bool raw) {
    if ((threadIdx.x & 31) == 0) {
        TileArgs &t = targs();
        t.map[0] = surf;
        t.map[1] = vol;
        t.out = out;
        t.defer = defer;
        t.defer_sc = defer_sc;
        t.defer_n = defer_n;
        t.scene = scene;
        t.cap = make_key(r2cap, 0xffffffffu);
        t.r2cap = r2cap;
        t.rcap = sqrtf(r2cap);
        t.g = g;
        t.k = k;
        t.raw = raw;
    }
    __syncwarp();
}

__device__ __forceinline__ TileScratch &scratch() {
    return reinterpret_cast<TileScratch *>(tile_smem)[threadIdx.x >> 5];
}

struct Query {
    v3 x;
    v3 dirv;       // facing normal (surface) or view direction wo (volume)
    int map;       // 0 surface, 1 volume
    uint32_t out;  // query index (destination)
};

__device__ __forceinline__ Query shfl_query(const Query &q, int j) {
    Query r;
    r.x = mk3(__shfl_sync(kFull, q.x.x, j), __shfl_sync(kFull, q.x.y, j), __shfl_sync(kFull, q.x.z, j));
    r.dirv = mk3(__shfl_sync(kFull, q.dirv.x, j), __shfl_sync(kFull, q.dirv.y, j),
                 __shfl_sync(kFull, q.dirv.z, j));
    r.map = __shfl_sync(kFull, q.map, j);
    r.out = __shfl_sync(kFull, q.out, j);
    return r;
}

// One query of the list: position, the weight direction and its map.
__device__ __forceinline__ Query load_query(const PScene &Sc, const float4 *qa, const float4 *qd,
                                            uint32_t i) {
    Query q;
    const float4 a = qa[i], d = qd[i];
    const int obj = __float_as_int(a.w);
    q.x = mk3(a.x, a.y, a.z);
    const v3 wo = mk3(d.x, d.y, d.z);
    q.map = obj != kNone ? 0 : 1;
    q.dirv = obj != kNone ? facing_normal(Sc, obj, q.x, wo) : wo;
    q.out = i;
    return q;
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

__device__ __forceinline__ float gap(float lo, float hi, float v) {
    return fmaxf(fmaxf(lo - v, v - hi), 0.0f);
}

__device__ __forceinline__ void count(int i, unsigned long long v = 1) {
    if ((threadIdx.x & 31) == 0) scratch().st[i] += v;
}

// Writes one estimate (lane 0): the flux sum and squared radius (raw; -1
// when nothing was found), or the normalised radiance estimate (the
// render's own expressions).
__device__ __forceinline__ void write_estimate(float4 *out, uint32_t i, v3 e, int found, float r2,
                                               bool surface, bool raw) {
    float r2out = -1.0f;
    if (found > 0) {
        r2out = r2;
        if (!raw) {
            const float sc = surface ? (1.0f / (3.14159265f * r2)) * 0.318309886f
                                     : 1.0f / (4.18879020f * r2 * sqrtf(r2));
            e = e * sc;
        }
    } else {
        e = mk3(0.f, 0.f, 0.f);
    }
    if ((threadIdx.x & 31) == 0) out[i] = make_float4(e.x, e.y, e.z, raw ? r2out : 0.0f);
}

// Queues the lanes of `mask` for the list-search launch.
__device__ __forceinline__ void defer(const Query &q, unsigned mask) {
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(targs().defer_n, (uint32_t)__popc(mask));
    base = __shfl_sync(kFull, base, 0);
    if ((mask >> lane) & 1u) {
        const uint32_t at = base + __popc(mask & ((1u << lane) - 1u));
        targs().defer[at] = q.out;
        if (targs().defer_sc) targs().defer_sc[at] = targs().scene;
    }
    count(kStList, (unsigned long long)__popc(mask));
}

// Every record of map `mid` within sqrt(rho2) of the box [lo, hi] into
// cpos/cat. Returns the count, or -1 when more than kTileCap qualify.
__device__ __noinline__ int collect(int mid, v3 lo, v3 hi, float rho2) {
    TileScratch &ts = scratch();
    const MapView &m = targs().map[mid];
    const int lane = threadIdx.x & 31;
    uint32_t *st = ts.stack;
    const unsigned lt = (1u << lane) - 1u;
    if (lane == 0) st[0] = 1u;
    __syncwarp();
    int top = 1, n = 0;
    const uint32_t first_leaf = 1u << m.depth;
    const int chunks = 1 << m.leaf_shift;
    while (top > 0) {
        --top;
        const uint32_t node = st[top];
        __syncwarp();
        const int dn = 31 - __clz(node);
        if (dn == m.depth) {
            for (int c = 0; c < chunks; ++c) {
                const uint32_t r = ((node - first_leaf) << (5 + m.leaf_shift)) + ((uint32_t)c << 5) + lane;
                bool in = false;
                float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
                if (r < m.n) {
                    p = __ldg(&m.pos[r]);
                    const float gx = gap(lo.x, hi.x, p.x), gy = gap(lo.y, hi.y, p.y),
                                gz = gap(lo.z, hi.z, p.z);
                    in = gx * gx + gy * gy + gz * gz <= rho2;
                }
                const unsigned mk = __ballot_sync(kFull, in);
                if (n + __popc(mk) > kTileCap) return -1;
                if (in) {
                    const int at = n + __popc(mk & lt);
                    ts.cpos[at] = p;
                    ts.cat[at] = r;
                }
                n += __popc(mk);
            }
        } else {
            int w = (m.depth - dn) % 5;
            if (w == 0) w = 5;
            const int nc = 1 << w;
            const uint32_t child = (node << w) + lane;
            bool ok = false;
            if (lane < nc) {
                const float4 bl = __ldg(&m.lo[child]), bh = __ldg(&m.hi[child]);
                const float gx = fmaxf(fmaxf(bl.x - hi.x, lo.x - bh.x), 0.0f);
                const float gy = fmaxf(fmaxf(bl.y - hi.y, lo.y - bh.y), 0.0f);
                const float gz = fmaxf(fmaxf(bl.z - hi.z, lo.z - bh.z), 0.0f);
                ok = gx * gx + gy * gy + gz * gz <= rho2;
            }
            const unsigned mk = __ballot_sync(kFull, ok);
            const int rank = __popc(mk & lt);
            if (ok && top + rank < kStackCap) st[top + rank] = child;
            top = min(top + __popc(mk), kStackCap);
            __syncwarp();
        }
    }
    __syncwarp();
    return n;
}

// The need-th smallest key (1-based) among the band entries bd2/bslot[0..B),
// all with lo2 <= d2 <= hi2. The window of squared distances holding it is
// narrowed (interpolating in r^3, else halving the float bit range) until at
// most 32 entries remain, which are ranked by full key.
__device__ __noinline__ uint64_t band_select(int B, int need, float lo2, float hi2) {
    TileScratch &ts = scratch();
    const int lane = threadIdx.x & 31;
    uint32_t blo = __float_as_uint(lo2), bhi = __float_as_uint(hi2) + 1u;  // [blo, bhi)
    int below = 0, inwin = B;
    bool interp = true;
    while (inwin > 32 && bhi - blo > 1u) {
        uint32_t t;
        if (interp) {
            const float rl = sqrtf(__uint_as_float(blo)), rh = sqrtf(__uint_as_float(bhi - 1u));
            const float f = ((float)(need - below) - 0.5f) / (float)inwin;
            const float vl = rl * rl * rl, vh = rh * rh * rh;
            const float rt = cbrtf(vl + f * (vh - vl));
            t = __float_as_uint(rt * rt);
        } else {
            t = blo + ((bhi - blo) >> 1);
        }
        t = min(max(t, blo + 1u), bhi - 1u);
        int c = 0;
        for (int e = lane; e < B; e += 32) {
            const uint32_t b = __float_as_uint(ts.b.bd2[e]);
            c += (b >= blo && b < t) ? 1 : 0;
        }
        c = (int)__reduce_add_sync(kFull, (uint32_t)c);
        const int before = inwin;
        if (below + c >= need) {
            bhi = t;
            inwin = c;
        } else {
            below += c;
            blo = t;
            inwin -= c;
        }
        interp = 4 * inwin <= 3 * before;  // interpolation pays while it cuts a quarter
    }
    const int want = need - below;  // 1-based rank inside the window
    const unsigned lt = (1u << lane) - 1u;
    if (inwin <= 32) {
        int n = 0;
        for (int base = 0; base < B; base += 32) {
            const int e = base + lane;
            bool in = false;
            uint64_t key = 0;
            if (e < B) {
                const uint32_t b = __float_as_uint(ts.b.bd2[e]);
                in = b >= blo && b < bhi;
                if (in) key = make_key(ts.b.bd2[e], __float_as_uint(ts.cpos[ts.b.bslot[e]].w));
            }
            const unsigned mk = __ballot_sync(kFull, in);
            if (in) ts.b.win[n + __popc(mk & lt)] = key;
            n += __popc(mk);
        }
        __syncwarp();
        const uint64_t mine = lane < n ? ts.b.win[lane] : ~0ull;
        int rank = 0;
        for (int f = 0; f < n; ++f) rank += ts.b.win[f] < mine ? 1 : 0;
        const unsigned hit = __ballot_sync(kFull, lane < n && rank == want - 1);
        const uint64_t kth = __shfl_sync(kFull, mine, __ffs(hit) - 1);
        __syncwarp();
        return kth;
    }
    // more than 32 entries at one squared distance: rank by photon index
    const float v = __uint_as_float(blo);
    uint64_t lo_i = 0, hi_i = 0xffffffffull;  // the index is in [lo_i, hi_i]
    while (lo_i < hi_i) {
        const uint64_t mid = (lo_i + hi_i) >> 1;
        int c = 0;
        for (int e = lane; e < B; e += 32)
            if (ts.b.bd2[e] == v && __float_as_uint(ts.cpos[ts.b.bslot[e]].w) <= (uint32_t)mid) ++c;
        c = (int)__reduce_add_sync(kFull, (uint32_t)c);
        if (c >= want) hi_i = mid; else lo_i = mid + 1;
    }
    return make_key(v, (uint32_t)lo_i);
}

struct Pick {
    int found;     // records selected (k, or all within the cap when fewer)
    bool ok;       // false: the bounds contradicted the candidates
    uint64_t kth;  // the k-th key when found == k
};

// Selects the k nearest candidates of q into sel[0..found) given bounds
// lo2 <= (k-th squared distance) <= hi2 (hi2 <= r2cap).
__device__ __forceinline__ Pick pick_k(int n, v3 q, float lo2, float hi2) {
    TileScratch &ts = scratch();
    const int lane = threadIdx.x & 31;
    const int k = targs().k;
    const uint64_t cap = targs().cap;
    const unsigned lt = (1u << lane) - 1u;
    int n_in = 0, B = 0;
    // kScanSlots slots per lane and step: their loads and distances are
    // independent; the ballots and stores keep slot order
    for (int base = 0; base < n; base += 32 * kScanSlots) {
        bool in[kScanSlots], band[kScanSlots];
        float d2[kScanSlots];
        unsigned mi[kScanSlots], mb[kScanSlots];
#pragma unroll
        for (int u = 0; u < kScanSlots; ++u) {
            const int c = base + 32 * u + lane;
            in[u] = band[u] = false;
            d2[u] = 0.0f;
            if (c < n) {
                const float4 p = ts.cpos[c];
                const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
                d2[u] = dx * dx + dy * dy + dz * dz;
                in[u] = d2[u] < lo2;
                band[u] = !in[u] && d2[u] <= hi2 && make_key(d2[u], __float_as_uint(p.w)) < cap;
            }
        }
        int tin = 0;
#pragma unroll
        for (int u = 0; u < kScanSlots; ++u) {
            mi[u] = __ballot_sync(kFull, in[u]);
            mb[u] = __ballot_sync(kFull, band[u]);
            tin += __popc(mi[u]);
        }
        if (n_in + tin >= k) {  // the lower bound was too high
            __syncwarp();
            return Pick{0, false, 0};
        }
#pragma unroll
        for (int u = 0; u < kScanSlots; ++u) {
            const int c = base + 32 * u + lane;
            if (in[u]) ts.b.sel[n_in + __popc(mi[u] & lt)] = (uint16_t)c;
            if (band[u]) {
                const int at = B + __popc(mb[u] & lt);
                ts.b.bd2[at] = d2[u];
                ts.b.bslot[at] = (uint16_t)c;
            }
            n_in += __popc(mi[u]);
            B += __popc(mb[u]);
        }
    }
    __syncwarp();
    const int need = k - n_in;
    if (B < need) {
        if (hi2 < targs().r2cap) return Pick{0, false, 0};  // the upper bound was too low
        for (int e = lane; e < B; e += 32) ts.b.sel[n_in + e] = ts.b.bslot[e];
        __syncwarp();
        return Pick{n_in + B, true, cap};
    }
    const uint64_t kth = band_select(B, need, lo2, hi2);
    int sel = n_in;
    for (int base = 0; base < B; base += 32 * kPickSlots) {
        bool sl[kPickSlots];
        uint16_t slot[kPickSlots];
#pragma unroll
        for (int u = 0; u < kPickSlots; ++u) {
            const int e = base + 32 * u + lane;
            sl[u] = false;
            slot[u] = 0;
            if (e < B) {
                slot[u] = ts.b.bslot[e];
                sl[u] = make_key(ts.b.bd2[e], __float_as_uint(ts.cpos[slot[u]].w)) <= kth;
            }
        }
#pragma unroll
        for (int u = 0; u < kPickSlots; ++u) {
            const unsigned ms = __ballot_sync(kFull, sl[u]);
            if (sl[u]) ts.b.sel[sel + __popc(ms & lt)] = slot[u];
            sel += __popc(ms);
        }
    }
    __syncwarp();
    return Pick{sel, true, kth};
}

// The lanes of `mask` (queries of one map, lane order = spatial order) from
// one shared candidate set; lb / ub: each lane's bounds on its capped k-th
// distance. Returns false when the set does not fit; otherwise sets d_lane
// to the capped k-th distance of the lane's query (-1 if it was deferred).
template <int S>
__device__ __noinline__ bool tile_queries(Query q, unsigned mask, float lb, float ub, float *d_lane) {
    TileScratch &ts = scratch();
    const int lane = threadIdx.x & 31;
    const int k = targs().k;
    const int mid = __shfl_sync(kFull, q.map, __ffs(mask) - 1);
    const MapView &m = targs().map[mid];
    const bool member = (mask >> lane) & 1u;
    const float inf = __int_as_float(0x7f800000);
    const v3 lo = mk3(warp_min(member ? q.x.x : inf), warp_min(member ? q.x.y : inf),
                      warp_min(member ? q.x.z : inf));
    const v3 hi = mk3(warp_max(member ? q.x.x : -inf), warp_max(member ? q.x.y : -inf),
                      warp_max(member ? q.x.z : -inf));
    const float rho = warp_max(member ? ub : 0.0f);
    const int n = collect(mid, lo, hi, rho * rho);
    if (n < 0) return false;
    count(kStGroups);
    count(kStCandidates, (unsigned long long)n);
    const float r2cap = targs().r2cap, rcap = targs().rcap;
    float prev_r = -1.0f;
    v3 xp = mk3(0.f, 0.f, 0.f);
    for (unsigned mm = mask; mm; mm &= mm - 1) {
        const int j = __ffs(mm) - 1;
        const Query qj = shfl_query(q, j);
        float lo_r = __shfl_sync(kFull, lb, j), hi_r = __shfl_sync(kFull, ub, j);
        const float ubj = hi_r;
        if (prev_r >= 0.0f) {
            const v3 dv = qj.x - xp;
            const float dl = sqrtf(dot(dv, dv));
            lo_r = fmaxf(lo_r, (prev_r - dl) * (1.0f - kRel) - kAbs);
            hi_r = fminf(hi_r, (prev_r + dl) * (1.0f + kRel) + kAbs);
        }
        float lo2 = fmaxf(lo_r, 0.0f) * fmaxf(lo_r, 0.0f);
        float hi2 = fminf(hi_r * hi_r, r2cap);
        Pick pk;
        for (;;) {
            pk = pick_k(n, qj.x, lo2, hi2);
            if (pk.ok) break;
            lo2 = 0.0f;  // inconsistent bounds: select over the whole set
            hi2 = r2cap;
        }
        // the set holds every record within the upper bound; a result
        // beyond it would mean the bound failed: defer to the list search
        const float kd2 = pk.found == k ? key_d2(pk.kth) : r2cap;
        if ((pk.found == k && kd2 > ubj * ubj) || (pk.found < k && ubj < rcap)) {
            count(kStViolations);
            defer(q, 1u << j);
            if (lane == j) *d_lane = -1.0f;
            prev_r = -1.0f;
            continue;
        }
        float tx[S], ty[S], tz[S];
#pragma unroll
        for (int s = 0; s < S; ++s) {
            tx[s] = ty[s] = tz[s] = 0.0f;
            const int e = lane + 32 * s;
            if (e < pk.found) {
                const v3 t = flux_term(m, ts.cat[ts.b.sel[e]], mid, qj.dirv, targs().g);
                tx[s] = t.x;
                ty[s] = t.y;
                tz[s] = t.z;
            }
        }
        const v3 e = mk3(warp_fixed_sum<S>(tx), warp_fixed_sum<S>(ty), warp_fixed_sum<S>(tz));
        write_estimate(targs().out, qj.out, e, pk.found, kd2, mid == 0, targs().raw);
        __syncwarp();
        const float dj = pk.found == k ? sqrtf(kd2) : rcap;
        if (lane == j) *d_lane = dj;
        prev_r = dj;
        xp = qj.x;
        count(kStTiled);
    }
    return true;
}

// Bounds for the single query of lane j whose set within its upper bound
// does not fit: the radius is bisected (in r^3) between the bounds. A
// collection that overflows holds more than kTileCap >= k records, so its
// radius is an upper bound; one with fewer than k records (and below the
// cap) is a lower bound; one in between holds the k nearest. Returns
// false when no such radius turns up.
__device__ __noinline__ bool shrink_single(Query q, int j, float *lb, float *ub) {
    const int k = targs().k;
    const int mid = __shfl_sync(kFull, q.map, j);
    const v3 x = mk3(__shfl_sync(kFull, q.x.x, j), __shfl_sync(kFull, q.x.y, j),
                     __shfl_sync(kFull, q.x.z, j));
    float lo = __shfl_sync(kFull, *lb, j), hi = fminf(__shfl_sync(kFull, *ub, j), targs().rcap);
    for (int it = 0; it < 24; ++it) {
        const float r = cbrtf(0.5f * (lo * lo * lo + hi * hi * hi));
        const int n = collect(mid, x, x, r * r);
        if (n < 0) {
            hi = r;
        } else if (n < k && r < targs().rcap) {
            lo = r;
        } else {
            if ((threadIdx.x & 31) == j) {
                *ub = r * (1.0f + kRel) + kAbs;
                *lb = fmaxf(*lb, lo * (1.0f - kRel) - kAbs);
            }
            return true;
        }
    }
    return false;
}

// Tightens each lane's bounds with the exact distances of the lanes in
// `mask` (d_lane >= 0).
__device__ __forceinline__ void tighten(const Query &q, unsigned mask, float d_lane, float *lb, float *ub) {
    for (unsigned mm = mask; mm; mm &= mm - 1) {
        const int j = __ffs(mm) - 1;
        const float dj = __shfl_sync(kFull, d_lane, j);
        const float jx = __shfl_sync(kFull, q.x.x, j), jy = __shfl_sync(kFull, q.x.y, j),
                    jz = __shfl_sync(kFull, q.x.z, j);
        if (dj >= 0.0f) {
            const float dx = q.x.x - jx, dy = q.x.y - jy, dz = q.x.z - jz;
            const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
            *ub = fminf(*ub, (dj + dist) * (1.0f + kRel) + kAbs);
            *lb = fmaxf(*lb, (dj - dist) * (1.0f - kRel) - kAbs);
        }
    }
}

// One chunk (groups of 32 consecutive queries of the sorted order, from
// query chunk * 32 * groups) of a scene, with the warp's arguments set.
template <int S>
__device__ __forceinline__ void tile_chunk(const PScene &Sc, const MapView &surf, const MapView &vol,
                                           const float4 *qa, const float4 *qd, const uint32_t *order,
                                           uint32_t n, uint32_t chunk, float anchor, int groups,
                                           float r2cap, bool raw, float4 *out) {
    const int lane = threadIdx.x & 31;
    const float rcap = sqrtf(r2cap);
    const uint32_t wfirst = chunk * (uint32_t)(32 * groups);
    // exact distances known so far (lane j: one point; kd < 0: none): the
    // anchor, later the previous group
    float kx = 0.f, ky = 0.f, kz = 0.f, kd = -1.0f;
    int wkind;
    {
        const uint32_t ai = order[wfirst + min((uint32_t)kAnchorAt, n - 1 - wfirst)];
        const float4 a = qa[ai];
        wkind = __float_as_int(a.w) != kNone ? 0 : 1;
        if (lane == 0) {
            kx = a.x;
            ky = a.y;
            kz = a.z;
            kd = anchor;
        }
    }
    for (int g = 0; g < groups; ++g) {
        const uint32_t first = wfirst + (uint32_t)(32 * g);
        if (first >= n) break;
        const uint32_t cnt = min(32u, n - first);
        Query q;
        q.x = q.dirv = mk3(0.f, 0.f, 0.f);
        q.map = 1;
        q.out = 0;
        if ((uint32_t)lane < cnt) q = load_query(Sc, qa, qd, order[first + lane]);
        const int gkind = __shfl_sync(kFull, q.map, 0);
        const unsigned valid = __ballot_sync(kFull, (uint32_t)lane < cnt);
        const unsigned members = __ballot_sync(kFull, (uint32_t)lane < cnt && q.map == gkind);
        const uint32_t mn = gkind == 0 ? surf.n : vol.n;
        float dnew = -1.0f;
        if (gkind != wkind) {
            kd = -1.0f;
            wkind = gkind;
        }
        if (mn == 0) {
            // an empty map: nothing found
            if ((members >> lane) & 1u) out[q.out] = make_float4(0.f, 0.f, 0.f, raw ? -1.0f : 0.0f);
        } else {
            float ub = rcap, lb = 0.0f;
            for (int j = 0; j < 32; ++j) {
                const float jx = __shfl_sync(kFull, kx, j), jy = __shfl_sync(kFull, ky, j);
                const float jz = __shfl_sync(kFull, kz, j), jd = __shfl_sync(kFull, kd, j);
                if (jd >= 0.0f) {
                    const float dx = q.x.x - jx, dy = q.x.y - jy, dz = q.x.z - jz;
                    const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
                    ub = fminf(ub, (jd + dist) * (1.0f + kRel) + kAbs);
                    lb = fmaxf(lb, (jd - dist) * (1.0f - kRel) - kAbs);
                }
            }
            // segments of the members in spatial order: the whole group,
            // then halves of a segment whose set does not fit, down to
            // single queries (growing again after a fit); each finished
            // segment tightens the bounds of the rest
            unsigned rem = members;
            int sz = 32;
            while (rem) {
                const unsigned seg = __popc(rem) <= sz ? rem : rem & ((1u << __fns(rem, 0, sz + 1)) - 1u);
                if (tile_queries<S>(q, seg, lb, ub, &dnew)) {
                    rem &= ~seg;
                    if (rem) tighten(q, seg, dnew, &lb, &ub);
                    sz = min(2 * sz, 32);
                } else if (__popc(seg) > 1) {
                    count(kStHalvings);
                    sz = __popc(seg) >> 1;
                } else if (shrink_single(q, __ffs(seg) - 1, &lb, &ub) &&
                           tile_queries<S>(q, seg, lb, ub, &dnew)) {
                    count(kStShrunk);
                    rem &= ~seg;
                    if (rem) tighten(q, seg, dnew, &lb, &ub);
                } else {
                    defer(q, seg);
                    rem &= ~seg;
                }
            }
        }
        const unsigned odd = valid & ~members;
        if (odd) defer(q, odd);
        // this group's exact distances bound the next group
        kx = q.x.x;
        ky = q.x.y;
        kz = q.x.z;
        kd = ((members >> lane) & 1u) ? dnew : -1.0f;
    }
}

template <int S>
__global__ void __launch_bounds__(kTileWarps * 32, kTileBlocks)
    query_knn_tile_kernel(PScene Sc, MapView surf, MapView vol, const float4 *qa, const float4 *qd,
                          const uint32_t *order, uint32_t n, const uint32_t *n_dev, int groups,
                          const float *anchor_d, int k, float r2cap, bool raw, float4 *out,
                          uint32_t *defer_list, uint32_t *defer_n, uint32_t *chunk_counter,
                          unsigned long long *stats) {
    const int lane = threadIdx.x & 31;
    if (n_dev) n = min(n, *n_dev);
    set_targs(surf, vol, out, defer_list, nullptr, defer_n, 0u, r2cap, Sc.g, k, raw);
    TileScratch &ts = scratch();
    if (lane < kStCount) ts.st[lane] = 0;
    __syncwarp();
    const uint32_t nchunks = (n + 32u * (uint32_t)groups - 1u) / (32u * (uint32_t)groups);
    // persistent warps: each takes the next chunk from the counter until
    // none is left, so a block's resources are never held by finished warps
    // waiting on a slow one
    for (;;) {
        uint32_t chunk = 0;
        if (lane == 0) chunk = atomicAdd(chunk_counter, 1u);
        chunk = __shfl_sync(kFull, chunk, 0);
        if (chunk >= nchunks) break;
        tile_chunk<S>(Sc, surf, vol, qa, qd, order, n, chunk, anchor_d[chunk], groups, r2cap, raw, out);
    }
    __syncwarp();
    if (stats && lane < kStCount && ts.st[lane]) atomicAdd(&stats[lane], ts.st[lane]);
}

// The scene of global chunk c: the last descriptor whose chunk_begin <= c.
__device__ __forceinline__ int scene_of_chunk(const TileScene *scenes, int nsc, uint32_t c) {
    int lo = 0, hi = nsc - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (scenes[mid].chunk_begin <= c) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// The same pass over the chunks of many scenes (their descriptors in device
// memory, chunks numbered scene after scene): one persistent launch; a warp
// loads a scene's arguments when its next chunk belongs to another scene.
template <int S>
__global__ void __launch_bounds__(kTileWarps * 32, kTileBlocks)
    query_knn_tile_multi_kernel(const TileScene *scenes, int nsc, uint32_t total_chunks, int groups,
                                const float *anchor_d, bool raw, uint32_t *defer_list,
                                uint32_t *defer_sc, uint32_t *defer_n, uint32_t *chunk_counter,
                                unsigned long long *stats) {
    const int lane = threadIdx.x & 31;
    TileScratch &ts = scratch();
    if (lane < kStCount) ts.st[lane] = 0;
    __syncwarp();
    int cur = -1;
    for (;;) {
        uint32_t chunk = 0;
        if (lane == 0) chunk = atomicAdd(chunk_counter, 1u);
        chunk = __shfl_sync(kFull, chunk, 0);
        if (chunk >= total_chunks) break;
        const int sidx = scene_of_chunk(scenes, nsc, chunk);
        const TileScene &d = scenes[sidx];
        if (sidx != cur) {
            set_targs(d.surf, d.vol, d.val, defer_list, defer_sc, defer_n, (uint32_t)sidx, d.r2cap, d.sc->g,
                      d.k, raw);
            cur = sidx;
        }
        tile_chunk<S>(*d.sc, d.surf, d.vol, d.qa, d.qd, d.order, d.n, chunk - d.chunk_begin, anchor_d[chunk],
                      groups, d.r2cap, raw, d.val);
    }
    __syncwarp();
    if (stats && lane < kStCount && ts.st[lane]) atomicAdd(&stats[lane], ts.st[lane]);
}

// Exact capped k-th distance of each warp chunk's anchor query (list search).
template <int S>
__global__ void __launch_bounds__(128)
    anchor_kernel(MapView surf, MapView vol, const float4 *qa, const uint32_t *order, uint32_t n,
                  const uint32_t *n_dev, int groups, int k, float r2cap, float *anchor_d) {
    __shared__ WarpScratch ws[4];
    if (n_dev) n = min(n, *n_dev);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t chunk = blockIdx.x * 4 + wib;
    const uint32_t wfirst = chunk * (uint32_t)(32 * groups);
    if (wfirst >= n) return;
    const float4 a = qa[order[wfirst + min((uint32_t)kAnchorAt, n - 1 - wfirst)]];
    const MapView &m = __float_as_int(a.w) != kNone ? surf : vol;
    const uint64_t cap = make_key(r2cap, 0xffffffffu);
    Knn<S> kn;
    kn.reset(cap, k);
    knn_search<S>(m, mk3(a.x, a.y, a.z), kn, ws[wib], lane, cap);
    if (lane == 0) anchor_d[chunk] = kn.worst < cap ? sqrtf(key_d2(kn.worst)) : sqrtf(r2cap);
}

// The anchors of the chunks of many scenes (global chunk numbering).
template <int S>
__global__ void __launch_bounds__(128)
    anchor_multi_kernel(const TileScene *scenes, int nsc, uint32_t total_chunks, int groups,
                        float *anchor_d) {
    __shared__ WarpScratch ws[4];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t chunk = blockIdx.x * 4 + wib;
    if (chunk >= total_chunks) return;
    const TileScene &d = scenes[scene_of_chunk(scenes, nsc, chunk)];
    const uint32_t wfirst = (chunk - d.chunk_begin) * (uint32_t)(32 * groups);
    const float4 a = d.qa[d.order[wfirst + min((uint32_t)kAnchorAt, d.n - 1 - wfirst)]];
    const MapView &m = __float_as_int(a.w) != kNone ? d.surf : d.vol;
    const uint64_t cap = make_key(d.r2cap, 0xffffffffu);
    Knn<S> kn;
    kn.reset(cap, d.k);
    knn_search<S>(m, mk3(a.x, a.y, a.z), kn, ws[wib], lane, cap);
    if (lane == 0) anchor_d[chunk] = kn.worst < cap ? sqrtf(key_d2(kn.worst)) : sqrtf(d.r2cap);
}

// The deferred queries of many scenes (defer_sc: each one's scene).
template <int S>
__global__ void __launch_bounds__(128)
    deferred_multi_kernel(const TileScene *scenes, const uint32_t *defer_list, const uint32_t *defer_sc,
                          const uint32_t *defer_n, bool raw) {
    __shared__ WarpScratch ws[4];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t total = *defer_n;
    for (uint32_t w = blockIdx.x * 4 + wib; w < total; w += gridDim.x * 4) {
        const TileScene &d = scenes[defer_sc[w]];
        const uint64_t cap = make_key(d.r2cap, 0xffffffffu);
        const Query q = load_query(*d.sc, d.qa, d.qd, defer_list[w]);
        const MapView &m = q.map == 0 ? d.surf : d.vol;
        v3 e = mk3(0.f, 0.f, 0.f);
        int found = 0;
        float r2 = d.r2cap;
        if (m.n > 0) {
            Knn<S> kn;
            kn.reset(cap, d.k);
            knn_search<S>(m, q.x, kn, ws[wib], lane, cap);
            e = flux_sum<S>(kn, m, lane, q.map, q.dirv, d.sc->g, cap, d.r2cap, &found, &r2);
        }
        write_estimate(d.val, q.out, e, found, r2, q.map == 0, raw);
    }
}

// The deferred queries, one warp each (grid-stride over the list).
template <int S>
__global__ void __launch_bounds__(128)
    deferred_kernel(PScene Sc, MapView surf, MapView vol, const float4 *qa, const float4 *qd,
                    const uint32_t *defer_list, const uint32_t *defer_n, int k, float r2cap, bool raw,
                    float4 *out) {
    __shared__ WarpScratch ws[4];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t total = *defer_n;
    const uint64_t cap = make_key(r2cap, 0xffffffffu);
    for (uint32_t w = blockIdx.x * 4 + wib; w < total; w += gridDim.x * 4) {
        const Query q = load_query(Sc, qa, qd, defer_list[w]);
        const MapView &m = q.map == 0 ? surf : vol;
        v3 e = mk3(0.f, 0.f, 0.f);
        int found = 0;
        float r2 = r2cap;
        if (m.n > 0) {
            Knn<S> kn;
            kn.reset(cap, k);
            knn_search<S>(m, q.x, kn, ws[wib], lane, cap);
            e = flux_sum<S>(kn, m, lane, q.map, q.dirv, Sc.g, cap, r2cap, &found, &r2);
        }
        write_estimate(out, q.out, e, found, r2, q.map == 0, raw);
    }
}

}  // namespace

cudaError_t knn_values_tiles(const PScene &S, const MapView &surf, const MapView &vol,
                             const float4 *qa, const float4 *qd, const uint32_t *order, uint32_t n,
                             const uint32_t *n_dev, int groups, int k, float radius, bool raw,
                             float4 *val, const TileBuffers &buf, int sm_count, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (groups < 1 || groups > 4) return cudaErrorInvalidValue;
    const float r2 = radius * radius;
    const uint32_t chunks = tile_chunks(n, groups);
    const dim3 grid((chunks + kTileWarps - 1) / kTileWarps), block(kTileWarps * 32);
    const int smem = (int)(kTileWarps * sizeof(TileScratch));
    const dim3 dgrid(std::max(sm_count, 1) * 8);
    // defer_n[0]: deferred queries, defer_n[1]: the chunk counter
    cudaError_t e = cudaMemsetAsync(buf.defer_n, 0, 2 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    int per_sm = 1;
    // persistent tile launch: as many blocks as fit on the GPU at once
#define PM_TILE_LAUNCH(SL)                                                                              \
    anchor_kernel<SL><<<grid, block, 0, s>>>(surf, vol, qa, order, n, n_dev, groups, k, r2, buf.anchor_d); \
    e = cudaFuncSetAttribute(query_knn_tile_kernel<SL>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem); \
    if (e != cudaSuccess) return e;                                                                     \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, query_knn_tile_kernel<SL>, kTileWarps * 32, smem); \
    if (e != cudaSuccess) return e;                                                                     \
    query_knn_tile_kernel<SL><<<std::min<uint32_t>(grid.x, (uint32_t)std::max(sm_count, 1) * (uint32_t)std::max(per_sm, 1)), \
                                block, smem, s>>>(S, surf, vol, qa, qd, order, n, n_dev, groups, buf.anchor_d, k, \
                                                  r2, raw, val, buf.defer, buf.defer_n, buf.defer_n + 1, buf.stats); \
    deferred_kernel<SL><<<dgrid, 128, 0, s>>>(S, surf, vol, qa, qd, buf.defer, buf.defer_n, k, r2, raw, val)
    switch ((k + 31) / 32) {
        case 1: PM_TILE_LAUNCH(1); break;
        case 2: PM_TILE_LAUNCH(2); break;
        case 3: PM_TILE_LAUNCH(3); break;
        default: PM_TILE_LAUNCH(4); break;
    }
#undef PM_TILE_LAUNCH
    note_launches(3);
    return cudaGetLastError();
}

cudaError_t knn_values_tiles_multi(const TileScene *scenes, int nsc, uint32_t total_chunks, int groups,
                                   int slots, bool raw, const TileBuffers &buf, uint32_t *defer_sc,
                                   int sm_count, cudaStream_t s) {
    if (total_chunks == 0 || nsc == 0) return cudaSuccess;
    if (groups < 1 || groups > 4 || slots < 1 || slots > 4) return cudaErrorInvalidValue;
    const dim3 agrid((total_chunks + kTileWarps - 1) / kTileWarps), block(kTileWarps * 32);
    const int smem = (int)(kTileWarps * sizeof(TileScratch));
    const dim3 dgrid(std::max(sm_count, 1) * 8);
    cudaError_t e = cudaMemsetAsync(buf.defer_n, 0, 2 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    int per_sm = 1;
#define PM_MULTI_LAUNCH(SL)                                                                              \
    anchor_multi_kernel<SL><<<agrid, block, 0, s>>>(scenes, nsc, total_chunks, groups, buf.anchor_d);   \
    e = cudaFuncSetAttribute(query_knn_tile_multi_kernel<SL>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem); \
    if (e != cudaSuccess) return e;                                                                     \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, query_knn_tile_multi_kernel<SL>, kTileWarps * 32, smem); \
    if (e != cudaSuccess) return e;                                                                     \
    query_knn_tile_multi_kernel<SL><<<std::min<uint32_t>(agrid.x, (uint32_t)std::max(sm_count, 1) * (uint32_t)std::max(per_sm, 1)), \
                                      block, smem, s>>>(scenes, nsc, total_chunks, groups, buf.anchor_d, raw, \
                                                        buf.defer, defer_sc, buf.defer_n, buf.defer_n + 1, buf.stats); \
    deferred_multi_kernel<SL><<<dgrid, 128, 0, s>>>(scenes, buf.defer, defer_sc, buf.defer_n, raw)
    switch (slots) {
        case 1: PM_MULTI_LAUNCH(1); break;
        case 2: PM_MULTI_LAUNCH(2); break;
        case 3: PM_MULTI_LAUNCH(3); break;
        default: PM_MULTI_LAUNCH(4); break;
    }
#undef PM_MULTI_LAUNCH
    note_launches(3);
    return cudaGetLastError();
}

uint32_t tile_chunks(uint32_t n, int groups) { return (n + 32u * groups - 1) / (32u * groups); }

}  // namespace pm
