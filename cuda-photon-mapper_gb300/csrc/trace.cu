// trace.cu -- photon emission, scattering and storage.
//
// One persistent launch: each warp keeps 32 live photon paths and, whenever
// some lanes' paths end (escape, Russian roulette, bounce limit), refills
// exactly those lanes from a global path counter with a single atomic per
// warp (ballot of the empty lanes, ranks by popcount). Warps therefore stay
// full while paths of very different lengths finish, and no path state is
// ever written to memory. A path's randomness is a Philox stream keyed by
// (seed) and counted by (path, event, slot, scene), so a path's trajectory
// does not depend on which warp or lane traced it.
//
// Two passes over the same deterministic paths: the counting pass stores
// nothing and stops issuing paths once both maps are full; a scan of the
// per-path counts then fixes every record's final index (records in path
// order, cut at the map's target), a compaction lists the ids of the paths
// the maps need (those with a record below a map's extent: about a tenth of
// the issued paths when one map fills much later than the other), and the
// writing pass retraces exactly those and writes each record straight into
// the SoA float4 map arrays, its power scaled by the number of paths the map
// drew from. No per-path staging memory, no compaction of records.
#include "launch_count.cuh"
#include "trace.cuh"
#include "radix_sort.cuh"

#include <algorithm>

namespace pm {
namespace {

__device__ __forceinline__ uint32_t lanemask_lt() {
    return (1u << (threadIdx.x & 31)) - 1u;
}

struct Path {
    v3 o, d, thr;
    uint32_t id;
    int ev;
    bool glass;
    uint32_t ns, nv;
    uint32_t os, ov;  // writing pass: the path's first record index in each map
};

__device__ __forceinline__ void start_path(const TraceParams &P, uint32_t id, Path &p, const PScene &S) {
    pm_u32x4 r = philox(P.seed, id, 0u, 0u, P.scene_id);
    p.o = mk3(S.light[0], S.light[1], S.light[2]);
    p.d = sample_sphere(pm_u01(r.v[0]), pm_u01(r.v[1]));
    p.thr = mk3(1.0f, 1.0f, 1.0f);
    p.id = id;
    p.ev = 0;
    p.glass = false;
    p.ns = 0;
    p.nv = 0;
    if (P.store) {  // loaded now, used at the path's first stores
        p.os = P.off_s[id];
        p.ov = P.off_v[id];
    }
}

__device__ __forceinline__ void store(float4 *pos, float4 *pw, uint32_t j, v3 x, v3 thr, v3 d,
                                      float scale) {
    pos[j] = make_float4(x.x, x.y, x.z, __uint_as_float(j));
    pw[j] = make_float4(thr.x * scale, thr.y * scale, thr.z * scale, __uint_as_float(oct_encode(d)));
}

struct MapOut {
    uint32_t n, paths;
    float scale;
};

// One interaction of path p; returns false when the path ends.
__device__ bool step_path(const PScene &S, const TraceParams &P, Path &p, const MapOut &ms,
                          const MapOut &mv) {
    p.ev += 1;
    pm_u32x4 r = philox(P.seed, p.id, (uint32_t)p.ev, 0u, P.scene_id);
    float u0 = pm_u01(r.v[0]), u1 = pm_u01(r.v[1]), u2 = pm_u01(r.v[2]), u3 = pm_u01(r.v[3]);
    // brute force over the spheres: the lanes of a warp trace different
    // photons, and a uniform loop beats divergent grid walks here
    PHit h = intersect(S, p.o, p.d, 3.0e38f);
    float seg = h.obj != kNone ? h.t : box_exit(S, p.o, p.d);
    bool vol = false;
    v3 x = p.o;
    float ss = 0.0f, st = 1.0f;
    if (S.sigma_max > 0.0f && !p.glass) {
        if (S.het_res <= 0) {
            st = S.sigma_s + S.sigma_a;
            if (S.sigma_s > 0.0f) {
                float t = -pm_logf(1.0f - u0) / st;
                if (t < seg) {
                    vol = true;
                    x = p.o + p.d * t;
                    ss = S.sigma_s;
                }
            }
        } else {
            // Delta tracking against the majorant (Woodcock et al. 1965):
            // tentative collision j draws its distance and acceptance from
            // words 2(j % 2), 2(j % 2) + 1 of Philox block 1 + j / 2.
            float t = 0.0f;
            pm_u32x4 q;
            for (uint32_t j = 0; j < kMaxDeltaSteps; ++j) {
                if ((j & 1u) == 0u) q = philox(P.seed, p.id, (uint32_t)p.ev, 1u + (j >> 1), P.scene_id);
                const uint32_t ua = (j & 1u) ? q.v[2] : q.v[0], ub = (j & 1u) ? q.v[3] : q.v[1];
                t += -pm_logf(1.0f - pm_u01(ua)) * S.inv_sigma_max;
                if (!(t < seg)) break;
                v3 y = p.o + p.d * t;
                float s = sigma_s_at(S, y);
                float sty = s + S.sigma_a;
                if (pm_u01(ub) * S.sigma_max < sty) {
                    vol = true;
                    x = y;
                    ss = s;
                    st = sty;
                    break;
                }
            }
        }
    }
    if (vol) {
        if (P.store) {
            uint32_t j = p.ov + p.nv;
            if (j < mv.n) store(P.vpos, P.vpow, j, x, p.thr, p.d, mv.scale);
        }
        p.nv += 1;
        if (!(u1 < P.rr)) return false;
        float f = (ss / st) / P.rr;
        p.thr = p.thr * f;
        p.d = sample_hg(p.d, S.g, u2, u3);
        p.o = x;
        return p.ev < P.max_bounces;
    }
    if (h.obj == kNone) return false;  // leaves through the open side
    v3 hp = p.o + p.d * h.t;
    v3 n = outward_normal(S, h.obj, hp);
    int kind = material_kind(S, h.obj);
    float dn = dot(n, p.d);
    v3 nf = dn < 0.0f ? n : n * -1.0f;
    if (kind == PM_MAT_DIFFUSE) {
        if (P.store) {
            uint32_t j = p.os + p.ns;
            if (j < ms.n) store(P.spos, P.spow, j, hp, p.thr, p.d, ms.scale);
        }
        p.ns += 1;
        if (!(u1 < P.rr)) return false;
        v3 a = material_albedo(S, h.obj);
        p.thr = mk3(p.thr.x * a.x / P.rr, p.thr.y * a.y / P.rr, p.thr.z * a.z / P.rr);
        p.d = sample_cosine(nf, u2, u3);
        p.o = hp + nf * kOffset;
    } else if (kind == PM_MAT_MIRROR) {
        p.d = normalize(p.d - n * (2.0f * dn));
        p.o = hp + nf * kOffset;
    } else {
        float ci = -dn;
        bool entering = ci > 0.0f;
        float ior = material_ior(S, h.obj);
        float eta = entering ? 1.0f / ior : ior;
        v3 nn = entering ? n : n * -1.0f;
        ci = fabsf(ci);
        float ct;
        float F = fresnel(ci, eta, &ct);
        if (u1 < F) {
            p.d = normalize(p.d + nn * (2.0f * ci));
            p.o = hp + nn * kOffset;
        } else {
            p.d = normalize(p.d * eta + nn * (eta * ci - ct));
            p.o = hp - nn * kOffset;
            p.glass = entering;
        }
    }
    return p.ev < P.max_bounces;
}

// Path ids come in blocks of kIdBlock per atomic. A warp always holds the
// next block's atomic in flight (issued when it takes the current one), so
// refilling lanes rarely waits for the counter; every block a warp takes is
// traced in full (the ids stay a gap-free prefix, which the record extents
// need), and the counting pass stops requesting blocks once both maps are
// full.
constexpr uint32_t kIdBlock = 32;

// The persistent per-warp loop of one scene: keep 32 live paths, refill
// empty lanes from the warp's pool of path ids until no ids are left.
__device__ __forceinline__ void trace_loop(const PScene &S, const TraceParams &P) {
    const int lane = threadIdx.x & 31;
    MapOut ms = {0u, 0u, 0.0f}, mv = {0u, 0u, 0.0f};
    uint32_t cap = P.path_cap;
    if (P.store) {
        ms.n = P.ext_s[0]; ms.paths = P.ext_s[1];
        mv.n = P.ext_v[0]; mv.paths = P.ext_v[1];
        ms.scale = ms.paths ? P.power / (float)ms.paths : 0.0f;
        mv.scale = mv.paths ? P.power / (float)mv.paths : 0.0f;
        cap = P.list ? *P.list_n : max(ms.paths, mv.paths);
    }
    Path p;
    bool live = false;
    // warp-uniform pool [pool, pool_end); lane 0 holds the prefetched block
    uint32_t pool = 0, pool_end = 0, pending = 0;
    bool has_pending = cap > 0;
    if (has_pending && lane == 0) pending = atomicAdd(P.path_counter, kIdBlock);
    for (;;) {
        const unsigned empty = __ballot_sync(0xffffffffu, !live);
        const uint32_t need = (uint32_t)__popc(empty);
        if (need && (pool < pool_end || has_pending)) {
            const uint32_t avail = pool_end - pool;
            uint32_t nb = 0;
            bool took = false;
            if (avail < need && has_pending) {
                nb = __shfl_sync(0xffffffffu, pending, 0);
                has_pending = false;
                took = true;
                bool more = nb < cap && cap - nb > kIdBlock;
                if (more && !P.store) {
                    int full = 0;
                    if (lane == 0)
                        full = *((volatile uint32_t *)P.stored_s) >= P.target_s &&
                               *((volatile uint32_t *)P.stored_v) >= P.target_v;
                    more = __shfl_sync(0xffffffffu, full, 0) == 0;
                }
                if (more) {
                    if (lane == 0) pending = atomicAdd(P.path_counter, kIdBlock);
                    has_pending = true;
                }
            }
            const uint32_t r = (uint32_t)__popc(empty & lanemask_lt());
            uint32_t id = cap;
            if (r < avail) id = pool + r;
            else if (took) id = nb + (r - avail);
            if (took) {
                const uint32_t used = need > avail ? need - avail : 0u;
                pool = nb + min(used, kIdBlock);
                pool_end = nb + kIdBlock;
                if (nb >= cap) pool = pool_end;  // nothing left below the cap
            } else {
                pool += min(need, avail);
            }
            if (!live && id < cap) {
                // the writing pass retraces only paths with a record in a map:
                // those of its list, or (without a list) the ids whose counts
                // are nonzero
                uint32_t pid = id;
                bool needed = true;
                if (P.store) {
                    if (P.list) pid = P.list[id];
                    else needed = (id < ms.paths && P.cnt_s[id] > 0u) || (id < mv.paths && P.cnt_v[id] > 0u);
                }
                if (needed) {
                    start_path(P, pid, p, S);
                    live = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, live)) {
            if (pool >= pool_end && !has_pending) break;
            continue;
        }
        if (live) {
            if (!step_path(S, P, p, ms, mv)) {
                if (!P.store) {
                    uint32_t ns = min(p.ns, (uint32_t)P.max_bounces);
                    uint32_t nv = min(p.nv, (uint32_t)P.max_bounces);
                    P.cnt_s[p.id] = ns;
                    P.cnt_v[p.id] = nv;
                    if (ns) atomicAdd(P.stored_s, ns);
                    if (nv) atomicAdd(P.stored_v, nv);
                }
                live = false;
            }
        }
    }
}

__global__ void __launch_bounds__(128) trace_kernel(PScene S, TraceParams P) { trace_loop(S, P); }

// Many scenes in one persistent launch: every block walks the scene list
// (starting at a different scene per block, so scenes are worked on side
// by side), stages the scene in shared memory and traces its paths with
// the single-scene loop until the scene's path ids run out.
__global__ void __launch_bounds__(128) trace_batch_kernel(const PScene *scenes,
                                                          const TraceParams *params, int n) {
    __shared__ PScene sS;
    __shared__ TraceParams sP;
    for (int j = 0; j < n; ++j) {
        const int sc = (int)((blockIdx.x + (unsigned)j) % (unsigned)n);
        __syncthreads();
        const uint32_t *a = reinterpret_cast<const uint32_t *>(&scenes[sc]);
        uint32_t *b = reinterpret_cast<uint32_t *>(&sS);
        for (int i = threadIdx.x; i < (int)(sizeof(PScene) / 4); i += blockDim.x) b[i] = a[i];
        const uint32_t *c = reinterpret_cast<const uint32_t *>(&params[sc]);
        uint32_t *d = reinterpret_cast<uint32_t *>(&sP);
        for (int i = threadIdx.x; i < (int)(sizeof(TraceParams) / 4); i += blockDim.x) d[i] = c[i];
        __syncthreads();
        trace_loop(sS, sP);
    }
}

// Smallest path count whose records reach the target (or all issued paths).
__device__ void find_extent(const uint32_t *off, const uint32_t *cnt, uint32_t issued, uint32_t total,
                            uint32_t target, uint32_t *extent) {
    if (target == 0) {
        extent[0] = 0;
        extent[1] = 0;
        return;
    }
    if (total <= target) {
        extent[0] = total;   // records
        extent[1] = issued;  // paths
        return;
    }
    uint32_t lo = 0, hi = issued;  // first p with off[p] + cnt[p] >= target
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (off[mid] + cnt[mid] >= target) hi = mid; else lo = mid + 1;
    }
    extent[0] = target;
    extent[1] = lo + 1;
}

__global__ void map_extent_kernel(const uint32_t *off, const uint32_t *cnt, uint32_t issued,
                                  const uint32_t *issued_dev, const uint32_t *total_p,
                                  uint32_t target, uint32_t *extent) {
    if (issued_dev) issued = min(*issued_dev, issued);
    find_extent(off, cnt, issued, *total_p, target, extent);
}

__global__ void map_extents_kernel(const ExtentJob *jobs, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ExtentJob j = jobs[i];
    if (j.cap == 0) {
        j.extent[0] = 0;
        j.extent[1] = 0;
        return;
    }
    const uint32_t total = j.off[j.cap - 1] + j.cnt[j.cap - 1];
    *j.total = total;
    find_extent(j.off, j.cnt, min(*j.issued, j.cap), total, j.target, j.extent);
}

constexpr uint32_t kNeedTile = 1024;

__device__ __forceinline__ bool path_needed(uint32_t id, const uint32_t *cnt_s, const uint32_t *cnt_v,
                                            uint32_t ps, uint32_t pv) {
    return (id < ps && cnt_s[id] > 0u) || (id < pv && cnt_v[id] > 0u);
}

// Needed paths per tile of kNeedTile ids.
__global__ void __launch_bounds__(kNeedTile) need_count_kernel(uint32_t issued, const uint32_t *cnt_s,
                                                               const uint32_t *cnt_v, const uint32_t *ext_s,
                                                               const uint32_t *ext_v, uint32_t *tile_cnt) {
    __shared__ uint32_t warp_n[kNeedTile / 32];
    const uint32_t id = blockIdx.x * kNeedTile + threadIdx.x;
    const bool need = id < issued && path_needed(id, cnt_s, cnt_v, ext_s[1], ext_v[1]);
    const uint32_t b = __popc(__ballot_sync(0xffffffffu, need));
    if ((threadIdx.x & 31) == 0) warp_n[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x < 32) {
        const uint32_t v = __reduce_add_sync(0xffffffffu, warp_n[threadIdx.x]);
        if (threadIdx.x == 0) tile_cnt[blockIdx.x] = v;
    }
}

// Each tile's needed ids, in order, at the tile's offset.
__global__ void __launch_bounds__(kNeedTile) need_scatter_kernel(uint32_t issued, const uint32_t *cnt_s,
                                                                 const uint32_t *cnt_v, const uint32_t *ext_s,
                                                                 const uint32_t *ext_v, const uint32_t *tile_off,
                                                                 uint32_t *list) {
    __shared__ uint32_t warp_off[kNeedTile / 32];
    const uint32_t id = blockIdx.x * kNeedTile + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool need = id < issued && path_needed(id, cnt_s, cnt_v, ext_s[1], ext_v[1]);
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (lane == 0) warp_off[warp] = __popc(m);
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the 32 warp counts
        const uint32_t v = warp_off[lane];
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        warp_off[lane] = x - v;
    }
    __syncthreads();
    if (need) list[tile_off[blockIdx.x] + warp_off[warp] + __popc(m & ((1u << lane) - 1u))] = id;
}

}  // namespace

uint32_t needed_tiles(uint32_t n) { return (n + kNeedTile - 1) / kNeedTile + 1; }

cudaError_t needed_paths(uint32_t issued, const uint32_t *cnt_s, const uint32_t *cnt_v,
                         const uint32_t *ext_s, const uint32_t *ext_v, uint32_t *tile_cnt,
                         uint32_t *tile_off, uint32_t *scan_tmp, uint32_t *list, uint32_t *list_n,
                         cudaStream_t s) {
    if (issued == 0) return cudaMemsetAsync(list_n, 0, sizeof(uint32_t), s);
    const uint32_t tiles = (issued + kNeedTile - 1) / kNeedTile;
    need_count_kernel<<<tiles, kNeedTile, 0, s>>>(issued, cnt_s, cnt_v, ext_s, ext_v, tile_cnt);
    note_launch();
    cudaError_t e = exclusive_scan_u32_large(tile_cnt, tile_off, tiles, list_n, scan_tmp, s);
    if (e != cudaSuccess) return e;
    need_scatter_kernel<<<tiles, kNeedTile, 0, s>>>(issued, cnt_s, cnt_v, ext_s, ext_v, tile_off, list);
    note_launch();
    return cudaGetLastError();
}

cudaError_t trace_photons(const PScene &S, const TraceParams &P, int sm_count, cudaStream_t s) {
    // 4 warps per CTA, enough CTAs to fill every SM several times over.
    trace_kernel<<<sm_count * 8, 128, 0, s>>>(S, P); note_launch();
    return cudaGetLastError();
}

cudaError_t map_extent(uint32_t issued, const uint32_t *cnt, uint32_t *off, uint32_t *total,
                       uint32_t *scan_tmp, uint32_t target, uint32_t *extent, cudaStream_t s) {
    if (issued == 0) return cudaMemsetAsync(extent, 0, 2 * sizeof(uint32_t), s);
    cudaError_t e = exclusive_scan_u32_large(cnt, off, issued, total, scan_tmp, s);
    if (e != cudaSuccess) return e;
    map_extent_kernel<<<1, 1, 0, s>>>(off, cnt, issued, nullptr, total, target, extent); note_launch();
    return cudaGetLastError();
}

cudaError_t map_extent_dev(uint32_t cap, const uint32_t *issued_dev, const uint32_t *cnt,
                           uint32_t *off, uint32_t *total, uint32_t *scan_tmp, uint32_t target,
                           uint32_t *extent, cudaStream_t s) {
    if (cap == 0) return cudaMemsetAsync(extent, 0, 2 * sizeof(uint32_t), s);
    cudaError_t e = exclusive_scan_u32_large(cnt, off, cap, total, scan_tmp, s);
    if (e != cudaSuccess) return e;
    map_extent_kernel<<<1, 1, 0, s>>>(off, cnt, cap, issued_dev, total, target, extent); note_launch();
    return cudaGetLastError();
}

cudaError_t map_extents_multi(const ExtentJob *jobs, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    map_extents_kernel<<<(n + 127) / 128, 128, 0, s>>>(jobs, n); note_launch();
    return cudaGetLastError();
}

cudaError_t trace_photons_batch(const PScene *scenes, const TraceParams *params, int n,
                                int sm_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    trace_batch_kernel<<<sm_count * 8, 128, 0, s>>>(scenes, params, n); note_launch();
    return cudaGetLastError();
}

namespace {

__global__ void pad_map_kernel(float4 *pos, float4 *pw, const uint32_t *n_dev, uint32_t cap) {
    const uint32_t n = *n_dev;
    const float inf = __int_as_float(0x7f800000);
    for (uint32_t i = n + blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
        pos[i] = make_float4(inf, inf, inf, __uint_as_float(i));
        pw[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

}  // namespace

cudaError_t pad_map(float4 *pos, float4 *pw, const uint32_t *n_dev, uint32_t cap, cudaStream_t s) {
    if (cap == 0) return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>((cap + 255) / 256, 4096);
    pad_map_kernel<<<blocks, 256, 0, s>>>(pos, pw, n_dev, cap); note_launch();
    return cudaGetLastError();
}

}  // namespace pm
