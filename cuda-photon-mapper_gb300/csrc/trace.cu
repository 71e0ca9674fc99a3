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
// Records go to fixed per-path slots (path * max_bounces + k). Compaction
// then scans the per-path counts and copies, in path order, exactly the
// map's target number of records into SoA float4 arrays, scaling power by
// the number of paths the map drew from.
#include "trace.cuh"
#include "radix_sort.cuh"

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
}

__device__ __forceinline__ void store(float4 *pos, float4 *pw, uint32_t slot, v3 x, v3 thr, v3 d) {
    pos[slot] = make_float4(x.x, x.y, x.z, 0.0f);
    pw[slot] = make_float4(thr.x, thr.y, thr.z, __uint_as_float(oct_encode(d)));
}

// One interaction of path p; returns false when the path ends.
__device__ bool step_path(const PScene &S, const TraceParams &P, Path &p) {
    p.ev += 1;
    pm_u32x4 r = philox(P.seed, p.id, (uint32_t)p.ev, 0u, P.scene_id);
    float u0 = pm_u01(r.v[0]), u1 = pm_u01(r.v[1]), u2 = pm_u01(r.v[2]), u3 = pm_u01(r.v[3]);
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
            // Delta tracking against the majorant (Woodcock et al. 1965).
            float t = 0.0f;
            for (uint32_t j = 0; j < kMaxDeltaSteps; ++j) {
                pm_u32x4 q = philox(P.seed, p.id, (uint32_t)p.ev, 1u + j, P.scene_id);
                t += -pm_logf(1.0f - pm_u01(q.v[0])) / S.sigma_max;
                if (!(t < seg)) break;
                v3 y = p.o + p.d * t;
                float s = sigma_s_at(S, y);
                float sty = s + S.sigma_a;
                if (pm_u01(q.v[1]) * S.sigma_max < sty) {
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
        if (p.nv < (uint32_t)P.max_bounces)
            store(P.vpos, P.vpow, p.id * (uint32_t)P.max_bounces + p.nv, x, p.thr, p.d);
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
        if (p.ns < (uint32_t)P.max_bounces)
            store(P.spos, P.spow, p.id * (uint32_t)P.max_bounces + p.ns, hp, p.thr, p.d);
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

__global__ void __launch_bounds__(128) trace_kernel(PScene S, TraceParams P) {
    const int lane = threadIdx.x & 31;
    Path p;
    bool live = false;
    for (;;) {
        unsigned empty = __ballot_sync(0xffffffffu, !live);
        if (empty) {
            const int leader = __ffs(empty) - 1;
            uint32_t base = P.path_cap;
            if (lane == leader) {
                bool full = *((volatile uint32_t *)P.stored_s) >= P.target_s &&
                            *((volatile uint32_t *)P.stored_v) >= P.target_v;
                if (!full) base = atomicAdd(P.path_counter, (uint32_t)__popc(empty));
            }
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!live) {
                uint32_t id = base + (uint32_t)__popc(empty & lanemask_lt());
                if (base < P.path_cap && id < P.path_cap) {
                    start_path(P, id, p, S);
                    live = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, live)) break;
        if (live) {
            if (!step_path(S, P, p)) {
                uint32_t ns = min(p.ns, (uint32_t)P.max_bounces), nv = min(p.nv, (uint32_t)P.max_bounces);
                P.cnt_s[p.id] = ns;
                P.cnt_v[p.id] = nv;
                if (ns) atomicAdd(P.stored_s, ns);
                if (nv) atomicAdd(P.stored_v, nv);
                live = false;
            }
        }
    }
}

// Smallest path count whose records reach the target (or all issued paths).
__global__ void map_extent_kernel(const uint32_t *off, const uint32_t *cnt, uint32_t issued,
                                  const uint32_t *total_p, uint32_t target, uint32_t *extent) {
    uint32_t total = *total_p;
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

__global__ void compact_kernel(const uint32_t *off, const uint32_t *cnt, const uint32_t *extent,
                               const float4 *spos, const float4 *spow, int mb, float power,
                               float4 *pos, float4 *pw) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n = extent[0], paths = extent[1];
    if (p >= paths) return;
    float scale = power / (float)paths;
    uint32_t o = off[p], c = cnt[p];
    for (uint32_t k = 0; k < c; ++k) {
        uint32_t j = o + k;
        if (j >= n) break;
        float4 a = spos[(size_t)p * mb + k];
        float4 b = spow[(size_t)p * mb + k];
        pos[j] = make_float4(a.x, a.y, a.z, __uint_as_float(j));
        pw[j] = make_float4(b.x * scale, b.y * scale, b.z * scale, b.w);
    }
}

}  // namespace

cudaError_t trace_photons(const PScene &S, const TraceParams &P, int sm_count, cudaStream_t s) {
    // 4 warps per CTA, enough CTAs to fill every SM several times over.
    trace_kernel<<<sm_count * 8, 128, 0, s>>>(S, P);
    return cudaGetLastError();
}

cudaError_t compact_map(uint32_t issued, const uint32_t *cnt, uint32_t *off, uint32_t *total,
                        uint32_t *scan_tmp, uint32_t target, uint32_t *extent, const float4 *spos,
                        const float4 *spow, int mb, float power, float4 *pos, float4 *pw,
                        cudaStream_t s) {
    if (issued == 0) return cudaMemsetAsync(extent, 0, 2 * sizeof(uint32_t), s);
    cudaError_t e = exclusive_scan_u32_large(cnt, off, issued, total, scan_tmp, s);
    if (e != cudaSuccess) return e;
    map_extent_kernel<<<1, 1, 0, s>>>(off, cnt, issued, total, target, extent);
    compact_kernel<<<(issued + 255) / 256, 256, 0, s>>>(off, cnt, extent, spos, spow, mb, power,
                                                        pos, pw);
    return cudaGetLastError();
}

}  // namespace pm
