// gather.cu -- the k-NN queries of pm_knn, the single-kernel frame render
// (eye rays, specular chains, volume march; one warp per pixel), the batched
// multi-scene render, and the k-NN estimates of query lists. The warp k-NN
// search and the estimate sum live in knn_core.cuh.
#include "launch_count.cuh"

#include <atomic>
#include "cache.cuh"
#include "eye_path.cuh"
#include "knn_core.cuh"

namespace pm {
namespace {

constexpr int kWarpsPerBlock = 4;
using namespace wknn;

template <int S>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) knn_kernel(MapView m, const float4 *q,
                                                                  uint32_t nq, int k, float r2cap,
                                                                  uint32_t *idx_out, float *d2_out) {
    __shared__ WarpScratch ws[kWarpsPerBlock];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t qi = blockIdx.x * kWarpsPerBlock + wib;
    if (qi >= nq) return;
    float4 qq = q[qi];
    const uint64_t cap = make_key(r2cap, 0xffffffffu);
    Knn<S> kn;
    kn.reset(cap, k);
    knn_search<S>(m, mk3(qq.x, qq.y, qq.z), kn, ws[wib], lane, cap);
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int j = lane * S + s;
        if (j < k) {
            idx_out[(size_t)qi * k + j] = (uint32_t)kn.key[s];
            d2_out[(size_t)qi * k + j] = key_d2(kn.key[s]);
        }
    }
}

// One pixel (one warp): eye ray, specular chain, volume march with a k-NN
// in-scattering estimate per step, k-NN estimate at the diffuse hit.
template <int S>
__device__ __forceinline__ void render_pixel(const PScene &Sc, const MapView &surf,
                                             const MapView &vol, const RenderParams &R,
                                             uint32_t pix, WarpScratch &wsc, int lane, float4 *rad,
                                             uchar4 *rgba) {
    const uint32_t px = pix % (uint32_t)R.width, py = pix / (uint32_t)R.width;
    const float u = ((float)px / (float)R.width - 0.5f) * R.aspect;
    const float v = -((float)py / (float)R.height - 0.5f);
    v3 o = mk3(Sc.cam[0], Sc.cam[1], Sc.cam[2]);
    v3 d = normalize(mk3(u, v, Sc.focal));
    const uint64_t cap = make_key(R.r2cap, 0xffffffffu);
    v3 L = mk3(0.f, 0.f, 0.f);
    float tau = 0.0f;
    bool glass = false;
    uint32_t nsurf = 0, nvol = 0;
    for (int depth = 0; depth < kMaxSpecular; ++depth) {
        PHit h = intersect_fast(Sc, o, d, 3.0e38f);
        const float tend = h.obj != kNone ? h.t : 3.0e38f;
        if (R.step > 0.0f && Sc.sigma_max > 0.0f && !glass) {
            float t0, t1;
            box_span(Sc, o, d, &t0, &t1);
            t1 = fminf(t1, tend);
            if (t0 < t1) {
                const int nst = (int)fminf(ceilf((t1 - t0) / R.step), (float)kMaxMarchSteps);
                const v3 wo = d * -1.0f;
                Knn<S> kn;
                bool warm = false;  // the previous sample found k records
                for (int j = 0; j < nst; ++j) {
                    const float ta = t0 + (float)j * R.step;
                    const float tb = fminf(t0 + (float)(j + 1) * R.step, t1);
                    const float dt = tb - ta;
                    const float tm = 0.5f * (ta + tb);
                    const v3 x = o + d * tm;
                    const float ss = Sc.het_res > 0 ? sigma_s_at(Sc, x) : Sc.sigma_s;
                    const float st = ss + Sc.sigma_a;
                    const float tau_mid = tau + st * (0.5f * dt);
                    if (vol.n > 0) {
                        if (warm) {
                            rescore<S>(vol, x, kn, wsc, cap, lane);
                        } else {
                            kn.reset(cap, R.k);
                        }
                        knn_search<S>(vol, x, kn, wsc, lane, cap, warm, R.tune);
                        int found;
                        float r2;
                        v3 e = flux_sum<S>(kn, vol, lane, 1, wo, Sc.g, cap, R.r2cap, &found, &r2);
                        warm = found == R.k;
                        ++nvol;
                        if (found > 0) {
                            const float scale = pm_expf(-tau_mid) * dt * (1.0f / (4.18879020f * r2 * sqrtf(r2)));
                            L = L + e * scale;
                        }
                    }
                    tau = tau + st * dt;
                }
            }
        }
        if (h.obj == kNone) break;
        const v3 hp = o + d * h.t;
        const v3 n = outward_normal(Sc, h.obj, hp);
        const int kind = material_kind(Sc, h.obj);
        const float dn = dot(n, d);
        const v3 nf = dn < 0.0f ? n : n * -1.0f;
        if (kind == PM_MAT_DIFFUSE) {
            if (surf.n > 0) {
                Knn<S> kn;
                kn.reset(cap, R.k);
                knn_search<S>(surf, hp, kn, wsc, lane, cap, false, R.tune);
                int found;
                float r2;
                v3 e = flux_sum<S>(kn, surf, lane, 0, nf, 0.0f, cap, R.r2cap, &found, &r2);
                ++nsurf;
                if (found > 0) {
                    const v3 a = material_albedo(Sc, h.obj);
                    const float scale = pm_expf(-tau) * (1.0f / (3.14159265f * r2)) * 0.318309886f;
                    L = L + mk3(a.x * (e.x * scale), a.y * (e.y * scale), a.z * (e.z * scale));
                }
            }
            break;
        }
        if (kind == PM_MAT_MIRROR) {
            d = normalize(d - n * (2.0f * dn));
            o = hp + nf * kOffset;
        } else {
            float ci = -dn;
            const bool entering = ci > 0.0f;
            const float ior = material_ior(Sc, h.obj);
            const float eta = entering ? 1.0f / ior : ior;
            const v3 nn = entering ? n : n * -1.0f;
            ci = fabsf(ci);
            float ct;
            const float F = fresnel(ci, eta, &ct);
            pm_u32x4 r = philox(R.seed, pix, (uint32_t)depth, kEyeSalt, R.scene_id);
            if (pm_u01(r.v[0]) < F) {
                d = normalize(d + nn * (2.0f * ci));
                o = hp + nn * kOffset;
            } else {
                d = normalize(d * eta + nn * (eta * ci - ct));
                o = hp - nn * kOffset;
                glass = entering;
            }
        }
    }
    if (lane == 0) {
        if (rad) rad[pix] = make_float4(L.x, L.y, L.z, 1.0f);
        if (rgba)
            rgba[pix] = make_uchar4(to_u8_sat((double)(L.x * R.exposure) * 255.0),
                                    to_u8_sat((double)(L.y * R.exposure) * 255.0),
                                    to_u8_sat((double)(L.z * R.exposure) * 255.0), 255);
        if (R.counters) {
            if (nsurf) atomicAdd(&R.counters[0], (unsigned long long)nsurf);
            if (nvol) atomicAdd(&R.counters[1], (unsigned long long)nvol);
        }
    }
}

// 7 resident blocks per SM (<= 73 registers): occupancy pays more than the
// spills it costs (measured 2-5 % faster on presets 1 and 2, equal on 3).
template <int S>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 7) render_kernel(PScene Sc, MapView surf,
                                                                     MapView vol, RenderParams R,
                                                                     float4 *rad, uchar4 *rgba) {
    __shared__ WarpScratch ws[kWarpsPerBlock];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t pix = blockIdx.x * kWarpsPerBlock + wib;
    const uint32_t npix = (uint32_t)R.width * (uint32_t)R.height;
    if (pix >= npix) return;
    render_pixel<S>(Sc, surf, vol, R, pix, ws[wib], lane, rad, rgba);
}

// Many scenes in one persistent launch. The work is a list of chunks --
// scene s contributes ceil(pixels_s / (4 * tile_s)) chunks of 4 warps x
// tile_s pixels -- handed out one per block by an atomic counter, so scenes
// of very different sizes and costs share the GPU dynamically. A block
// keeps the current scene in shared memory and dispatches each pixel to the
// k-list width of that scene's k, so every pixel is rendered exactly as
// the single-scene render_kernel renders it.
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 5)
    render_batch_kernel(const BatchRenderScene *scenes, const uint32_t *chunk_prefix, int nscenes,
                        uint32_t *work) {
    __shared__ WarpScratch ws[kWarpsPerBlock];
    __shared__ BatchRenderScene cur;
    __shared__ uint32_t s_chunk;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t total = chunk_prefix[nscenes];
    int cur_scene = -1;
    for (;;) {
        if (threadIdx.x == 0) s_chunk = atomicAdd(work, 1u);
        __syncthreads();
        const uint32_t chunk = s_chunk;
        if (chunk >= total) break;
        int lo = 0, hi = nscenes;  // last scene whose first chunk <= chunk
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (chunk_prefix[mid] <= chunk) lo = mid; else hi = mid;
        }
        if (lo != cur_scene) {
            const uint32_t *src = reinterpret_cast<const uint32_t *>(&scenes[lo]);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&cur);
            for (int i = threadIdx.x; i < (int)(sizeof(BatchRenderScene) / 4); i += blockDim.x)
                dst[i] = src[i];
            __syncthreads();
            cur_scene = lo;
        }
        const uint32_t npix = (uint32_t)cur.R.width * (uint32_t)cur.R.height;
        const uint32_t tile = (uint32_t)cur.tile;
        const uint32_t first = (chunk - chunk_prefix[lo]) * kWarpsPerBlock * tile + (uint32_t)wib * tile;
        for (uint32_t t = 0; t < tile; ++t) {
            const uint32_t pix = first + t;
            if (pix >= npix) break;
            switch (cur.slots) {
                case 1: render_pixel<1>(cur.sc, cur.surf, cur.vol, cur.R, pix, ws[wib], lane, cur.rad, cur.rgba); break;
                case 2: render_pixel<2>(cur.sc, cur.surf, cur.vol, cur.R, pix, ws[wib], lane, cur.rad, cur.rgba); break;
                case 3: render_pixel<3>(cur.sc, cur.surf, cur.vol, cur.R, pix, ws[wib], lane, cur.rad, cur.rgba); break;
                default: render_pixel<4>(cur.sc, cur.surf, cur.vol, cur.R, pix, ws[wib], lane, cur.rad, cur.rgba); break;
            }
        }
        __syncthreads();
    }
}

// k-NN estimates of runs of spatially sorted queries: warp w takes queries
// order[w * run .. (w + 1) * run) (indices into sel, or the queries
// themselves when sel is null), each warm-started from the previous query's
// list when both read the same map and the previous one found k records --
// the march's warm start, applied to spatial neighbours. Results land at
// out[order[j]]: the exact estimate query_knn_kernel computes, or with raw
// set the flux sum and the squared radius (-1 when nothing was found), from
// which the render's own arithmetic finishes the estimate.
// 9 blocks of 4 warps per SM (registers capped): the residency that measured
// fastest (7 by registers alone, 12 spilled too much).
template <int S>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 9)
    query_knn_run_kernel(PScene Sc, MapView surf, MapView vol, const float4 *qa, const float4 *qd,
                         const uint32_t *sel, const uint32_t *order, uint32_t n, int run, int k,
                         float r2cap, bool raw, float4 *out, uint32_t *run_ctr) {
    __shared__ WarpScratch ws[kWarpsPerBlock];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t nruns = (n + (uint32_t)run - 1) / (uint32_t)run;
    const uint64_t cap = make_key(r2cap, 0xffffffffu);
    // with run_ctr, persistent warps take runs from the counter until none
    // is left; without, warp w of the grid takes run w
    uint32_t r = blockIdx.x * kWarpsPerBlock + wib;
    for (;;) {
    if (run_ctr) {
        if (lane == 0) r = atomicAdd(run_ctr, 1u);
        r = __shfl_sync(0xffffffffu, r, 0);
    }
    if (r >= nruns) break;
    const uint32_t first = r * (uint32_t)run;
    const uint32_t last = min(first + (uint32_t)run, n);
    Knn<S> kn;
    kn.reset(cap, k);
    int prev_kind = -1;  // 0 surface, 1 volume
    bool warm = false;
    for (uint32_t j = first; j < last; ++j) {
        const uint32_t i = order[j];
        const uint32_t src = sel ? sel[i] : i;
        const float4 a = qa[src], d = qd[src];
        const int obj = __float_as_int(a.w);
        const v3 x = mk3(a.x, a.y, a.z), wo = mk3(d.x, d.y, d.z);
        const bool surface = obj != kNone;
        const int kind = surface ? 0 : 1;
        const MapView &m = surface ? surf : vol;
        v3 e = mk3(0.f, 0.f, 0.f);
        float r2out = -1.0f;
        bool found_k = false;
        if (m.n > 0) {
            const bool use_warm = warm && kind == prev_kind;
            if (use_warm) rescore<S>(m, x, kn, ws[wib], cap, lane);
            else kn.reset(cap, k);
            knn_search<S>(m, x, kn, ws[wib], lane, cap, use_warm);
            int found;
            float r2;
            const v3 dirv = surface ? facing_normal(Sc, obj, x, wo) : wo;
            e = flux_sum<S>(kn, m, lane, surface ? 0 : 1, dirv, Sc.g, cap, r2cap, &found, &r2);
            found_k = found == k;
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
        }
        if (lane == 0) out[i] = make_float4(e.x, e.y, e.z, raw ? r2out : 0.0f);
        warm = found_k;
        prev_kind = kind;
    }
    if (!run_ctr) break;
    }  // runs
}

int slots_for(int k) { return (k + 31) / 32; }

}  // namespace

cudaError_t knn_query(const MapView &m, const float4 *q, uint32_t nq, int k, float radius,
                      uint32_t *idx, float *d2, cudaStream_t s) {
    if (nq == 0) return cudaSuccess;
    const float r2 = radius * radius;
    const dim3 grid((nq + kWarpsPerBlock - 1) / kWarpsPerBlock), block(kWarpsPerBlock * 32);
    switch (slots_for(k)) {
        case 1: knn_kernel<1><<<grid, block, 0, s>>>(m, q, nq, k, r2, idx, d2); note_launch(); break;
        case 2: knn_kernel<2><<<grid, block, 0, s>>>(m, q, nq, k, r2, idx, d2); note_launch(); break;
        case 3: knn_kernel<3><<<grid, block, 0, s>>>(m, q, nq, k, r2, idx, d2); note_launch(); break;
        default: knn_kernel<4><<<grid, block, 0, s>>>(m, q, nq, k, r2, idx, d2); note_launch(); break;
    }
    return cudaGetLastError();
}

cudaError_t render_batch(const BatchRenderScene *scenes, const uint32_t *chunk_prefix, int nscenes,
                         uint32_t *work, int sm_count, cudaStream_t s) {
    if (nscenes <= 0) return cudaSuccess;
    // resident blocks per SM, per device (kept from the first eager call so
    // that graph capture issues no query)
    static std::atomic<int> per_sm_of[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int per_sm = dev < 64 ? per_sm_of[dev].load() : 0;
    if (per_sm == 0) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, render_batch_kernel,
                                                          kWarpsPerBlock * 32, 0);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        if (dev < 64) per_sm_of[dev].store(per_sm);
    }
    e = cudaMemsetAsync(work, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    render_batch_kernel<<<sm_count * per_sm, kWarpsPerBlock * 32, 0, s>>>(scenes, chunk_prefix,
                                                                          nscenes, work);
    note_launch();
    return cudaGetLastError();
}

int slots_for_k(int k) { return (k + 31) / 32; }

cudaError_t render_frame(const PScene &S, const MapView &surf, const MapView &vol,
                         const RenderParams &R, float4 *rad, uchar4 *rgba, cudaStream_t s) {
    const uint32_t npix = (uint32_t)R.width * (uint32_t)R.height;
    if (npix == 0) return cudaSuccess;
    const dim3 grid((npix + kWarpsPerBlock - 1) / kWarpsPerBlock), block(kWarpsPerBlock * 32);
    switch (slots_for(R.k)) {
        case 1: render_kernel<1><<<grid, block, 0, s>>>(S, surf, vol, R, rad, rgba); note_launch(); break;
        case 2: render_kernel<2><<<grid, block, 0, s>>>(S, surf, vol, R, rad, rgba); note_launch(); break;
        case 3: render_kernel<3><<<grid, block, 0, s>>>(S, surf, vol, R, rad, rgba); note_launch(); break;
        default: render_kernel<4><<<grid, block, 0, s>>>(S, surf, vol, R, rad, rgba); note_launch(); break;
    }
    return cudaGetLastError();
}

cudaError_t cache_knn_values_runs(const PScene &S, const MapView &surf, const MapView &vol,
                                  const float4 *qa, const float4 *qd, const uint32_t *sel,
                                  const uint32_t *order, uint32_t n, int run, int k, float radius,
                                  bool raw, float4 *val, uint32_t *run_ctr, int sm_count,
                                  cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const float r2 = radius * radius;
    const uint32_t warps = (n + (uint32_t)run - 1) / (uint32_t)run;
    dim3 grid((warps + kWarpsPerBlock - 1) / kWarpsPerBlock), block(kWarpsPerBlock * 32);
    if (run_ctr) {
        cudaError_t e = cudaMemsetAsync(run_ctr, 0, sizeof(uint32_t), s);
        if (e != cudaSuccess) return e;
    }
#define PM_RUN_LAUNCH(SL)                                                                                   \
    do {                                                                                                    \
        if (run_ctr) {                                                                                      \
            int per_sm = 1;                                                                                 \
            cudaError_t eo = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, query_knn_run_kernel<SL>, \
                                                                           kWarpsPerBlock * 32, 0);         \
            if (eo != cudaSuccess) return eo;                                                               \
            grid.x = std::min<uint32_t>(grid.x, (uint32_t)std::max(sm_count, 1) * (uint32_t)std::max(per_sm, 1)); \
        }                                                                                                   \
        query_knn_run_kernel<SL><<<grid, block, 0, s>>>(S, surf, vol, qa, qd, sel, order, n, run, k, r2, raw, val, \
                                                        run_ctr);                                           \
    } while (0)
    switch (slots_for(k)) {
        case 1: PM_RUN_LAUNCH(1); break;
        case 2: PM_RUN_LAUNCH(2); break;
        case 3: PM_RUN_LAUNCH(3); break;
        default: PM_RUN_LAUNCH(4); break;
    }
#undef PM_RUN_LAUNCH
    note_launch();
    return cudaGetLastError();
}

}  // namespace pm
