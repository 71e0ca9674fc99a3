// gather.cu -- warp-cooperative k-nearest-photon search, radiance estimates
// and the frame render (eye rays, specular chains, volume march).
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
#include "launch_count.cuh"

#include <atomic>
#include "cache.cuh"
#include "eye_path.cuh"

namespace pm {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kStackCap = 192;     // 32 entries per wide level, 6 levels: depth <= 29
constexpr int kWarpsPerBlock = 4;


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

// Kahan sum within a lane, then a compensated butterfly across the warp:
// every lane ends with the same value.
__device__ __forceinline__ void kahan_add(float &sum, float &comp, float x) {
    float y = x - comp;
    float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}
__device__ __forceinline__ float warp_csum(float sum, float comp) {
    float s = sum, e = -comp;
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        float s2 = __shfl_xor_sync(kFull, s, off);
        float e2 = __shfl_xor_sync(kFull, e, off);
        float t = s + s2;
        float bb = t - s;
        float err = (s - (t - bb)) + (s2 - bb);
        e = (e + e2) + err;
        s = t;
    }
    return s + e;
}

// Radiance-estimate numerator: sum of photon flux times weight over the
// k-NN list. mode 0: surface (weight 1 for photons arriving on the side nf
// faces, else 0); mode 1: volume (HG phase toward wo). Returns found count
// and the squared radius in *r2.
template <int S>
__device__ v3 flux_sum(const Knn<S> &kn, const MapView &m, int lane, int mode, v3 dirv, float g,
                       uint64_t cap, float r2cap, int *found, float *r2) {
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    int cnt = 0;
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int j = lane * S + s;
        if (j < kn.k && kn.key[s] != cap) {
            ++cnt;
            float4 pw = __ldg(&m.pow[kn.at[s]]);
            v3 dir = oct_decode(__float_as_uint(pw.w));
            float w;
            if (mode == 0) w = dot(dirv, dir) < 0.0f ? 1.0f : 0.0f;
            else w = hg_phase(g, dot(dir, dirv));
            kahan_add(sx, cx, pw.x * w);
            kahan_add(sy, cy, pw.y * w);
            kahan_add(sz, cz, pw.z * w);
        }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) cnt += __shfl_xor_sync(kFull, cnt, off);
    *found = cnt;
    *r2 = cnt == kn.k ? key_d2(kn.worst) : r2cap;
    return mk3(warp_csum(sx, cx), warp_csum(sy, cy), warp_csum(sz, cz));
}

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

// k-NN radiance estimate of one render query (warp per query): the same
// search, flux sum and normalisation the render kernel applies at that
// point, without the transmittance and albedo factors.
template <int S>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    query_knn_kernel(PScene Sc, MapView surf, MapView vol, const float4 *qa, const float4 *qd,
                     const uint32_t *sel, const uint32_t *out_index, uint32_t n, int k, float r2cap,
                     float4 *out) {
    __shared__ WarpScratch ws[kWarpsPerBlock];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t qi = blockIdx.x * kWarpsPerBlock + wib;
    if (qi >= n) return;
    const uint32_t src = sel ? sel[qi] : qi;
    const float4 a = qa[src], d = qd[src];
    const int obj = __float_as_int(a.w);
    const v3 x = mk3(a.x, a.y, a.z), wo = mk3(d.x, d.y, d.z);
    const bool surface = obj != kNone;
    const MapView &m = surface ? surf : vol;
    v3 e = mk3(0.f, 0.f, 0.f);
    if (m.n > 0) {
        const uint64_t cap = make_key(r2cap, 0xffffffffu);
        Knn<S> kn;
        kn.reset(cap, k);
        knn_search<S>(m, x, kn, ws[wib], lane, cap);
        int found;
        float r2;
        const v3 dirv = surface ? facing_normal(Sc, obj, x, wo) : wo;
        e = flux_sum<S>(kn, m, lane, surface ? 0 : 1, dirv, Sc.g, cap, r2cap, &found, &r2);
        if (found > 0) {
            const float sc = surface ? (1.0f / (3.14159265f * r2)) * 0.318309886f
                                     : 1.0f / (4.18879020f * r2 * sqrtf(r2));
            e = e * sc;
        } else {
            e = mk3(0.f, 0.f, 0.f);
        }
    }
    if (lane == 0) out[out_index ? out_index[qi] : qi] = make_float4(e.x, e.y, e.z, 0.0f);
}

// k-NN estimates of runs of spatially sorted queries: warp w takes queries
// order[w * run .. (w + 1) * run) (indices into sel, or the queries
// themselves when sel is null), each warm-started from the previous query's
// list when both read the same map and the previous one found k records --
// the march's warm start, applied to spatial neighbours. Results land at
// out[order[j]]: the exact estimate query_knn_kernel computes, or with raw
// set the flux sum and the squared radius (-1 when nothing was found), from
// which the render's own arithmetic finishes the estimate.
template <int S>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    query_knn_run_kernel(PScene Sc, MapView surf, MapView vol, const float4 *qa, const float4 *qd,
                         const uint32_t *sel, const uint32_t *order, uint32_t n, int run, int k,
                         float r2cap, bool raw, float4 *out) {
    __shared__ WarpScratch ws[kWarpsPerBlock];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t first = (blockIdx.x * kWarpsPerBlock + wib) * (uint32_t)run;
    if (first >= n) return;
    const uint32_t last = min(first + (uint32_t)run, n);
    const uint64_t cap = make_key(r2cap, 0xffffffffu);
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

cudaError_t cache_knn_values(const PScene &S, const MapView &surf, const MapView &vol,
                             const float4 *qa, const float4 *qd, const uint32_t *sel,
                             const uint32_t *out_index, uint32_t n, int k, float radius, float4 *val,
                             cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const float r2 = radius * radius;
    const dim3 grid((n + kWarpsPerBlock - 1) / kWarpsPerBlock), block(kWarpsPerBlock * 32);
    switch (slots_for(k)) {
        case 1: query_knn_kernel<1><<<grid, block, 0, s>>>(S, surf, vol, qa, qd, sel, out_index, n, k, r2, val); break;
        case 2: query_knn_kernel<2><<<grid, block, 0, s>>>(S, surf, vol, qa, qd, sel, out_index, n, k, r2, val); break;
        case 3: query_knn_kernel<3><<<grid, block, 0, s>>>(S, surf, vol, qa, qd, sel, out_index, n, k, r2, val); break;
        default: query_knn_kernel<4><<<grid, block, 0, s>>>(S, surf, vol, qa, qd, sel, out_index, n, k, r2, val); break;
    }
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_knn_values_runs(const PScene &S, const MapView &surf, const MapView &vol,
                                  const float4 *qa, const float4 *qd, const uint32_t *sel,
                                  const uint32_t *order, uint32_t n, int run, int k, float radius,
                                  bool raw, float4 *val, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const float r2 = radius * radius;
    const uint32_t warps = (n + (uint32_t)run - 1) / (uint32_t)run;
    const dim3 grid((warps + kWarpsPerBlock - 1) / kWarpsPerBlock), block(kWarpsPerBlock * 32);
    switch (slots_for(k)) {
        case 1: query_knn_run_kernel<1><<<grid, block, 0, s>>>(S, surf, vol, qa, qd, sel, order, n, run, k, r2, raw, val); break;
        case 2: query_knn_run_kernel<2><<<grid, block, 0, s>>>(S, surf, vol, qa, qd, sel, order, n, run, k, r2, raw, val); break;
        case 3: query_knn_run_kernel<3><<<grid, block, 0, s>>>(S, surf, vol, qa, qd, sel, order, n, run, k, r2, raw, val); break;
        default: query_knn_run_kernel<4><<<grid, block, 0, s>>>(S, surf, vol, qa, qd, sel, order, n, run, k, r2, raw, val); break;
    }
    note_launch();
    return cudaGetLastError();
}

}  // namespace pm
