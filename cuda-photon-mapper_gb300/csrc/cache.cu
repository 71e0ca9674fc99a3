// cache.cu -- the learned radiance cache: query lists, hash-grid encoding,
// the fused tcgen05 training and inference kernels, Adam, composite.
//
// Network: x (64 features) -> 4 x [64 x 64, ReLU] -> [64 x 16] -> rgb in
// columns 0..2; no biases (feature 52 is a constant 1). Features:
//   0..31   16 hash-grid levels x 2 fp16 features, trilinear
//   32..47  real spherical harmonics of wo, degrees 0..3
//   48..50  facing normal (diffuse queries; zero in the medium)
//   51      1 for a diffuse query, 0 for a medium query
//   52      1
// Loss: relative L2, sum_c (y_c - t_c)^2 / (y_c^2 + eps) with y_c held
// constant in the denominator, averaged over 3 x batch (targets are
// divided by their mean first; eps = 0.01 by default).
//
// Tensor-core tiles hold 128 samples (one per TMEM lane; thread s of the
// 128-thread CTA owns sample s). Activations live in shared memory as bf16
// in the no-swizzle core-matrix layout of tc.cuh. The training kernel keeps
// every layer's activations (H0 = x .. H4) and activation gradients (dZ1 ..
// dZ4) of the tile in "pair" buffers of 128 samples x 128 features, so that
//   forward  Z_{l+1} = H_l W_l       A = H_l  (K-major),  B = W_l (K-major)
//   backward dH_l = dZ_{l+1} W_l^T   A = dZ   (K-major),  B = W_l (MN-major)
//   weights  [dW_a | . ; . | dW_b] = [H_a ; H_b]^T [dZ_a+1 , dZ_b+1]
//                                    A, B = the pair buffers (MN-major)
// all read the same bytes: no transposed copies. The weight gradients of a
// CTA accumulate over its tiles in TMEM (M = 128 rows = two layers' inputs,
// N = 128 columns = their two output blocks; the off-diagonal blocks are
// unused) and are added to global memory once at the end.
#include "cache.cuh"
#include "eye_path.cuh"
#include "launch_count.cuh"
#include "radix_sort.cuh"
#include "tc.cuh"

#include <cuda_bf16.h>
#include <algorithm>
#include <cmath>

namespace pm {
namespace {

constexpr int kThreads = kCacheTile;

// Shared-memory layout of the training kernel (bytes).
constexpr uint32_t kWBytes = 4 * 8192 + 2048;          // bf16 weights, B-operand layout
constexpr uint32_t kPair = 32768;                      // 128 samples x 128 features bf16
constexpr uint32_t kOffP0 = kWBytes;                   // H0 | H1
constexpr uint32_t kOffP1 = kOffP0 + kPair;            // H2 | H3
constexpr uint32_t kOffP2 = kOffP1 + kPair;            // H4 | unused
constexpr uint32_t kOffQ0 = kOffP2 + kPair;            // dZ1 | dZ2
constexpr uint32_t kOffQ1 = kOffQ0 + kPair;            // dZ3 | dZ4
constexpr uint32_t kOffGY = kOffQ1 + kPair;            // dL/dy, 128 x 16
constexpr uint32_t kOffXS = kOffGY + 4096;             // next tile's encoded features (staging)
constexpr uint32_t kXTile = 16384;                     // 128 samples x 64 features bf16
constexpr uint32_t kTrainSmem = kOffXS + kXTile;
constexpr uint32_t kPairSbo = 2048;                    // 8-sample groups in a pair buffer
// Inference: weights + one 128 x 64 activation tile per pipeline.
constexpr uint32_t kOffAct = kWBytes;
constexpr uint32_t kActSbo = 1024;

// TMEM columns of the training kernel.
constexpr uint32_t kColDW01 = 128, kColDW23 = 256, kColDW4 = 384, kTrainCols = 512;
constexpr uint32_t kInferCols = 64;  // per pipeline

// Byte offset of feature f (a multiple of 8) of sample s in an activation
// buffer whose 8-sample groups are sbo bytes apart.
__device__ __forceinline__ uint32_t row_off(int s, int f, uint32_t sbo) {
    return (uint32_t)(s >> 3) * sbo + (uint32_t)(f >> 3) * 128u + (uint32_t)(s & 7) * 16u;
}

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ void st8(unsigned char *base, uint32_t off, const float *v) {
    *reinterpret_cast<uint4 *>(base + off) = make_uint4(pack_bf2(v[0], v[1]), pack_bf2(v[2], v[3]),
                                                        pack_bf2(v[4], v[5]), pack_bf2(v[6], v[7]));
}

__device__ __forceinline__ void ld8(const unsigned char *base, uint32_t off, float *v) {
    const uint4 u = *reinterpret_cast<const uint4 *>(base + off);
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        v[2 * j] = __uint_as_float(w[j] << 16);
        v[2 * j + 1] = __uint_as_float(w[j] & 0xffff0000u);
    }
}

// Byte offset of fp32 weight i ([in][out] layers) in the bf16 B-operand
// image: element (out, in) of layer l at l * 8192 + core_offset(out, in,
// 64); the output layer (16 x 64) at 32768.
__device__ __forceinline__ uint32_t weight_image_offset(int i) {
    if (i < 4 * 4096) {
        const int l = i >> 12, r = i & 4095;
        return (uint32_t)l * 8192u + core_offset(r & 63, r >> 6, 64);
    }
    const int r = i - 4 * 4096;
    return 32768u + core_offset(r & 15, r >> 4, 64);
}

static_assert(kWBytes == kCacheWImageBytes, "weight image size");

// The CTA's copy of the weight image: one bulk copy (TMA) issued by thread
// 0 on `mbar` (phase 0), which every thread then waits for. False when the
// bounded wait ran out.
__device__ bool load_weight_image(unsigned char *sw, const uint4 *img, uint64_t *mbar,
                                  uint32_t polls) {
    if (threadIdx.x == 0) {
        mbar_init(mbar);
        bulk_load(sw, img, kWBytes, mbar);
    }
    __syncthreads();
    return mbar_wait_drain(mbar, 0, polls);
}

// A bounded wait of the inference kernel: under a lowered first bound
// (kLowered) the drain of mbar_wait_drain, else the plain wait under the
// default bound. Kept apart because the runtime bound and the drain path
// cost the inference kernel its register allocation (61 instead of 96
// registers, 18 % slower on preset 2).
template <bool kLowered>
__device__ __forceinline__ bool infer_wait(uint64_t *mbar, uint32_t phase, uint32_t polls) {
    if (kLowered) return mbar_wait_drain(mbar, phase, polls);
    return mbar_wait(mbar, phase);
}

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

// One table-gradient term as a fixed-point integer: the exact product with
// 2^kTableGradShift (a power of two), rounded once to the nearest integer.
__device__ __forceinline__ long long to_grad_fixed(float x) {
    return __float2ll_rn(x * 0x1p44f);
}
static_assert(kTableGradShift == 44, "to_grad_fixed and from_grad_fixed use 2^44");
__device__ __forceinline__ float from_grad_fixed(long long q) { return __ll2float_rn(q) * 0x1p-44f; }

// Table slots and trilinear weights of the 8 corners around p (in [0,1]^3)
// on level l: vertices 0..res per axis, dense indexing while (res+1)^3 fits
// the level, the spatial hash x ^ 2654435761 y ^ 805459861 z beyond.
__device__ __forceinline__ void level_corners(const CacheGrid &g, int l, float px, float py,
                                              float pz, uint32_t *idx, float *w) {
    const int r = g.res[l];
    const float fx = px * (float)r, fy = py * (float)r, fz = pz * (float)r;
    const int ix = min((int)fx, r - 1), iy = min((int)fy, r - 1), iz = min((int)fz, r - 1);
    const float tx = fx - (float)ix, ty = fy - (float)iy, tz = fz - (float)iz;
    const uint32_t stride = (uint32_t)r + 1u;
    const bool dense = (uint64_t)stride * stride * stride <= (1ull << g.log2_t);
    const uint32_t mask = (1u << g.log2_t) - 1u;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t cx = (uint32_t)ix + (c & 1), cy = (uint32_t)iy + ((c >> 1) & 1),
                       cz = (uint32_t)iz + (c >> 2);
        idx[c] = dense ? cx + stride * (cy + stride * cz)
                       : (cx ^ (cy * 2654435761u) ^ (cz * 805459861u)) & mask;
        const float wx = (c & 1) ? tx : 1.0f - tx;
        const float wy = (c & 2) ? ty : 1.0f - ty;
        const float wz = (c & 4) ? tz : 1.0f - tz;
        w[c] = (wx * wy) * wz;
    }
}

// Real spherical harmonics of a unit direction, degrees 0..3.
__device__ __forceinline__ void sh16(float x, float y, float z, float *o) {
    const float xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = -0.48860251190291987f * y;
    o[2] = 0.48860251190291987f * z;
    o[3] = -0.48860251190291987f * x;
    o[4] = 1.0925484305920792f * x * y;
    o[5] = -1.0925484305920792f * y * z;
    o[6] = 0.94617469575755997f * zz - 0.31539156525251999f;
    o[7] = -1.0925484305920792f * x * z;
    o[8] = 0.54627421529603959f * (xx - yy);
    o[9] = 0.59004358992664352f * y * (-3.0f * xx + yy);
    o[10] = 2.8906114426405538f * x * y * z;
    o[11] = 0.45704579946446572f * y * (1.0f - 5.0f * zz);
    o[12] = 0.3731763325901154f * z * (5.0f * zz - 3.0f);
    o[13] = 0.45704579946446572f * x * (1.0f - 5.0f * zz);
    o[14] = 1.4453057213202769f * z * (xx - yy);
    o[15] = 0.59004358992664352f * x * (-xx + 3.0f * yy);
}

struct QueryPos {
    float px, py, pz;
};

__device__ __forceinline__ QueryPos unit_pos(const CacheGrid &g, float4 a) {
    QueryPos q;
    q.px = clamp01((a.x - g.lo[0]) * g.inv_size[0]);
    q.py = clamp01((a.y - g.lo[1]) * g.inv_size[1]);
    q.pz = clamp01((a.z - g.lo[2]) * g.inv_size[2]);
    return q;
}

// Encodes one query into row `row` of an activation buffer (features
// 0..63, bf16); dbg (nullable) receives the fp32 features.
__device__ void encode_row(unsigned char *act, uint32_t sbo, int row, const CacheGrid &g,
                           const __half2 *tab, const PScene &Sc, float4 a, float4 d, bool valid,
                           float *dbg) {
    float v[8];
    if (!valid) {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = 0.0f;
#pragma unroll
        for (int c = 0; c < 8; ++c) st8(act, row_off(row, 8 * c, sbo), v);
        return;
    }
    const QueryPos q = unit_pos(g, a);
    const size_t T = (size_t)1 << g.log2_t;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int l = 4 * c + j;
            float f0 = 0.0f, f1 = 0.0f;
            if (l < g.levels) {
                uint32_t idx[8];
                float w[8];
                level_corners(g, l, q.px, q.py, q.pz, idx, w);
                const __half2 *lv = tab + (size_t)l * T;
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    // fused (the library builds with contraction off): the
                    // encoding has no bit-exact counterpart to match
                    const float2 h = __half22float2(__ldg(lv + idx[k]));
                    f0 = __fmaf_rn(w[k], h.x, f0);
                    f1 = __fmaf_rn(w[k], h.y, f1);
                }
            }
            v[2 * j] = f0;
            v[2 * j + 1] = f1;
        }
        st8(act, row_off(row, 8 * c, sbo), v);
        if (dbg)
#pragma unroll
            for (int j = 0; j < 8; ++j) dbg[8 * c + j] = v[j];
    }
    float sh[16];
    sh16(d.x, d.y, d.z, sh);
    st8(act, row_off(row, 32, sbo), sh);
    st8(act, row_off(row, 40, sbo), sh + 8);
    const int obj = __float_as_int(a.w);
    v3 nf = mk3(0.0f, 0.0f, 0.0f);
    float kind = 0.0f;
    if (obj != kNone) {
        nf = facing_normal(Sc, obj, mk3(a.x, a.y, a.z), mk3(d.x, d.y, d.z));
        kind = 1.0f;
    }
    float t[16] = {nf.x, nf.y, nf.z, kind, 1.0f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    st8(act, row_off(row, 48, sbo), t);
    st8(act, row_off(row, 56, sbo), t + 8);
    if (dbg) {
#pragma unroll
        for (int j = 0; j < 16; ++j) dbg[32 + j] = sh[j];
#pragma unroll
        for (int j = 0; j < 16; ++j) dbg[48 + j] = t[j];
    }
}

// Runs `issue` on thread 0 after the CTA's shared-memory writes are visible
// to the tensor core, commits, and waits for completion. false when the
// wait's first bound (polls) ran out; the MMAs have completed either way
// (mbar_wait_drain), so the caller may stop at the end of its tile.
template <class F>
__device__ __forceinline__ bool tc_round(uint64_t *mbar, uint32_t &phase, uint32_t polls, F issue) {
    publish_smem();
    __syncthreads();
    after_sync();
    if (threadIdx.x == 0) {
        issue();
        mma_commit(mbar);
    }
    const bool ok = mbar_wait_drain(mbar, phase, polls);
    phase ^= 1u;
    after_sync();
    return ok;
}

// The same for one 128-thread pipeline of a larger CTA: named barrier `bar`
// instead of the CTA barrier; `issuer` is the pipeline's first thread.
template <bool kLowered, class F>
__device__ __forceinline__ bool tc_round_group(uint64_t *mbar, uint32_t &phase, uint32_t bar,
                                               bool issuer, uint32_t polls, F issue) {
    publish_smem();
    named_sync(bar, kThreads);
    after_sync();
    if (issuer) {
        issue();
        mma_commit(mbar);
    }
    const bool ok = infer_wait<kLowered>(mbar, phase, polls);
    phase ^= 1u;
    after_sync();
    return ok;
}

// K-major operand descriptor sequence helper: nk MMAs of K = 16.
__device__ __forceinline__ void mma_chain(uint32_t d, uint32_t a, uint32_t a_step, uint32_t a_lbo,
                                          uint32_t a_sbo, uint32_t b, uint32_t b_step,
                                          uint32_t b_lbo, uint32_t b_sbo, int nk, uint32_t idesc,
                                          bool acc_first) {
    for (int k = 0; k < nk; ++k)
        mma_bf16(d, smem_desc(a + k * a_step, a_lbo, a_sbo), smem_desc(b + k * b_step, b_lbo, b_sbo),
                 idesc, (k > 0 || acc_first) ? 1u : 0u);
}

// Hidden-layer epilogue: TMEM columns 0..63 of this thread's row -> ReLU ->
// bf16 at dst (activation buffer with 8-sample stride sbo).
__device__ __forceinline__ void relu_out(uint32_t taddr, unsigned char *dst, uint32_t sbo, int row) {
#pragma unroll 1
    for (int c = 0; c < 64; c += 16) {
        float v[16];
        tmem_ld16(taddr, c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j], 0.0f);
        st8(dst, row_off(row, c, sbo), v);
        st8(dst, row_off(row, c + 8, sbo), v + 8);
    }
}

// Backward epilogue: dZ = dH (TMEM 0..63) where H > 0, else 0.
__device__ __forceinline__ void relu_grad(uint32_t taddr, const unsigned char *h, unsigned char *dz,
                                          int row) {
#pragma unroll 1
    for (int c = 0; c < 64; c += 16) {
        float v[16], hv[16];
        tmem_ld16(taddr, c, v);
        ld8(h, row_off(row, c, kPairSbo), hv);
        ld8(h, row_off(row, c + 8, kPairSbo), hv + 8);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = hv[j] > 0.0f ? v[j] : 0.0f;
        st8(dz, row_off(row, c, kPairSbo), v);
        st8(dz, row_off(row, c + 8, kPairSbo), v + 8);
    }
}

// The encoded features of samples 0..rows-1 (query sel[i], zero rows from n
// on) as tile images: tile t = samples 128t..128t+127 in the K-major
// core-matrix layout with 8-sample groups 1 KB apart (16 KB per tile), the
// layout the training kernel copies into its first activation buffer. One
// thread per sample: the 128 hash-table reads of an encoding run at full
// occupancy here instead of on the tensor-core kernel's critical path.
__global__ void __launch_bounds__(256)
    encode_kernel(CacheGrid g, const __half2 *tab, PScene Sc, const float4 *qa, const float4 *qd,
                  const uint32_t *sel, uint32_t n, uint32_t rows, unsigned char *xt, float *x_out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
        const bool valid = i < n;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), d = a;
        if (valid) {
            const uint32_t qi = sel ? sel[i] : i;
            a = qa[qi];
            d = qd[qi];
        }
        encode_row(xt + (size_t)(i >> 7) * kXTile, kActSbo, (int)(i & 127u), g, tab, Sc, a, d, valid,
                   (valid && x_out) ? x_out + (size_t)i * 64 : nullptr);
    }
}

__global__ void __launch_bounds__(kThreads, 1)
    train_kernel(CacheParams p, const unsigned char *xt, const float4 *val, uint32_t n,
                 float inv_scale, float loss_norm, float rel_eps, float *y_out) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar, wbar, xbar;
    __shared__ uint32_t taddr_s;
    __shared__ int abort_s;
    __shared__ float red[kThreads / 32];
    const int s = threadIdx.x, warp = s >> 5;
    const uint32_t ntiles = (n + kThreads - 1) / kThreads;

    bool ok = load_weight_image(sm, p.w_img, &wbar, p.wait_polls);
    for (uint32_t i = s; i < kPair / 16; i += kThreads)  // the unused half of P2 stays finite
        reinterpret_cast<uint4 *>(sm + kOffP2)[i] = make_uint4(0, 0, 0, 0);
    if (s == 0) {
        mbar_init(&mbar);
        mbar_init(&xbar);
        abort_s = 0;
        // the first tile's features into the staging buffer
        if (blockIdx.x < ntiles) bulk_load(sm + kOffXS, xt + (size_t)blockIdx.x * kXTile, kXTile, &xbar);
    }
    if (warp == 0) tmem_alloc(&taddr_s, kTrainCols);
    publish_smem();
    __syncthreads();
    after_sync();
    const uint32_t taddr = taddr_s;
    const uint32_t base = smem_addr(sm);
    const uint32_t aP[3] = {base + kOffP0, base + kOffP1, base + kOffP2};
    const uint32_t aQ[2] = {base + kOffQ0, base + kOffQ1};
    const uint32_t aW = base, aGY = base + kOffGY;
    uint32_t phase = 0, xphase = 0;
    bool xpending = blockIdx.x < ntiles;  // a staging copy in flight
    float lsum = 0.0f;
    bool first = true;
    if (!ok) abort_s = 1;
    __syncthreads();
    if (abort_s) ok = false;

    for (uint32_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const uint32_t i = tile * kThreads + s;
        const bool valid = i < n;
        // this tile's features: staging buffer -> H0 (the first half of
        // pair P0, whose 8-sample groups are 2 KB apart)
        ok &= mbar_wait_drain(&xbar, xphase, p.wait_polls);
        xphase ^= 1u;
        xpending = false;
#pragma unroll
        for (int j = 0; j < (int)(kXTile / 16 / kThreads); ++j) {
            const uint32_t u = (uint32_t)(j * kThreads + s);
            *reinterpret_cast<uint4 *>(sm + kOffP0 + (u >> 6) * 2048u + (u & 63u) * 16u) =
                *reinterpret_cast<const uint4 *>(sm + kOffXS + u * 16u);
        }
        const uint32_t next = tile + gridDim.x;
        const bool prefetch = next < ntiles;
        // forward, hidden layers: H_{l+1} = relu(H_l W_l); the first round
        // also starts the copy of the next tile's features into the staging
        // buffer, whose reads above the round's barrier have completed
        for (int l = 0; l < 4; ++l) {
            const uint32_t src = aP[l >> 1] + (uint32_t)(l & 1) * 1024u;
            ok &= tc_round(&mbar, phase, p.wait_polls, [&] {
                mma_chain(taddr, src, 256, 128, kPairSbo, aW + (uint32_t)l * 8192u, 256, 128, 1024, 4,
                          idesc_bf16(128, 64), false);
                if (l == 0 && prefetch) bulk_load(sm + kOffXS, xt + (size_t)next * kXTile, kXTile, &xbar);
            });
            if (l == 0) xpending = prefetch;
            const int o = l + 1;
            relu_out(taddr, sm + kOffP0 + (uint32_t)(o >> 1) * kPair + (uint32_t)(o & 1) * 1024u,
                     kPairSbo, s);
        }
        // output layer: y = H4 W4
        ok &= tc_round(&mbar, phase, p.wait_polls, [&] {
            mma_chain(taddr, aP[2], 256, 128, kPairSbo, aW + 32768u, 256, 128, 1024, 4,
                      idesc_bf16(128, 16), false);
        });
        float y[16];
        tmem_ld16(taddr, 0, y);
        float gy[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) gy[j] = 0.0f;
        if (valid) {
            const float4 t4 = val[i];
            const float isc = p.scale_dev ? 1.0f / __ldg(p.scale_dev) : inv_scale;
            const float t[3] = {t4.x * isc, t4.y * isc, t4.z * isc};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float diff = y[c] - t[c];
                const float den = y[c] * y[c] + rel_eps;
                lsum += diff * diff / den;
                gy[c] = 2.0f * diff / den * loss_norm;
            }
            if (y_out)
                reinterpret_cast<float4 *>(y_out)[i] = make_float4(y[0], y[1], y[2], 0.0f);
        }
        {
            const uint32_t go = (uint32_t)(s >> 3) * 256u + (uint32_t)(s & 7) * 16u;
            st8(sm + kOffGY, go, gy);
            st8(sm + kOffGY, go + 128u, gy + 8);
        }
        // dH4 = GY W4^T (B = the output layer read MN-major)
        ok &= tc_round(&mbar, phase, p.wait_polls, [&] {
            mma_chain(taddr, aGY, 0, 128, 256, aW + 32768u, 0, 1024, 128, 1,
                      idesc_bf16(128, 64, 0, 1), false);
        });
        relu_grad(taddr, sm + kOffP2, sm + kOffQ1 + 1024u, s);  // dZ4
        // dH_l = dZ_{l+1} W_l^T for l = 3, 2, 1
        for (int l = 3; l >= 1; --l) {
            const uint32_t dz = aQ[l >> 1] + (uint32_t)(l & 1) * 1024u;  // dZ_{l+1}
            ok &= tc_round(&mbar, phase, p.wait_polls, [&] {
                mma_chain(taddr, dz, 256, 128, kPairSbo, aW + (uint32_t)l * 8192u, 2048, 1024, 128, 4,
                          idesc_bf16(128, 64, 0, 1), false);
            });
            const unsigned char *h = sm + kOffP0 + (uint32_t)(l >> 1) * kPair + (uint32_t)(l & 1) * 1024u;
            unsigned char *dzl = sm + kOffQ0 + (uint32_t)((l - 1) >> 1) * kPair + (uint32_t)((l - 1) & 1) * 1024u;
            relu_grad(taddr, h, dzl, s);
        }
        // dX = dZ1 W0^T, and the weight gradients of the tile
        const bool acc = !first;
        ok &= tc_round(&mbar, phase, p.wait_polls, [&] {
            mma_chain(taddr, aQ[0], 256, 128, kPairSbo, aW, 2048, 1024, 128, 4,
                      idesc_bf16(128, 64, 0, 1), false);
            mma_chain(taddr + kColDW01, aP[0], 4096, kPairSbo, 128, aQ[0], 4096, kPairSbo, 128, 8,
                      idesc_bf16(128, 128, 1, 1), acc);
            mma_chain(taddr + kColDW23, aP[1], 4096, kPairSbo, 128, aQ[1], 4096, kPairSbo, 128, 8,
                      idesc_bf16(128, 128, 1, 1), acc);
            mma_chain(taddr + kColDW4, aP[2], 4096, kPairSbo, 128, aGY, 512, 256, 128, 8,
                      idesc_bf16(128, 16, 1, 1), acc);
        });
        first = false;
        float dx[32];
        tmem_ld16(taddr, 0, dx);
        tmem_ld16(taddr, 16, dx + 16);
        // the gradient of the 32 hash-grid features; table_scatter_kernel
        // spreads it over the table entries after this kernel
        if (valid && ok) {
            float4 *row = p.dx + (size_t)i * 8;
#pragma unroll
            for (int j = 0; j < 8; ++j)
                row[j] = make_float4(dx[4 * j], dx[4 * j + 1], dx[4 * j + 2], dx[4 * j + 3]);
        }
        if (!ok) abort_s = 1;
        __syncthreads();
        if (abort_s) {
            ok = false;
            break;
        }
    }
    // a staging copy still in flight (the loop stopped early) completes
    // before the CTA's shared memory is released
    if (xpending) mbar_wait(&xbar, xphase, kMbarSpin);
    // weight gradients of this CTA -> its row of partial sums (every CTA
    // has at least one tile: the grid is at most the tile count)
    float *part = p.w_part + (size_t)blockIdx.x * kCacheWeights;
    if (!first && ok) {
        const int half = warp >> 1;
        const int in = s & 63;
#pragma unroll 1
        for (int pr = 0; pr < 2; ++pr) {
            const int l = 2 * pr + half;
            const uint32_t col = (pr == 0 ? kColDW01 : kColDW23) + (uint32_t)half * 64u;
#pragma unroll 1
            for (int c = 0; c < 64; c += 16) {
                float v[16];
                tmem_ld16(taddr, (int)col + c, v);
#pragma unroll
                float4 *dst = reinterpret_cast<float4 *>(part + l * 4096 + in * 64 + c);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            }
        }
        if (warp < 2) {
            float v[16];
            tmem_ld16(taddr, (int)kColDW4, v);
#pragma unroll
            float4 *dst = reinterpret_cast<float4 *>(part + 4 * 4096 + s * 16);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        }
    }
    if (first || !ok)  // no valid gradient: the row must not carry stale sums
        for (int i = s; i < kCacheWeights; i += kThreads) part[i] = 0.0f;
    if (!ok && s == 0) atomicExch(p.status, 1);
#pragma unroll
    for (int off = 16; off; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    if ((s & 31) == 0) red[warp] = lsum;
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (s == 0) p.loss_part[blockIdx.x] = (red[0] + red[1] + red[2] + red[3]) * loss_norm;
    if (warp == 0) tmem_free(taddr, kTrainCols);
}

// Inference: kInferPipes independent 128-query pipelines per CTA share one
// copy of the weights; each has its own activation tile, TMEM columns,
// mbarrier and named barrier, so while one pipeline waits on the tensor core
// or on hash-table reads the others issue.
constexpr int kInferPipes = 4;
constexpr uint32_t kInferSmem = kOffAct + 16384u * kInferPipes;

template <bool kLowered>
__global__ void __launch_bounds__(kThreads * kInferPipes)
    infer_kernel(CacheGrid g, CacheParams p, PScene Sc, const float4 *qa, const float4 *qd,
                 const uint32_t *order, uint32_t n, float out_scale, float4 *val) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar[kInferPipes], wbar;
    __shared__ uint32_t taddr_s;
    __shared__ int abort_s[kInferPipes];
    const int pipe = threadIdx.x / kThreads, s = threadIdx.x % kThreads;
    const int warp = threadIdx.x >> 5;
    const uint32_t bar = 1u + (uint32_t)pipe;
    const bool issuer = s == 0;
    const uint32_t ntiles = (n + kThreads - 1) / kThreads;
    if (threadIdx.x == 0) {
        mbar_init(&wbar);
        bulk_load(sm, p.w_img, kWBytes, &wbar);
    }
    __syncthreads();
    const bool wok = infer_wait<kLowered>(&wbar, 0, p.wait_polls);
    if (issuer) {
        mbar_init(&mbar[pipe]);
        abort_s[pipe] = wok ? 0 : 1;
    }
    if (warp == 0) tmem_alloc(&taddr_s, kInferCols * kInferPipes);
    publish_smem();
    __syncthreads();
    after_sync();
    const uint32_t taddr = taddr_s + (uint32_t)pipe * kInferCols;
    const uint32_t aW = smem_addr(sm), aA = aW + kOffAct + (uint32_t)pipe * 16384u;
    unsigned char *act = sm + kOffAct + pipe * 16384;
    uint32_t phase = 0;
    bool ok = abort_s[pipe] == 0;
    for (uint32_t tile = blockIdx.x * kInferPipes + pipe; tile < ntiles && ok;
         tile += gridDim.x * kInferPipes) {
        const uint32_t j = tile * kThreads + s;
        const bool valid = j < n;
        uint32_t i = j;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), d = a;
        if (valid) {
            if (order) i = order[j];
            a = qa[i];
            d = qd[i];
        }
        encode_row(act, kActSbo, s, g, p.table_h, Sc, a, d, valid, nullptr);
        for (int l = 0; l < 4; ++l) {
            ok &= tc_round_group<kLowered>(&mbar[pipe], phase, bar, issuer, p.wait_polls, [&] {
                mma_chain(taddr, aA, 256, 128, kActSbo, aW + (uint32_t)l * 8192u, 256, 128, 1024, 4,
                          idesc_bf16(128, 64), false);
            });
            relu_out(taddr, act, kActSbo, s);
        }
        ok &= tc_round_group<kLowered>(&mbar[pipe], phase, bar, issuer, p.wait_polls, [&] {
            mma_chain(taddr, aA, 256, 128, kActSbo, aW + 32768u, 256, 128, 1024, 4,
                      idesc_bf16(128, 16), false);
        });
        float y[16];
        tmem_ld16(taddr, 0, y);
        if (valid && ok) {
            const float osc = p.scale_dev ? __ldg(p.scale_dev) : out_scale;
            val[i] = make_float4(fmaxf(y[0], 0.0f) * osc, fmaxf(y[1], 0.0f) * osc, fmaxf(y[2], 0.0f) * osc, 0.0f);
        }
        if (!ok) abort_s[pipe] = 1;
        asm volatile("tcgen05.fence::before_thread_sync;");
        named_sync(bar, kThreads);
        if (abort_s[pipe]) {
            ok = false;
            break;
        }
    }
    if (!ok && issuer) atomicExch(p.status, 1);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) tmem_free(taddr_s, kInferCols * kInferPipes);
}

__global__ void adam_kernel(float *p, float *gr, float *m, float *v, __half2 *ph, uint32_t npairs,
                            float lr, float b1, float b2, float eps, float c1, float c2, bool lazy,
                            uint4 *w_img, const float *sched) {
    if (sched) {
        lr = sched[0];
        c1 = sched[1];
        c2 = sched[2];
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npairs; i += gridDim.x * blockDim.x) {
        const float2 gg = reinterpret_cast<float2 *>(gr)[i];
        if (lazy && gg.x == 0.0f && gg.y == 0.0f) continue;
        float2 pp = reinterpret_cast<float2 *>(p)[i];
        float2 mm = reinterpret_cast<float2 *>(m)[i];
        float2 vv = reinterpret_cast<float2 *>(v)[i];
        mm.x = b1 * mm.x + (1.0f - b1) * gg.x;
        mm.y = b1 * mm.y + (1.0f - b1) * gg.y;
        vv.x = b2 * vv.x + (1.0f - b2) * gg.x * gg.x;
        vv.y = b2 * vv.y + (1.0f - b2) * gg.y * gg.y;
        pp.x -= lr * (mm.x * c1) / (sqrtf(vv.x * c2) + eps);
        pp.y -= lr * (mm.y * c1) / (sqrtf(vv.y * c2) + eps);
        reinterpret_cast<float2 *>(p)[i] = pp;
        reinterpret_cast<float2 *>(m)[i] = mm;
        reinterpret_cast<float2 *>(v)[i] = vv;
        reinterpret_cast<float2 *>(gr)[i] = make_float2(0.0f, 0.0f);
        if (ph) ph[i] = __floats2half2_rn(pp.x, pp.y);
        if (w_img) {
            unsigned char *img = reinterpret_cast<unsigned char *>(w_img);
            *reinterpret_cast<__nv_bfloat16 *>(img + weight_image_offset(2 * i)) = __float2bfloat16(pp.x);
            *reinterpret_cast<__nv_bfloat16 *>(img + weight_image_offset(2 * i + 1)) = __float2bfloat16(pp.y);
        }
    }
}

// The table gradient of n samples from their feature gradients (p.dx): a
// block of kCacheMaxLevels warps takes 32 consecutive samples, warp l their
// level l (the training order keeps each batch in (map, Morton) order, so
// the 32 samples are spatial neighbours). Each term w * dL/dfeature is
// rounded to fixed point and added with an integer atomic. On the coarse
// levels (resolution <= kScatterGroupRes) neighbouring samples share
// corners: lanes whose corner is the same table entry (match_any) add their
// terms in shared memory first and the lowest of them issues the atomics --
// the same integer sums, fewer atomics on the most contended entries. Does
// nothing once a tensor-core wait of the training kernel has given up (its
// rows are then incomplete).
constexpr int kScatterGroupRes = 111;
__global__ void __launch_bounds__(kCacheMaxLevels * 32) table_scatter_kernel(CacheGrid g, CacheParams p,
                                                                          const float4 *qa,
                                                                          const uint32_t *sel, uint32_t n) {
    __shared__ longlong2 red[kCacheMaxLevels][32];
    if (*(volatile int *)p.status) return;
    const int lane = threadIdx.x & 31, l = threadIdx.x >> 5;
    if (l >= g.levels) return;
    const uint32_t i = blockIdx.x * 32u + (uint32_t)lane;
    const bool valid = i < n;
    const float2 gr = valid ? reinterpret_cast<const float2 *>(p.dx)[(size_t)i * kCacheMaxLevels + l]
                            : make_float2(0.0f, 0.0f);
    if (!__any_sync(0xffffffffu, gr.x != 0.0f || gr.y != 0.0f)) return;
    QueryPos q{0.0f, 0.0f, 0.0f};
    if (valid) q = unit_pos(g, qa[sel ? sel[i] : i]);
    uint32_t idx[8];
    float w[8];
    level_corners(g, l, q.px, q.py, q.pz, idx, w);
    unsigned long long *lv = reinterpret_cast<unsigned long long *>(p.table_grad) + 2 * ((size_t)l << g.log2_t);
    const bool group = g.res[l] <= kScatterGroupRes;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        long long s0 = to_grad_fixed(w[k] * gr.x), s1 = to_grad_fixed(w[k] * gr.y);
        bool lead = true;
        if (group) {
            const unsigned peers = __match_any_sync(0xffffffffu, idx[k]);
            lead = lane == __ffs(peers) - 1;
            if (peers != (1u << lane)) {
                red[l][lane] = make_longlong2(s0, s1);
                __syncwarp(peers);
                if (lead)
                    for (unsigned m = peers & (peers - 1u); m; m &= m - 1u) {
                        const longlong2 o = red[l][__ffs(m) - 1];
                        s0 += o.x;
                        s1 += o.y;
                    }
                __syncwarp(peers);
            }
        }
        if (lead) {
            if (s0) atomicAdd(lv + 2 * idx[k], (unsigned long long)s0);
            if (s1) atomicAdd(lv + 2 * idx[k] + 1, (unsigned long long)s1);
        }
    }
}

// The table's lazy Adam step from the fixed-point gradient: entries whose
// two sums are zero keep their value and moments; the others are updated
// and their sums cleared.
__global__ void adam_table_kernel(float *p, longlong2 *gr, float *m, float *v, __half2 *ph,
                                  uint32_t npairs, float lr, float b1, float b2, float eps, float c1,
                                  float c2, const float *sched) {
    if (sched) {
        lr = sched[0];
        c1 = sched[1];
        c2 = sched[2];
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npairs; i += gridDim.x * blockDim.x) {
        const longlong2 q = gr[i];
        if (q.x == 0 && q.y == 0) continue;
        const float2 gg = make_float2(from_grad_fixed(q.x), from_grad_fixed(q.y));
        float2 pp = reinterpret_cast<float2 *>(p)[i];
        float2 mm = reinterpret_cast<float2 *>(m)[i];
        float2 vv = reinterpret_cast<float2 *>(v)[i];
        mm.x = b1 * mm.x + (1.0f - b1) * gg.x;
        mm.y = b1 * mm.y + (1.0f - b1) * gg.y;
        vv.x = b2 * vv.x + (1.0f - b2) * gg.x * gg.x;
        vv.y = b2 * vv.y + (1.0f - b2) * gg.y * gg.y;
        pp.x -= lr * (mm.x * c1) / (sqrtf(vv.x * c2) + eps);
        pp.y -= lr * (mm.y * c1) / (sqrtf(vv.y * c2) + eps);
        reinterpret_cast<float2 *>(p)[i] = pp;
        reinterpret_cast<float2 *>(m)[i] = mm;
        reinterpret_cast<float2 *>(v)[i] = vv;
        gr[i] = make_longlong2(0, 0);
        ph[i] = __floats2half2_rn(pp.x, pp.y);
    }
}

// The fixed-point table gradient as floats (debug copies).
__global__ void table_grad_float_kernel(const long long *gr, float *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = from_grad_fixed(gr[i]);
}

// w_grad[i] += sum over the CTAs' partial rows, and *loss += the CTAs'
// losses, both in CTA order (deterministic).
__global__ void wgrad_reduce_kernel(const float *part, const float *loss_part, int parts,
                                    float *w_grad, float *loss) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        float l = 0.0f;
        for (int b = 0; b < parts; ++b) l += loss_part[b];
        *loss += l;
    }
    if (i >= kCacheWeights) return;
    float acc = 0.0f;
    for (int b = 0; b < parts; ++b) acc += part[(size_t)b * kCacheWeights + i];
    w_grad[i] += acc;
}

__global__ void weight_image_kernel(const float *w, uint4 *w_img) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kCacheWeights) return;
    *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<unsigned char *>(w_img) + weight_image_offset(i)) =
        __float2bfloat16(w[i]);
}

__global__ void init_kernel(float *p, float *gr, float *m, float *v, __half2 *ph, uint32_t npairs,
                            uint64_t seed, uint32_t salt, int hidden_pairs, float a_hidden,
                            float a_out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npairs; i += gridDim.x * blockDim.x) {
        const pm_u32x4 r = philox(seed, i, salt, 0x1A17u, 0u);
        const float a = (hidden_pairs < 0 || (int)i < hidden_pairs) ? a_hidden : a_out;
        const float x0 = (2.0f * pm_u01(r.v[0]) - 1.0f) * a;
        const float x1 = (2.0f * pm_u01(r.v[1]) - 1.0f) * a;
        reinterpret_cast<float2 *>(p)[i] = make_float2(x0, x1);
        if (gr) reinterpret_cast<float2 *>(gr)[i] = make_float2(0.0f, 0.0f);
        reinterpret_cast<float2 *>(m)[i] = make_float2(0.0f, 0.0f);
        reinterpret_cast<float2 *>(v)[i] = make_float2(0.0f, 0.0f);
        if (ph) ph[i] = __floats2half2_rn(x0, x1);
    }
}

__global__ void half_copy_kernel(const float *p, __half2 *ph, uint32_t npairs) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npairs; i += gridDim.x * blockDim.x) {
        const float2 v = reinterpret_cast<const float2 *>(p)[i];
        ph[i] = __floats2half2_rn(v.x, v.y);
    }
}

struct CountSink {
    static constexpr bool kCountOnly = true;
    uint32_t n = 0, ns = 0;
    __device__ void volume_steps(int steps) { n += (uint32_t)steps; }
    __device__ void volume(v3, v3, float) { ++n; }
    __device__ void surface(v3, int, v3, float) { ++n; ++ns; }
};

// The query list keeps each block of 32 consecutive pixels (one warp of
// the kernels below; the block's queries one contiguous range from
// off[first pixel]) in sample-major order: the first query of every pixel
// of the block, then the second ones, ..., pixels in order within a step.
// The lanes' stores and loads of one step then land side by side, and the
// order is also the one inference wants (neighbouring rays at similar
// depths). Query s of lane p sits at
//   base + sum_q min(c_q, s) + #{q < p : c_q > s}
// for the block's per-pixel counts c_q. The writer tracks it per lane with
// the block's counts sorted ascending in shared memory: `base` the first
// slot of step s, `live` the lanes with more than s queries.
constexpr int kListWarps = 4;  // warps (pixel blocks) per CTA of the list kernels
static_assert(kListWarps * 32 == (int)kListBlock, "one CTA of the list kernels covers kListBlock pixels");
struct WriteSink {
    static constexpr bool kCountOnly = false;
    __device__ void volume_steps(int) {}
    float4 *qa, *qd;
    uint32_t *slist;
    uint32_t sat;
    uint32_t cap;      // slots of the list: records past it are dropped
    const uint2 *srt;  // (count, lane) of the block's pixels, ascending
    uint32_t base, live, lt, s, j;
    __device__ uint32_t next() {
        const uint32_t at = base + (uint32_t)__popc(live & lt);
        base += (uint32_t)__popc(live);
        ++s;
        while (j < 32u && srt[j].x <= s) live &= ~(1u << srt[j++].y);
        return at;
    }
    __device__ void volume(v3 x, v3 wo, float w) {
        const uint32_t at = next();
        if (at >= cap) return;
        qa[at] = make_float4(x.x, x.y, x.z, __int_as_float(kNone));
        qd[at] = make_float4(wo.x, wo.y, wo.z, w);
    }
    __device__ void surface(v3 x, int obj, v3 wo, float w) {
        const uint32_t at = next();
        if (at >= cap) return;
        slist[sat++] = at;
        qa[at] = make_float4(x.x, x.y, x.z, __int_as_float(obj));
        qd[at] = make_float4(wo.x, wo.y, wo.z, w);
    }
};

// Calls f(i) for the list index i of each query of this lane's pixel, in
// the pixel's own order (s = 0, 1, ...). Warp-synchronous: every lane of
// the warp calls it, lanes past npix with no queries; the warp's first
// pixel must be below npix.
template <typename F>
__device__ __forceinline__ void for_pixel_queries(const uint32_t *off, uint32_t pix, uint32_t npix, F &&f) {
    const int lane = threadIdx.x & 31;
    const bool valid = pix < npix;
    const uint32_t o = valid ? off[pix] : 0u, c = valid ? off[pix + 1] - o : 0u;
    uint32_t base = __shfl_sync(0xffffffffu, o, 0);
    const uint32_t cmax = __reduce_max_sync(0xffffffffu, c);
    const unsigned lt = (1u << lane) - 1u;
    for (uint32_t s = 0; s < cmax; ++s) {
        const unsigned m = __ballot_sync(0xffffffffu, s < c);
        if (s < c) f(base + (uint32_t)__popc(m & lt));
        base += (uint32_t)__popc(m);
    }
}

__global__ void count_kernel(PScene Sc, RenderParams R, bool vol_on, bool surf_on, uint32_t *cnt,
                             uint32_t *scnt) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= (uint32_t)R.width * (uint32_t)R.height) return;
    CountSink c;
    walk_eye(Sc, R, pix, vol_on, surf_on, c);
    cnt[pix] = c.n;
    scnt[pix] = c.ns;
}

// The records of the warp's block of 32 pixels (pix this lane's; the
// block's first pixel below npix), srt the warp's 32 entries of shared
// memory.
__device__ __forceinline__ void write_block(const PScene &Sc, const RenderParams &R, bool vol_on, bool surf_on,
                                            const uint32_t *off, const uint32_t *soff, float4 *qa, float4 *qd,
                                            uint32_t *slist, uint32_t cap, uint32_t pix, uint32_t npix,
                                            uint2 *srt) {
    const int lane = threadIdx.x & 31;
    const bool valid = pix < npix;
    const uint32_t c = valid ? off[pix + 1] - off[pix] : 0u;
    // the block's counts sorted ascending (ties by lane)
    uint32_t rank = 0;
    for (int q = 0; q < 32; ++q) {
        const uint32_t cq = __shfl_sync(0xffffffffu, c, q);
        rank += (cq < c || (cq == c && q < lane)) ? 1u : 0u;
    }
    srt[rank] = make_uint2(c, (uint32_t)lane);
    __syncwarp();
    WriteSink ws;
    ws.qa = qa;
    ws.qd = qd;
    ws.slist = slist;
    ws.sat = valid ? soff[pix] : 0u;
    ws.cap = cap;
    ws.srt = srt;
    ws.base = __shfl_sync(0xffffffffu, valid ? off[pix] : 0u, 0);
    ws.live = __ballot_sync(0xffffffffu, c > 0u);
    ws.lt = (1u << lane) - 1u;
    ws.s = 0;
    ws.j = (uint32_t)__popc(__ballot_sync(0xffffffffu, c == 0u));
    if (valid) walk_eye(Sc, R, pix, vol_on, surf_on, ws);
}

__global__ void __launch_bounds__(kListWarps * 32)
    write_kernel(PScene Sc, RenderParams R, bool vol_on, bool surf_on, const uint32_t *off,
                 const uint32_t *soff, float4 *qa, float4 *qd, uint32_t *slist) {
    __shared__ uint2 srt[kListWarps][32];
    const uint32_t npix = (uint32_t)R.width * (uint32_t)R.height;
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix - (threadIdx.x & 31u) >= npix) return;  // the whole block of 32 pixels
    write_block(Sc, R, vol_on, surf_on, off, soff, qa, qd, slist, 0xffffffffu, pix, npix, srt[threadIdx.x >> 5]);
}

__global__ void __launch_bounds__(kListWarps * 32)
    composite_kernel(PScene Sc, const uint32_t *off, const float4 *qa, const float4 *qd,
                     const float4 *val, uint32_t npix, float exposure, float4 *rad, uchar4 *rgba) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix - (threadIdx.x & 31u) >= npix) return;
    v3 L = mk3(0.f, 0.f, 0.f);
    for_pixel_queries(off, pix, npix, [&](uint32_t i) {
        const int obj = __float_as_int(qa[i].w);
        const float w = qd[i].w;
        const float4 v = val[i];
        if (obj != kNone) {
            const v3 al = material_albedo(Sc, obj);
            L = L + mk3(al.x * (v.x * w), al.y * (v.y * w), al.z * (v.z * w));
        } else {
            L = L + mk3(v.x * w, v.y * w, v.z * w);
        }
    });
    if (pix >= npix) return;
    if (rad) rad[pix] = make_float4(L.x, L.y, L.z, 1.0f);
    if (rgba)
        rgba[pix] = make_uchar4(to_u8_sat((double)(L.x * exposure) * 255.0),
                                to_u8_sat((double)(L.y * exposure) * 255.0),
                                to_u8_sat((double)(L.z * exposure) * 255.0), 255);
}

// Same per-pixel loop, from raw values, with the render kernel's
// operations and order: volume scale = (T * dt) * (1 / (4/3 pi r^3)),
// L += e * scale; diffuse scale = (T * (1 / (pi r^2))) * (1 / pi),
// L += albedo * (e * scale).
__device__ __forceinline__ void composite_exact_pixel(const PScene &Sc, const uint32_t *off, const float4 *qa,
                                                      const float4 *qd, const float4 *raw, uint32_t pix,
                                                      uint32_t npix, float exposure, float4 *rad, uchar4 *rgba) {
    v3 L = mk3(0.f, 0.f, 0.f);
    for_pixel_queries(off, pix, npix, [&](uint32_t i) {
        const float4 v = raw[i];
        if (!(v.w >= 0.0f)) return;
        const float r2 = v.w;
        const v3 e = mk3(v.x, v.y, v.z);
        const float w = qd[i].w;
        const int obj = __float_as_int(qa[i].w);
        if (obj == kNone) {
            const float scale = w * (1.0f / (4.18879020f * r2 * sqrtf(r2)));
            L = L + e * scale;
        } else {
            const v3 a = material_albedo(Sc, obj);
            const float scale = w * (1.0f / (3.14159265f * r2)) * 0.318309886f;
            L = L + mk3(a.x * (e.x * scale), a.y * (e.y * scale), a.z * (e.z * scale));
        }
    });
    if (pix >= npix) return;
    if (rad) rad[pix] = make_float4(L.x, L.y, L.z, 1.0f);
    if (rgba)
        rgba[pix] = make_uchar4(to_u8_sat((double)(L.x * exposure) * 255.0),
                                to_u8_sat((double)(L.y * exposure) * 255.0),
                                to_u8_sat((double)(L.z * exposure) * 255.0), 255);
}

__global__ void __launch_bounds__(kListWarps * 32)
    composite_exact_kernel(PScene Sc, const uint32_t *off, const float4 *qa, const float4 *qd,
                           const float4 *raw, uint32_t npix, float exposure, float4 *rad, uchar4 *rgba) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix - (threadIdx.x & 31u) >= npix) return;
    composite_exact_pixel(Sc, off, qa, qd, raw, pix, npix, exposure, rad, rgba);
}

// The block's scene of a batched list launch staged in shared memory (the
// last j with blk[j] <= blockIdx.x: scenes without pixels have no blocks);
// returns the block's index within its scene.
__device__ uint32_t stage_list_scene(const ListScene *ls, const int *ids, const uint32_t *blk, int n,
                                     ListScene &cur) {
    __shared__ int sj;
    if (threadIdx.x == 0) {
        int lo = 0, hi = n;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (blk[mid] <= blockIdx.x) lo = mid; else hi = mid;
        }
        sj = lo;
    }
    __syncthreads();
    const int j = sj;
    const uint32_t *src = reinterpret_cast<const uint32_t *>(&ls[ids[j]]);
    uint32_t *dst = reinterpret_cast<uint32_t *>(&cur);
    for (int i = threadIdx.x; i < (int)(sizeof(ListScene) / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    return blockIdx.x - blk[j];
}

__global__ void __launch_bounds__(kListWarps * 32)
    list_count_multi_kernel(const ListScene *ls, const int *ids, const uint32_t *blk, int n) {
    __shared__ ListScene cur;
    const uint32_t pix = stage_list_scene(ls, ids, blk, n, cur) * blockDim.x + threadIdx.x;
    if (pix >= cur.npix) return;
    CountSink c;
    walk_eye(cur.sc, cur.R, pix, cur.vol_on != 0, cur.surf_on != 0, c);
    cur.cnt[pix] = c.n;
    cur.scnt[pix] = c.ns;
}

__global__ void __launch_bounds__(kListWarps * 32)
    list_write_multi_kernel(const ListScene *ls, const int *ids, const uint32_t *blk, int n) {
    __shared__ ListScene cur;
    __shared__ uint2 srt[kListWarps][32];
    const uint32_t pix = stage_list_scene(ls, ids, blk, n, cur) * blockDim.x + threadIdx.x;
    if (pix - (threadIdx.x & 31u) >= cur.npix) return;
    write_block(cur.sc, cur.R, cur.vol_on != 0, cur.surf_on != 0, cur.off, cur.soff, cur.qa, cur.qd, cur.slist,
                cur.nq, pix, cur.npix, srt[threadIdx.x >> 5]);
}

__global__ void __launch_bounds__(kListWarps * 32)
    list_composite_multi_kernel(const ListScene *ls, const int *ids, const uint32_t *blk, int n) {
    __shared__ ListScene cur;
    const uint32_t pix = stage_list_scene(ls, ids, blk, n, cur) * blockDim.x + threadIdx.x;
    if (pix - (threadIdx.x & 31u) >= cur.npix) return;
    composite_exact_pixel(cur.sc, cur.off, cur.qa, cur.qd, cur.raw, pix, cur.npix, cur.exposure, cur.rad,
                          cur.rgba);
}

__global__ void select_kernel(uint64_t seed, uint32_t frame, const unsigned long long *frame_dev, uint32_t total,
                              const uint32_t *slist, uint32_t ns_total, uint32_t n, float surf_frac,
                              uint32_t *sel) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (frame_dev) frame = (uint32_t)*frame_dev;
    const pm_u32x4 r = philox(seed, i, frame, 0x5E1Eu, 0u);
    if (ns_total > 0 && pm_u01(r.v[1]) < surf_frac)
        sel[i] = slist[(uint32_t)(((uint64_t)r.v[0] * ns_total) >> 32)];
    else
        sel[i] = (uint32_t)(((uint64_t)r.v[0] * total) >> 32);
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ uint32_t query_key(const CacheGrid &g, float4 a) {
    const QueryPos q = unit_pos(g, a);
    const uint32_t x = min((uint32_t)(q.px * 1024.0f), 1023u);
    const uint32_t y = min((uint32_t)(q.py * 1024.0f), 1023u);
    const uint32_t z = min((uint32_t)(q.pz * 1024.0f), 1023u);
    const uint32_t vol = __float_as_int(a.w) == kNone ? 1u : 0u;
    return (vol << 30) | (spread10(x) << 2) | (spread10(y) << 1) | spread10(z);
}

__global__ void sample_keys_kernel(CacheGrid g, const float4 *qa, const uint32_t *sel, uint32_t n,
                                   uint32_t *keys, uint32_t *vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = query_key(g, qa[sel ? sel[i] : i]);
    vals[i] = i;
}

__global__ void list_keys_kernel(const ListScene *ls, const int *tile_scene, size_t first, uint32_t n,
                                 uint32_t *keys, uint32_t *vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t g = first + i;
    const int sc = tile_scene[g / kSortTile];
    uint32_t key = 0xffffffffu, val = 0xffffffffu;
    if (sc >= 0) {
        const ListScene &d = ls[sc];
        const size_t loc = g - d.q_first;
        if (d.on && loc < d.nq) {
            key = query_key(d.box, d.qa[loc]);
            val = (uint32_t)loc;
        }
    }
    keys[i] = key;
    vals[i] = val;
}

// The sorted picks' records: pick pos[i] copied to pqa[i], pqd[i]; pord[i] = i.
__global__ void pick_records_kernel(const uint32_t *pos, const uint32_t *sel, const float4 *qa,
                                    const float4 *qd, uint32_t n, float4 *pqa, float4 *pqd, uint32_t *pord) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t q = sel[pos[i]];
    pqa[i] = qa[q];
    pqd[i] = qd[q];
    pord[i] = i;
}

// Sorted pick j -> slot j / nb of batch j % nb (batch b starting at
// b * (n / nb) + min(b, n % nb)): every batch takes every nb-th pick of the
// (map, Morton) order.
__global__ void train_order_kernel(const float4 *pqa, const float4 *pqd, const float4 *pval,
                                   const uint32_t *pos, const uint32_t *sel, uint32_t n, uint32_t nb,
                                   float4 *tqa, float4 *tqd, float4 *tgt, uint32_t *tsel) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t b = j % nb;
    const uint32_t t = b * (n / nb) + min(b, n % nb) + j / nb;
    tqa[t] = pqa[j];
    tqd[t] = pqd[j];
    tgt[t] = pval[j];
    tsel[t] = sel[pos[j]];
}

__global__ void iota_kernel(uint32_t *v, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

// One CTA of kSumThreads: thread t sums entries t, t + kSumThreads, ... in
// index order, then a fixed reduction tree; the result does not depend on
// scheduling.
constexpr int kSumThreads = 1024;
__global__ void __launch_bounds__(kSumThreads) value_sum_kernel(const float4 *val, uint32_t n, float *sum,
                                                               const float *skip_if_set) {
    __shared__ float red[kSumThreads];
    if (skip_if_set && *skip_if_set > 0.0f) return;
    float acc = 0.0f;
    for (uint32_t i = threadIdx.x; i < n; i += kSumThreads) {
        const float4 v = val[i];
        acc += (v.x + v.y + v.z) * (1.0f / 3.0f);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int h = kSumThreads / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) *sum = red[0];
}

__global__ void count_up_kernel(unsigned long long *c) { ++*c; }

__global__ void scale_init_kernel(const float *sum, uint32_t n, float *scale) {
    if (*scale > 0.0f) return;
    const float mean = *sum / (float)n;
    *scale = mean > 0.0f && isfinite(mean) ? mean : 1.0f;
}

__global__ void schedule_kernel(float *sched, unsigned long long *step, float lr0, float lr_min, float half_life,
                                float b1, float b2) {
    const unsigned long long s0 = *step;
    float lr = lr0;
    if (half_life > 0.0f) lr = lr_min + (lr0 - lr_min) * (float)exp2(-(double)s0 / (double)half_life);
    const unsigned long long s1 = s0 + 1;
    const float sf = (float)(s1 < (1ull << 30) ? s1 : (1ull << 30));
    sched[0] = lr;
    sched[1] = 1.0f / (1.0f - powf(b1, sf));
    sched[2] = 1.0f / (1.0f - powf(b2, sf));
    *step = s1;
}

}  // namespace

cudaError_t cache_count_queries(const PScene &S, const RenderParams &R, bool vol_on, bool surf_on,
                                uint32_t *cnt, uint32_t *scnt, cudaStream_t s) {
    const uint32_t npix = (uint32_t)R.width * (uint32_t)R.height;
    if (npix == 0) return cudaSuccess;
    count_kernel<<<(npix + kListWarps * 32 - 1) / (kListWarps * 32), kListWarps * 32, 0, s>>>(S, R, vol_on, surf_on, cnt, scnt);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_write_queries(const PScene &S, const RenderParams &R, bool vol_on, bool surf_on,
                                const uint32_t *off, const uint32_t *soff, float4 *qa, float4 *qd,
                                uint32_t *slist, cudaStream_t s) {
    const uint32_t npix = (uint32_t)R.width * (uint32_t)R.height;
    if (npix == 0) return cudaSuccess;
    write_kernel<<<(npix + kListWarps * 32 - 1) / (kListWarps * 32), kListWarps * 32, 0, s>>>(S, R, vol_on, surf_on, off, soff, qa, qd, slist);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_composite(const PScene &S, const uint32_t *off, const float4 *qa,
                            const float4 *qd, const float4 *val, uint32_t npix, float exposure,
                            float4 *rad, uchar4 *rgba, cudaStream_t s) {
    if (npix == 0) return cudaSuccess;
    composite_kernel<<<(npix + kListWarps * 32 - 1) / (kListWarps * 32), kListWarps * 32, 0, s>>>(S, off, qa, qd, val, npix, exposure, rad, rgba);
    note_launch();
    return cudaGetLastError();
}

cudaError_t render_composite(const PScene &S, const uint32_t *off, const float4 *qa,
                             const float4 *qd, const float4 *raw, uint32_t npix, float exposure,
                             float4 *rad, uchar4 *rgba, cudaStream_t s) {
    if (npix == 0) return cudaSuccess;
    composite_exact_kernel<<<(npix + kListWarps * 32 - 1) / (kListWarps * 32), kListWarps * 32, 0, s>>>(S, off, qa, qd, raw, npix, exposure, rad,
                                                              rgba);
    note_launch();
    return cudaGetLastError();
}

cudaError_t list_count_multi(const ListScene *ls, const int *ids, const uint32_t *blk, int n, uint32_t blocks,
                             cudaStream_t s) {
    if (n <= 0 || blocks == 0) return cudaSuccess;
    list_count_multi_kernel<<<blocks, kListWarps * 32, 0, s>>>(ls, ids, blk, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t list_write_multi(const ListScene *ls, const int *ids, const uint32_t *blk, int n, uint32_t blocks,
                             cudaStream_t s) {
    if (n <= 0 || blocks == 0) return cudaSuccess;
    list_write_multi_kernel<<<blocks, kListWarps * 32, 0, s>>>(ls, ids, blk, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t list_composite_multi(const ListScene *ls, const int *ids, const uint32_t *blk, int n,
                                 uint32_t blocks, cudaStream_t s) {
    if (n <= 0 || blocks == 0) return cudaSuccess;
    list_composite_multi_kernel<<<blocks, kListWarps * 32, 0, s>>>(ls, ids, blk, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t list_keys_multi(const ListScene *ls, const int *tile_scene, size_t first, uint32_t n, uint32_t *keys,
                            uint32_t *vals, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    list_keys_kernel<<<(n + 255) / 256, 256, 0, s>>>(ls, tile_scene, first, n, keys, vals);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_pick_records(const uint32_t *pos, const uint32_t *sel, const float4 *qa, const float4 *qd,
                               uint32_t n, float4 *pqa, float4 *pqd, uint32_t *pord, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    pick_records_kernel<<<(n + 255) / 256, 256, 0, s>>>(pos, sel, qa, qd, n, pqa, pqd, pord);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_train_order(const float4 *pqa, const float4 *pqd, const float4 *pval,
                              const uint32_t *pos, const uint32_t *sel, uint32_t n, uint32_t nb,
                              float4 *tqa, float4 *tqd, float4 *tgt, uint32_t *tsel, cudaStream_t s) {
    if (n == 0 || nb == 0) return cudaSuccess;
    train_order_kernel<<<(n + 255) / 256, 256, 0, s>>>(pqa, pqd, pval, pos, sel, n, nb, tqa, tqd, tgt, tsel);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_select(uint64_t seed, uint32_t frame, uint32_t total, const uint32_t *slist,
                         uint32_t ns_total, uint32_t n, float surf_frac, uint32_t *sel,
                         cudaStream_t s, const unsigned long long *frame_dev) {
    if (n == 0) return cudaSuccess;
    select_kernel<<<(n + 255) / 256, 256, 0, s>>>(seed, frame, frame_dev, total, slist, ns_total, n, surf_frac,
                                                  sel);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_sample_keys(const CacheGrid &g, const float4 *qa, const uint32_t *sel, uint32_t n,
                              uint32_t *keys, uint32_t *vals, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    sample_keys_kernel<<<(n + 255) / 256, 256, 0, s>>>(g, qa, sel, n, keys, vals);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_iota(uint32_t *v, uint32_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    iota_kernel<<<(n + 255) / 256, 256, 0, s>>>(v, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_value_sum(const float4 *val, uint32_t n, float *sum, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    value_sum_kernel<<<1, kSumThreads, 0, s>>>(val, n, sum, nullptr);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_scale_init(const float4 *val, uint32_t n, float *sum, float *scale, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    value_sum_kernel<<<1, kSumThreads, 0, s>>>(val, n, sum, scale);
    note_launch();
    scale_init_kernel<<<1, 1, 0, s>>>(sum, n, scale);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_count_up(unsigned long long *c, cudaStream_t s) {
    count_up_kernel<<<1, 1, 0, s>>>(c);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_schedule(float *sched, unsigned long long *step, float lr0, float lr_min, float half_life,
                           float beta1, float beta2, cudaStream_t s) {
    schedule_kernel<<<1, 1, 0, s>>>(sched, step, lr0, lr_min, half_life, beta1, beta2);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_init(const CacheGrid &g, const CacheParams &p, uint64_t seed, cudaStream_t s) {
    const uint32_t tpairs = (uint32_t)(((size_t)g.levels << g.log2_t));  // 2 floats per entry
    init_kernel<<<1024, 256, 0, s>>>(p.table, nullptr, p.table_m, p.table_v, p.table_h, tpairs, seed,
                                     0x7AB1Eu, -1, 1e-4f, 1e-4f);
    note_launch();
    cudaError_t e = cudaMemsetAsync(p.table_grad, 0, sizeof(longlong2) * tpairs, s);
    if (e != cudaSuccess) return e;
    const float a = sqrtf(6.0f / 64.0f);
    init_kernel<<<(kCacheWeights / 2 + 255) / 256, 256, 0, s>>>(p.w, p.w_grad, p.w_m, p.w_v, nullptr,
                                                                kCacheWeights / 2, seed, 0x3E16u,
                                                                4 * 4096 / 2, a, a);
    note_launch();
    return cache_weight_image(p, s);
}

cudaError_t cache_sync_half(const CacheGrid &g, const CacheParams &p, cudaStream_t s) {
    const uint32_t tpairs = (uint32_t)(((size_t)g.levels << g.log2_t));
    half_copy_kernel<<<1024, 256, 0, s>>>(p.table, p.table_h, tpairs);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_backward(const CacheGrid &g, const CacheParams &p, const PScene &S,
                           const float4 *qa, const float4 *qd, const uint32_t *sel,
                           const float4 *val, uint32_t n, float inv_scale, float loss_norm,
                           float rel_eps, float *x_out, float *y_out, int sm_count, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (n > p.dx_cap) return cudaErrorInvalidValue;
    // the opt-in is per device: set it on every call (a host-side attribute write)
    cudaError_t e = cudaFuncSetAttribute(train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kTrainSmem);
    if (e != cudaSuccess) return e;
    const uint32_t ntiles = (n + kThreads - 1) / kThreads;
    const uint32_t rows = ntiles * kThreads;
    const uint32_t egrid = std::min<uint32_t>((rows + 255) / 256, (uint32_t)sm_count * 16);
    encode_kernel<<<egrid, 256, 0, s>>>(g, p.table_h, S, qa, qd, sel, n, rows,
                                        reinterpret_cast<unsigned char *>(p.xt), x_out);
    note_launch();
    const uint32_t grid = std::min<uint32_t>(
        ntiles, (uint32_t)std::min(sm_count, p.parts_cap));
    train_kernel<<<grid, kThreads, kTrainSmem, s>>>(p, reinterpret_cast<const unsigned char *>(p.xt), val,
                                                    n, inv_scale, loss_norm, rel_eps, y_out);
    note_launch();
    wgrad_reduce_kernel<<<(kCacheWeights + 255) / 256, 256, 0, s>>>(p.w_part, p.loss_part, (int)grid,
                                                                  p.w_grad, p.loss);
    note_launch();
    table_scatter_kernel<<<(n + 31) / 32, kCacheMaxLevels * 32, 0, s>>>(g, p, qa, sel, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_adam(const CacheGrid &g, const CacheParams &p, float lr, float beta1,
                       float beta2, float eps, int step, cudaStream_t s) {
    const float c1 = 1.0f / (1.0f - powf(beta1, (float)step));
    const float c2 = 1.0f / (1.0f - powf(beta2, (float)step));
    const uint32_t tpairs = (uint32_t)(((size_t)g.levels << g.log2_t));
    adam_table_kernel<<<2048, 256, 0, s>>>(p.table, reinterpret_cast<longlong2 *>(p.table_grad),
                                           p.table_m, p.table_v, p.table_h, tpairs, lr, beta1, beta2, eps,
                                           c1, c2, p.sched);
    note_launch();
    adam_kernel<<<(kCacheWeights / 2 + 255) / 256, 256, 0, s>>>(p.w, p.w_grad, p.w_m, p.w_v, nullptr,
                                                                kCacheWeights / 2, lr, beta1, beta2,
                                                                eps, c1, c2, false, p.w_img, p.sched);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_table_grad_float(const CacheGrid &g, const CacheParams &p, float *out,
                                   cudaStream_t s) {
    const size_t n = (size_t)g.levels << (g.log2_t + 1);
    table_grad_float_kernel<<<1024, 256, 0, s>>>(p.table_grad, out, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_weight_image(const CacheParams &p, cudaStream_t s) {
    weight_image_kernel<<<(kCacheWeights + 255) / 256, 256, 0, s>>>(p.w, p.w_img);
    note_launch();
    return cudaGetLastError();
}

cudaError_t cache_infer(const CacheGrid &g, const CacheParams &p, const PScene &S,
                        const float4 *qa, const float4 *qd, const uint32_t *order, uint32_t n,
                        float out_scale, float4 *val, int sm_count, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const bool lowered = p.wait_polls != kMbarSpin;
    cudaError_t ea = cudaFuncSetAttribute(lowered ? infer_kernel<true> : infer_kernel<false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem);
    if (ea != cudaSuccess) return ea;
    const uint32_t ntiles = (n + kThreads - 1) / kThreads;
    // one CTA (four pipelines, 16 warps) per SM: two CTAs per SM fit when the
    // kernel compiles to 64 registers or fewer, but run slower (the table
    // reads of twice the pipelines compete for the same L1)
    const uint32_t ctas = (ntiles + kInferPipes - 1) / kInferPipes;
    const uint32_t grid = std::min<uint32_t>(ctas, (uint32_t)sm_count);
    if (lowered)
        infer_kernel<true><<<grid, kThreads * kInferPipes, kInferSmem, s>>>(g, p, S, qa, qd, order, n,
                                                                             out_scale, val);
    else
        infer_kernel<false><<<grid, kThreads * kInferPipes, kInferSmem, s>>>(g, p, S, qa, qd, order, n,
                                                                              out_scale, val);
    note_launch();
    return cudaGetLastError();
}

}  // namespace pm
