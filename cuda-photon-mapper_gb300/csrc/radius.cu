// radius.cu -- the reference's record-list radius gather over a built
// photon map.
//
// The reference's earlier kernels (kernelPBO.cu:165-182,
// "photonMappingKernel - Copy.cu":191-208) estimate irradiance at a point
// with normal N as the sum, over stored photons closer than sqrt(sqRadius),
// of energy * max(0, -N.dir) * (1 - distance) / exposure, the squared
// distance taken with the gated x, y, z accumulation of gatedSqDist3
// (:245-257). Here the photons come from the kd-tree instead of a linear
// scan of a per-object list: one warp per query walks every node whose box
// lies within the radius, each lane tests one record of a leaf, and the
// per-lane Kahan sums meet in a compensated butterfly. The weight keeps the
// reference's double-precision steps (its double literals promote it).
#include "gather.cuh"
#include "launch_count.cuh"

namespace pm {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kStackCap = 192;
constexpr int kWarps = 4;

__device__ __forceinline__ void kahan(float &sum, float &comp, float x) {
    float y = x - comp;
    float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

__device__ __forceinline__ float warp_total(float sum, float comp) {
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

__global__ void __launch_bounds__(kWarps * 32) radius_kernel(MapView m, const float4 *pts,
                                                             const float4 *nrm, uint32_t nq,
                                                             float sq_radius, float exposure,
                                                             float4 *out) {
    __shared__ uint32_t stack[kWarps][kStackCap];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t qi = blockIdx.x * kWarps + wib;
    if (qi >= nq) return;
    const float4 q = pts[qi], nv = nrm[qi];
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    if (m.n > 0) {
        uint32_t *st = stack[wib];
        const uint32_t first_leaf = 1u << m.depth;
        int top = 1;
        if (lane == 0) st[0] = 1u;
        __syncwarp();
        while (top > 0) {
            --top;
            const uint32_t node = st[top];
            __syncwarp();
            const int dn = 31 - __clz(node);
            if (dn == m.depth) {
                for (int ch = 0; ch < (1 << m.leaf_shift); ++ch) {
                    const uint32_t r = ((node - first_leaf) << (5 + m.leaf_shift)) +
                                       ((uint32_t)ch << 5) + lane;
                    if (r >= m.n) continue;
                    const float4 p = __ldg(&m.pos[r]);
                    // gatedSqDist3: x, then y, then z, each partial sum gated
                    float c = q.x - p.x;
                    float d = c * c;
                    bool in = !(d > sq_radius);
                    if (in) { c = q.y - p.y; d += c * c; in = !(d > sq_radius); }
                    if (in) { c = q.z - p.z; d += c * c; in = !(d > sq_radius); }
                    if (in) {
                        const float4 pw = __ldg(&m.pow[r]);
                        const v3 dir = oct_decode(__float_as_uint(pw.w));
                        const float nd = nv.x * dir.x + nv.y * dir.y + nv.z * dir.z;
                        float w = (float)fmax(0.0, (double)(-nd));
                        w = (float)((double)w * ((1.0 - (double)sqrtf(d)) / (double)exposure));
                        kahan(sx, cx, pw.x * w);
                        kahan(sy, cy, pw.y * w);
                        kahan(sz, cz, pw.z * w);
                    }
                }
            } else {
                int w = (m.depth - dn) % 5;
                if (w == 0) w = 5;
                const int nc = 1 << w;
                const uint32_t child = (node << w) + lane;
                bool ok = false;
                if (lane < nc) {
                    const float4 lo = __ldg(&m.lo[child]), hi = __ldg(&m.hi[child]);
                    const float dx = fmaxf(fmaxf(lo.x - q.x, q.x - hi.x), 0.0f);
                    const float dy = fmaxf(fmaxf(lo.y - q.y, q.y - hi.y), 0.0f);
                    const float dz = fmaxf(fmaxf(lo.z - q.z, q.z - hi.z), 0.0f);
                    ok = dx * dx + dy * dy + dz * dz <= sq_radius;
                }
                const unsigned mask = __ballot_sync(kFull, ok);
                const int rank = __popc(mask & ((1u << lane) - 1u));
                if (ok && top + rank < kStackCap) st[top + rank] = child;
                top = min(top + __popc(mask), kStackCap);
            }
            __syncwarp();
        }
    }
    const float ex = warp_total(sx, cx), ey = warp_total(sy, cy), ez = warp_total(sz, cz);
    if (lane == 0) out[qi] = make_float4(ex, ey, ez, 0.0f);
}

}  // namespace

cudaError_t radius_gather(const MapView &m, const float4 *pts, const float4 *nrm, uint32_t nq,
                          float sq_radius, float exposure, float4 *out, cudaStream_t s) {
    if (nq == 0) return cudaSuccess;
    radius_kernel<<<(nq + kWarps - 1) / kWarps, kWarps * 32, 0, s>>>(m, pts, nrm, nq, sq_radius,
                                                                     exposure, out);
    note_launch();
    return cudaGetLastError();
}

}  // namespace pm
