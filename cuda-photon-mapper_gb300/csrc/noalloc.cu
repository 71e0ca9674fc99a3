// noalloc.cu -- k-nearest-neighbour queries over caller-provided points
// without any device allocation.
//
// Some callers of this library cannot call cudaMalloc: code that runs
// inside another framework's memory pool or stream-ordered allocator and
// must not step outside it, plug-ins whose host forbids device allocation
// after start-up, and real-time loops that may not risk an allocation
// stall or failure mid-frame. pm_knn_noalloc serves them: the caller
// passes only inputs and outputs, and the temporary memory the kd-tree
// build needs (sort keys, the tree-ordered copy of the points, node boxes)
// lives in one file-scope device array of fixed size.
//
// That array exists once per device for the life of the process (every GPU
// that loads the library holds it until exit). All calls share it and it
// keeps the last call's contents; each call overwrites everything it
// reads, so nothing has to start at zero. Calls that overlap on the GPU
// (different streams, or different host threads on the same device) race
// on the array and must be serialised by the caller.
#include <cuda.h>

#include <mutex>

#include "gather.cuh"
#include "kdtree.cuh"
#include "launch_count.cuh"
#include "pm.h"
#include "radix_sort.cuh"

namespace pm {
namespace {

constexpr uint32_t kMaxPoints = PM_KNN_NOALLOC_MAX_POINTS;
constexpr int kMaxDevices = 64;

// Byte layout of the scratch array (each part 256-byte aligned).
constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kTiles = (kMaxPoints + kSortTile - 1) / kSortTile;
constexpr size_t kNodes = (size_t)2 << 12;  // tree_nodes(kMaxPoints): depth 12 for 2^17 points
constexpr size_t kOffKeys = 0;
constexpr size_t kOffKeysTmp = kOffKeys + align256(8 * kMaxPoints);
constexpr size_t kOffVals = kOffKeysTmp + align256(8 * kMaxPoints);
constexpr size_t kOffValsTmp = kOffVals + align256(4 * kMaxPoints);
constexpr size_t kOffHist = kOffValsTmp + align256(4 * kMaxPoints);
// digit counts of every tile plus the partial sums of their scan
constexpr size_t kHistWords = 256 * kTiles + (256 * kTiles + kSortTile - 1) / kSortTile + 1;
constexpr size_t kOffIpos = kOffHist + align256(4 * kHistWords);
constexpr size_t kOffTpos = kOffIpos + align256(16 * kMaxPoints);
constexpr size_t kOffLo = kOffTpos + align256(16 * kMaxPoints);
constexpr size_t kOffHi = kOffLo + align256(16 * kNodes);
constexpr size_t kOffMisc = kOffHi + align256(16 * kNodes);  // count + box
constexpr size_t kScratchBytes = kOffMisc + 256;
static_assert(kScratchBytes == PM_KNN_NOALLOC_SCRATCH_BYTES, "scratch size in pm.h is stale");
static_assert(6 * 128 * sizeof(float) <= kOffKeysTmp - kOffKeys, "prepare partials fit the key area");

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// The scratch array's device address per device, valid for the CUDA
// context it was looked up in.
struct ScratchAddr {
    CUcontext ctx;
    unsigned char *addr;
};
std::mutex g_mu;
ScratchAddr g_addr[kMaxDevices] = {};
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
CtxGetCurrentFn g_ctx_get_current = nullptr;

// Device address of g_scratch on the current device. In host code
// `g_scratch` names a host-side stand-in, not device memory, so kernels get
// this address instead. It is looked up (cudaGetSymbolAddress, with the
// device current) on the first call on each device, and again whenever the
// current context differs from the one it was looked up in (after a
// cudaDeviceReset, or under a context the caller made current through the
// driver API): an address from another context is not this one's memory.
cudaError_t scratch_address(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ctx_get_current) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorSymbolNotFound;
        g_ctx_get_current = (CtxGetCurrentFn)fn;
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
    ScratchAddr &slot = g_addr[dev];
    if (!ctx || !slot.addr || slot.ctx != ctx) {
        // also makes the device's primary context current when no context is
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return e;
        if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return cudaErrorDeviceUninitialized;
        slot.addr = (unsigned char *)p;
        slot.ctx = ctx;
    }
    *out = slot.addr;
    return cudaSuccess;
}

constexpr int kPrepBlocks = 128;
constexpr int kPrepThreads = 256;

// Copies the points with their index in .w (the tie-break key), grid-stride
// over kPrepBlocks CTAs, and writes each CTA's bounding box of its points to
// part[6 * block ..] (lo xyz, hi xyz).
__global__ void __launch_bounds__(kPrepThreads) prepare_kernel(const float4 *__restrict__ pts,
                                                               uint32_t n, float4 *ipos, float *part) {
    __shared__ float red[6][kPrepThreads / 32];
    const float inf = __int_as_float(0x7f800000);
    float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
    for (uint32_t i = blockIdx.x * kPrepThreads + threadIdx.x; i < n; i += kPrepBlocks * kPrepThreads) {
        const float4 p = pts[i];
        ipos[i] = make_float4(p.x, p.y, p.z, __uint_as_float(i));
        lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
        hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
    }
    for (int o = 16; o; o >>= 1)
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int a = 0; a < 3; ++a) { red[a][warp] = lo[a]; red[3 + a][warp] = hi[a]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int a = threadIdx.x;
        float v = red[a][0];
        for (int w = 1; w < kPrepThreads / 32; ++w) v = a < 3 ? fminf(v, red[a][w]) : fmaxf(v, red[a][w]);
        part[6 * blockIdx.x + a] = v;
    }
}

// The points' bounding box (the tree's root cell) from the CTAs' boxes, and
// the count the sort reads. Minima and maxima do not depend on the order they
// are taken in, so the box is exactly the one a single pass finds.
__global__ void box_kernel(const float *part, uint32_t n, uint32_t *count, float *box) {
    const int a = threadIdx.x;
    if (a < 6) {
        float v = part[a];
        for (int b = 1; b < kPrepBlocks; ++b)
            v = a < 3 ? fminf(v, part[6 * b + a]) : fmaxf(v, part[6 * b + a]);
        box[a] = v;
    }
    if (a == 0) *count = n;
}

}  // namespace
}  // namespace pm

using namespace pm;

extern "C" pm_status pm_knn_noalloc(const float4 *points, uint32_t n, const float4 *queries,
                                    uint32_t nq, int k, float radius, uint32_t *idx_out,
                                    float *d2_out, cudaStream_t stream) {
    if (n > kMaxPoints) return PM_ERR_LIMIT;
    if (k < 1 || k > 128 || !(radius > 0.0f)) return PM_ERR_INVALID;
    if ((n && !points) || (nq && (!queries || !idx_out || !d2_out))) return PM_ERR_INVALID;
    unsigned char *base = nullptr;
    if (scratch_address(&base) != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    float4 *ipos = (float4 *)(base + kOffIpos);
    float4 *tpos = (float4 *)(base + kOffTpos);
    float4 *lo = (float4 *)(base + kOffLo);
    float4 *hi = (float4 *)(base + kOffHi);
    uint32_t *count = (uint32_t *)(base + kOffMisc);
    float *box = (float *)(base + kOffMisc + 16);
    MapView m{};
    m.pos = tpos;
    m.pow = nullptr;
    m.lo = lo;
    m.hi = hi;
    m.n = n;
    m.depth = tree_depth(n);
    if (n > 0) {
        // the CTAs' boxes go to the start of the sort-key area, which the
        // build overwrites only after box_kernel has read them (stream order)
        float *part = (float *)(base + kOffKeys);
        prepare_kernel<<<kPrepBlocks, kPrepThreads, 0, stream>>>(points, n, ipos, part);
        note_launch();
        box_kernel<<<1, 32, 0, stream>>>(part, n, count, box);
        note_launch();
        KdBuildArgs a;
        a.n = n;
        a.n_dev = count;
        a.lo = make_float3(0.f, 0.f, 0.f);
        a.hi = make_float3(1.f, 1.f, 1.f);
        a.box_dev = box;
        a.pos_in = ipos;
        a.pow_in = nullptr;
        a.pos_out = tpos;
        a.pow_out = nullptr;
        a.node_lo = lo;
        a.node_hi = hi;
        a.keys = (uint64_t *)(base + kOffKeys);
        a.keys_tmp = (uint64_t *)(base + kOffKeysTmp);
        a.vals = (uint32_t *)(base + kOffVals);
        a.vals_tmp = (uint32_t *)(base + kOffValsTmp);
        a.hist = (uint32_t *)(base + kOffHist);
        a.order_out = nullptr;
        if (build_tree(a, stream) != cudaSuccess) {
            cudaGetLastError();
            return PM_ERR_CUDA;
        }
    }
    if (knn_query(m, queries, nq, k, radius, idx_out, d2_out, stream) != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    return PM_OK;
}
