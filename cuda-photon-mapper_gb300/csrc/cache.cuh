// cache.cuh -- learned radiance cache: a multiresolution hash-grid encoding
// and a 4 x 64 ReLU MLP (bf16 operands on the tcgen05 tensor cores, fp32
// accumulation in TMEM), trained online on the photon map's own k-NN
// radiance estimates and queried in their place when rendering.
//
// A frame is rendered as a query list (eye_path.cuh): every volume march
// sample and every diffuse hit of every pixel becomes one query record
//   qa = (x, y, z, object id bits; kNone for a volume query)
//   qd = (wo.x, wo.y, wo.z, w)     wo toward the viewer, w = transmittance (* dt)
// whose value -- the k-NN estimate or the network's prediction of it -- is
// summed per pixel in query order: L = sum w * albedo(obj) * value. The
// list holds each block of 32 consecutive pixels in one contiguous range
// (from off[first pixel], off the exclusive scan of the per-pixel counts),
// sample-major within it: the first query of each pixel of the block, then
// the second ones, ... (pixels in order within a step).
#pragma once
#include <cuda_fp16.h>
#include <cstdint>

#include "gather.cuh"
#include "phys_common.cuh"

namespace pm {

constexpr int kCacheIn = 64;        // 32 hash-grid + 16 SH(wo) + normal 3 + kind + bias + zero padding
constexpr int kCacheHidden = 64;
constexpr int kCacheLayers = 4;     // hidden layers
constexpr int kCacheOut = 16;       // output columns, rgb in the first three
constexpr int kCacheMaxLevels = 16;
constexpr int kCacheTile = 128;     // samples per tensor-core tile (one per TMEM lane)
// fp32 MLP parameters, each layer [in][out] row-major: four 64 x 64 hidden
// layers, then 64 x 16.
constexpr int kCacheWeights = kCacheLayers * kCacheIn * kCacheHidden + kCacheHidden * kCacheOut;
constexpr uint32_t kCacheWImageBytes = 4 * 8192 + 2048;
// Scale of the fixed-point table gradient: resolution 2^-44 (5.7e-14), range
// +-2^19 per entry -- a step's per-sample gradients are at most ~1e-1 and an
// entry receives at most batch x 8 corner terms.
constexpr int kTableGradShift = 44;

struct CacheGrid {
    int levels;              // <= kCacheMaxLevels
    uint32_t log2_t;         // entries per level = 2^log2_t
    int res[kCacheMaxLevels];
    float lo[3], inv_size[3];  // world box -> [0,1]^3
};

struct CacheParams {
    float *w;              // fp32 master weights (kCacheWeights)
    float *w_grad, *w_m, *w_v;
    float *w_part;         // per-CTA weight-gradient rows of one backward pass (parts_cap rows)
    int parts_cap;
    float *table;          // fp32 master table, levels * 2^log2_t * 2
    // Table gradient as exact fixed-point sums: two signed 64-bit integers
    // per entry, each term rounded once to a multiple of 2^-kTableGradShift
    // and added with integer atomics, so the sum (and every training step)
    // does not depend on the order the samples' atomics land in.
    long long *table_grad;
    float *table_m, *table_v;
    __half2 *table_h;      // fp16 copy read by the forward passes
    uint4 *w_img;          // bf16 weights in the kernels' shared-memory layout (kCacheWImageBytes)
    float *loss;           // device scalar, summed over a step
    float *loss_part;      // per-CTA loss of one backward pass (parts_cap), added to *loss in CTA order
    float4 *dx;            // per-sample gradient of the 32 hash-grid features (8 float4 per sample)
    uint4 *xt;             // per-sample encoded features, 128-sample tile images (128 B per sample)
    uint32_t dx_cap;       // samples dx and xt hold (a multiple of 128)
    int *status;           // set when a bounded tensor-core wait runs out
    uint32_t wait_polls;   // first bound of every mbarrier wait (kMbarSpin unless lowered for a test)
    // Device-side training state for frames replayed from a CUDA graph
    // (nullable; the host values passed to the calls are used otherwise):
    // the target scale (training divides targets by it, inference
    // multiplies outputs by it) and the Adam step's {lr, c1, c2}.
    const float *scale_dev = nullptr;
    const float *sched = nullptr;
};

// Per-pixel query counts and diffuse-query counts (0 or 1) (count pass);
// records plus the list of diffuse-query indices (write pass, after
// exclusive scans of the counts into off and soff).
cudaError_t cache_count_queries(const PScene &S, const RenderParams &R, bool vol_on, bool surf_on,
                                uint32_t *cnt, uint32_t *scnt, cudaStream_t s);
cudaError_t cache_write_queries(const PScene &S, const RenderParams &R, bool vol_on, bool surf_on,
                                const uint32_t *off, const uint32_t *soff, float4 *qa, float4 *qd,
                                uint32_t *slist, cudaStream_t s);
// rad / rgba of every pixel from the ordered sum of its queries' values.
cudaError_t cache_composite(const PScene &S, const uint32_t *off, const float4 *qa,
                            const float4 *qd, const float4 *val, uint32_t npix, float exposure,
                            float4 *rad, uchar4 *rgba, cudaStream_t s);
// k-NN estimates of queries sel[order[j]] (order[j] when sel is null) into
// val[order[j]], warp w taking the run order[w * run .. (w + 1) * run), each
// query warm-started from its predecessor in the run when both read the
// same map (for sparse sorted picks, where shared candidate sets do not
// pay): diffuse queries e / (pi r^2) / pi, volume queries e / (4/3 pi r^3)
// with the phase function toward wo; with raw set, e and r^2 (-1 when
// nothing was found). With run_ctr (one device word, nullable) the launch
// is persistent: as many warps as fit take runs from the counter.
cudaError_t cache_knn_values_runs(const PScene &S, const MapView &surf, const MapView &vol,
                                  const float4 *qa, const float4 *qd, const uint32_t *sel,
                                  const uint32_t *order, uint32_t n, int run, int k, float radius,
                                  bool raw, float4 *val, uint32_t *run_ctr, int sm_count,
                                  cudaStream_t s);
// The render's radiance from raw per-query values (flux sum, squared radius
// or -1): per pixel, in query order, with exactly the arithmetic of the
// single-kernel render (transmittance factors from the query records), so
// the image is bit-identical to render_frame's.
cudaError_t render_composite(const PScene &S, const uint32_t *off, const float4 *qa,
                             const float4 *qd, const float4 *raw, uint32_t npix, float exposure,
                             float4 *rad, uchar4 *rgba, cudaStream_t s);
// keys[i] = (1 for a volume query, 0 for a diffuse one) << 30 | the 30-bit
// Morton code of query sel[i]'s (or query i's, sel null) position in the
// grid box; vals[i] = i.
cudaError_t cache_sample_keys(const CacheGrid &g, const float4 *qa, const uint32_t *sel, uint32_t n,
                              uint32_t *keys, uint32_t *vals, cudaStream_t s);

// One scene of the batched query-list launches (device array entry): its
// geometry, camera and query kinds, and its slices of the batch's pools.
// The per-pixel arrays hold npix + 1 entries (the last count stays 0, so
// the last offset is the scene's total); the query slice holds nq slots.
struct ListScene {
    PScene sc;
    RenderParams R;
    uint32_t npix;
    int vol_on, surf_on;
    int on;                    // in the query-list render this frame
    uint32_t nq;               // queries of the slice (counted when the batch was made)
    size_t q_first;            // the slice's first slot in the query pool
    CacheGrid box;             // the sort box (lo, inv_size)
    uint32_t *cnt, *scnt;      // per pixel: queries, diffuse queries
    uint32_t *off, *soff;      // their scans, restarted at the scene's first pixel
    float4 *qa, *qd;           // the query slice
    uint32_t *slist;           // the slice's diffuse queries (at most one per pixel)
    const float4 *raw;         // the slice's k-NN estimates (flux sum, r^2)
    float exposure;
    float4 *rad;
    uchar4 *rgba;
};
constexpr uint32_t kListBlock = 128;  // pixels per CTA of the batched list launches
// The count, write and exact-composite passes above over the scenes
// ls[ids[0..n)] in one launch each: blk (device, n + 1 entries) is the
// exclusive scan of the scenes' blocks of kListBlock pixels, blocks its
// total.
// A scene's records never leave its slice: a query past nq is dropped.
cudaError_t list_count_multi(const ListScene *ls, const int *ids, const uint32_t *blk, int n, uint32_t blocks,
                             cudaStream_t s);
cudaError_t list_write_multi(const ListScene *ls, const int *ids, const uint32_t *blk, int n, uint32_t blocks,
                             cudaStream_t s);
cudaError_t list_composite_multi(const ListScene *ls, const int *ids, const uint32_t *blk, int n,
                                 uint32_t blocks, cudaStream_t s);
// Sort keys of the query pool's slots [first, first + n): slot g of scene
// s = tile_scene[g / kSortTile] (-1: none) gets cache_sample_keys' key of
// its query and value g - q_first while it lies below the scene's nq and
// the scene is on; every other slot key 0xffffffff (after all real keys)
// and value 0xffffffff.
cudaError_t list_keys_multi(const ListScene *ls, const int *tile_scene, size_t first, uint32_t n, uint32_t *keys,
                            uint32_t *vals, cudaStream_t s);
// The picks in sorted order (pos[i] the i-th pick, sel[pos[i]] its
// query): their records into pqa, pqd; pord[i] = i.
cudaError_t cache_pick_records(const uint32_t *pos, const uint32_t *sel, const float4 *qa, const float4 *qd,
                               uint32_t n, float4 *pqa, float4 *pqd, uint32_t *pord, cudaStream_t s);
// The training order of n sorted picks in nb batches: sorted pick j
// (records pqa/pqd[j], target pval[j], query sel[pos[j]]) to slot j / nb of
// batch j % nb, batch b holding n / nb + (b < n % nb) samples from
// b * (n / nb) + min(b, n % nb) -- each batch a spatially stratified
// sample, in (map, Morton) order within.
cudaError_t cache_train_order(const float4 *pqa, const float4 *pqd, const float4 *pval,
                              const uint32_t *pos, const uint32_t *sel, uint32_t n, uint32_t nb,
                              float4 *tqa, float4 *tqd, float4 *tgt, uint32_t *tsel, cudaStream_t s);
// v[i] = i for i < n.
cudaError_t cache_iota(uint32_t *v, uint32_t n, cudaStream_t s);
// Training picks from Philox(seed, frame, i): with probability surf_frac
// uniform over the diffuse queries slist[0..ns_total), else uniform over
// all `total` queries.
// With frame_dev (nullable), the frame number is read from device memory.
cudaError_t cache_select(uint64_t seed, uint32_t frame, uint32_t total, const uint32_t *slist,
                         uint32_t ns_total, uint32_t n, float surf_frac, uint32_t *sel,
                         cudaStream_t s, const unsigned long long *frame_dev = nullptr);
// ++*c on the device (a frame counter kept in device memory).
cudaError_t cache_count_up(unsigned long long *c, cudaStream_t s);
// *sum = mean over rgb of val[0..n), summed in a fixed order.
cudaError_t cache_value_sum(const float4 *val, uint32_t n, float *sum, cudaStream_t s);

cudaError_t cache_init(const CacheGrid &g, const CacheParams &p, uint64_t seed, cudaStream_t s);
// Refreshes the fp16 table from the fp32 master copy.
cudaError_t cache_sync_half(const CacheGrid &g, const CacheParams &p, cudaStream_t s);
// Forward + backward of the relative L2 loss (denominator y^2 + rel_eps)
// over n <= p.dx_cap samples (query sel[i], target val[i] * inv_scale); gradients and loss are added to p.w_grad,
// p.table_grad, p.loss with the factor loss_norm (1 / (3 * batch)). x_out
// (n x 64 encoded features) and y_out (n x 4 outputs) are debug copies,
// nullable.
cudaError_t cache_backward(const CacheGrid &g, const CacheParams &p, const PScene &S,
                           const float4 *qa, const float4 *qd, const uint32_t *sel,
                           const float4 *val, uint32_t n, float inv_scale, float loss_norm,
                           float rel_eps, float *x_out, float *y_out, int sm_count, cudaStream_t s);
// out[0 .. levels * 2^log2_t * 2) = the table gradient as floats.
cudaError_t cache_table_grad_float(const CacheGrid &g, const CacheParams &p, float *out,
                                   cudaStream_t s);
// Writes p.w_img from the fp32 weights.
cudaError_t cache_weight_image(const CacheParams &p, cudaStream_t s);
// One Adam step over all parameters; gradients are zeroed after use. The
// table takes lazy steps: entries without a gradient this step keep their
// value and moments (sparse updates of a hash table); the weights take full
// steps and refresh p.w_img.
cudaError_t cache_adam(const CacheGrid &g, const CacheParams &p, float lr, float beta1,
                       float beta2, float eps, int step, cudaStream_t s);
// The Adam schedule on the device (one thread): sched = {lr, c1, c2} for
// the step after *step (lr = lr_min + (lr0 - lr_min) 2^(-step / half_life),
// or lr0 when half_life <= 0; c1, c2 the bias corrections of the step
// count after it), and *step advanced.
cudaError_t cache_schedule(float *sched, unsigned long long *step, float lr0, float lr_min, float half_life,
                           float beta1, float beta2, cudaStream_t s);
// *scale, if still 0, set to the mean over rgb of val[0..n) (1 when that is
// not positive and finite); sum is one word of scratch. Does nothing once
// the scale is set, so a replayed frame keeps the first frame's scale.
cudaError_t cache_scale_init(const float4 *val, uint32_t n, float *sum, float *scale, cudaStream_t s);
// val[i] = max(network(query i), 0) * out_scale for the first n queries,
// taken in the order order[0..n) (nullable: index order).
cudaError_t cache_infer(const CacheGrid &g, const CacheParams &p, const PScene &S,
                        const float4 *qa, const float4 *qd, const uint32_t *order, uint32_t n,
                        float out_scale, float4 *val, int sm_count, cudaStream_t s);

}  // namespace pm
