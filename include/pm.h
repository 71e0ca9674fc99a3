/*
 * pm.h -- C ABI of the GB300 photon mapper (libphotonmap.so).
 *
 * Two groups of entry points:
 *
 *  1. The reference's own three exports, same names and signatures
 *     (gamalik/cuda-photon-mapper photonMappingKernel.cu:1523,1549,1569,
 *     declared by its caller at simplePBO.cpp:27-29). They drive an
 *     implicit per-process context on the current device, run on the
 *     default stream and return after the GPU finishes, like the
 *     reference. `pos` is any device buffer of width*height uchar4 (the
 *     reference passes a mapped OpenGL PBO; this build is headless).
 *
 *  2. The pm_* API: explicit context, explicit stream, status codes and
 *     no process exit. Calls on a context are asynchronous on the stream
 *     they are given unless documented otherwise; a context belongs to one
 *     host thread at a time.
 */
#ifndef PM_H
#define PM_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h>
#include <vector_types.h>

#if defined(__GNUC__)
#define PM_API __attribute__((visibility("default")))
#else
#define PM_API
#endif

#ifdef __cplusplus
#define PM_BOOL bool
extern "C" {
#else
#include <stdbool.h>
#define PM_BOOL bool
#endif

/* ---- 1. reference exports ------------------------------------------------ */

/* launch_init_random_numbers_kernel (photonMappingKernel.cu:1569-1582): fills
 * the 10,000-entry random table from the shared Marsaglia generator. */
PM_API void launch_init_random_numbers_kernel(void);

/* launch_emit_photons_kernel (photonMappingKernel.cu:1523-1546): clears the
 * 32^3 photon grid, places the spheres for animTime and emits the 10,000
 * photons. pos, image_width, image_height and interpolateFlag are unused,
 * as in the reference. */
PM_API void launch_emit_photons_kernel(uchar4 *pos, unsigned int image_width, unsigned int image_height,
                                float animTime, PM_BOOL interpolateFlag,
                                PM_BOOL participatingMediaFlag);

/* launch_photon_mapping_kernel (photonMappingKernel.cu:1549-1566): one eye
 * ray per pixel, writes width*height RGBA8 pixels (alpha 0) to pos, row 0
 * at the top. */
PM_API void launch_photon_mapping_kernel(uchar4 *pos, unsigned int image_width,
                                  unsigned int image_height, float animTime,
                                  PM_BOOL interpolateFlag, PM_BOOL participatingMediaFlag);

/* The reference prints and calls exit(EXIT_FAILURE) on a CUDA error
 * (checkCUDAError, photonMappingKernel.cu:49-55); the three exports above
 * do the same by default. With exit_on_error = 0 they record the error
 * instead (read it with pm_legacy_last_status / pm_legacy_last_error). */
PM_API void pm_legacy_set_exit_on_error(int exit_on_error);
PM_API int pm_legacy_last_status(void);
PM_API const char *pm_legacy_last_error(void);
/* Releases the implicit context of the three exports (all its device
 * memory); the next export call creates a fresh one. */
PM_API void pm_legacy_release(void);

/* ---- 2. pm_* API ----------------------------------------------------------- */

typedef enum pm_status {
    PM_OK = 0,
    PM_ERR_INVALID = 1,  /* bad argument */
    PM_ERR_CUDA = 2,     /* a CUDA call failed; see pm_last_error */
    PM_ERR_ALLOC = 3,    /* device allocation failed */
    PM_ERR_STATE = 4,    /* call out of order (e.g. render before build) */
    PM_ERR_LIMIT = 5,    /* size beyond a documented maximum */
    PM_ERR_TIMEOUT = 6   /* a bounded device wait gave up */
} pm_status;

typedef struct pm_ctx pm_ctx;

/* Legacy-mode flags: the reference's keyboard toggles 'i' and 'p'
 * (callbacksPBO.cpp:123-131). */
#define PM_LEGACY_INTERPOLATE 1
#define PM_LEGACY_MEDIA 2

/* Legacy grid and table sizes (photonMappingKernel.cu:15-17,28). */
#define PM_LEGACY_GRID 32
#define PM_LEGACY_PHOTONS 10000

PM_API pm_status pm_create(pm_ctx **out, int device);
PM_API void pm_destroy(pm_ctx *ctx);
PM_API const char *pm_last_error(const pm_ctx *ctx);
PM_API const char *pm_status_string(pm_status s);

/* Legacy mode on an explicit context and stream. */
PM_API pm_status pm_legacy_init_random(pm_ctx *ctx, cudaStream_t stream);
PM_API pm_status pm_legacy_emit(pm_ctx *ctx, float anim_time, int flags, cudaStream_t stream);
/* rgb_out (nullable, device): width*height*3 floats of radiance before
 * the 8-bit conversion. */
PM_API pm_status pm_legacy_render(pm_ctx *ctx, uchar4 *pos, unsigned width, unsigned height,
                           float anim_time, int flags, float *rgb_out, cudaStream_t stream);
/* Synchronous copies of the photon grid (float[32][32][32][3], the
 * reference's `photons` layout) and of the random table (float[10000][3]). */
PM_API pm_status pm_legacy_get_grid(pm_ctx *ctx, float *host_out);
PM_API pm_status pm_legacy_set_grid(pm_ctx *ctx, const float *host_in);
PM_API pm_status pm_legacy_get_random_numbers(pm_ctx *ctx, float *host_out);
/* Draws taken from the shared generator so far (30,000 per table fill,
 * 90,000 per emission with participating media). */
PM_API pm_status pm_legacy_rng_draws(pm_ctx *ctx, unsigned long long *draws);

/* ---- 3. physically based mode --------------------------------------------
 *
 * Photon tracing through a Cornell-style box with spheres and a
 * participating medium, a kd-tree over each photon map and a k-nearest
 * photon radiance estimate per pixel. The scene keeps the reference's layout
 * (float4 spheres = centre xyz + radius, float2 planes = axis code + offset,
 * photonMappingKernel.cu:59-73) and adds a material per object. Photon
 * records export in the reference's record layout {location, direction,
 * energy} ("photonMappingKernel - Copy.cu":30-31). */

#define PM_MAX_SPHERES 64
#define PM_MAX_PLANES 8

enum { PM_MAT_DIFFUSE = 0, PM_MAT_MIRROR = 1, PM_MAT_DIELECTRIC = 2 };
enum { PM_MAP_SURFACE = 0, PM_MAP_VOLUME = 1 };

typedef struct pm_material {
    int kind;          /* PM_MAT_* */
    float albedo[3];   /* diffuse reflectance (diffuse only) */
    float ior;         /* index of refraction (dielectric only) */
} pm_material;

typedef struct pm_scene {
    int num_spheres;
    float4 spheres[PM_MAX_SPHERES];          /* centre xyz, radius w */
    pm_material sphere_mat[PM_MAX_SPHERES];
    int num_planes;
    float2 planes[PM_MAX_PLANES];            /* axis (0=x,1=y,2=z) as float, offset */
    pm_material plane_mat[PM_MAX_PLANES];
    float box_min[3], box_max[3];            /* planes are bounded by this box; the medium fills it */
    float light[3];                          /* isotropic point light */
    float light_power;                       /* watts, white */
    float sigma_s, sigma_a, hg_g;            /* homogeneous medium (sigma_s = 0: none) */
    int het_res;                             /* >0: sigma_s from a het_res^3 value-noise grid */
    float het_min, het_max;                  /* range the noise grid is scaled to */
    float cam_pos[3];                        /* pinhole camera looking +z */
    float focal;
} pm_scene;

typedef struct pm_config {
    uint64_t seed;              /* Philox key (low and high words) */
    uint32_t scene_id;          /* Philox counter word 3: separates scenes of a batch */
    uint32_t surface_photons;   /* target size of the surface map */
    uint32_t volume_photons;    /* target size of the volume map */
    uint32_t max_paths;         /* cap on emitted paths, 0 = 16 x the larger target */
    int max_bounces;            /* interactions per path */
    float rr_survival;          /* Russian-roulette survival probability */
    int width, height;          /* image */
    int k;                      /* neighbours per radiance estimate (<= 128) */
    float radius;               /* gather radius cap */
    float march_step;           /* volume ray-march step, 0 = no march */
    int leaf_size;              /* kd-tree leaf size: 32 (one warp) */
    float exposure;             /* scale applied before the 8-bit conversion */
} pm_config;

/* The reference's record layout: one photon as three float3. */
typedef struct pm_photon_record {
    float location[3];
    float direction[3];   /* direction of travel when stored */
    float energy[3];      /* flux, watts per channel */
} pm_photon_record;

typedef struct pm_frame_stats {
    uint64_t paths_traced;              /* photon paths emitted this frame */
    uint32_t map_size[2];               /* records in the surface / volume map */
    uint32_t map_paths[2];              /* paths that the map's power is normalised by */
    uint64_t surface_gathers;           /* k-NN queries on the surface map */
    uint64_t volume_gathers;            /* k-NN queries on the volume map (march steps) */
    float ms_emit, ms_build, ms_render; /* device time of the last emit / build / render */
    float ms_gather;                    /* of ms_render: the k-NN estimates (the whole
                                           kernel for pm_render_single_kernel) */
} pm_frame_stats;

/* Fills *scene and *cfg with one of the benchmark presets:
 * 1 = small box, 2 spheres, 100k photons, 512^2, k=64;
 * 2 = 8 seeded spheres, 1M surface + 1M volume photons, 1024^2, k=100, step 0.01;
 * 3 = 64 spheres, heterogeneous medium, 8M + 8M photons, 1920x1080, k=128.
 * Host only; needs no GPU. */
PM_API pm_status pm_preset(int preset, uint64_t seed, pm_scene *scene, pm_config *cfg);

/* Installs a scene and configuration (copies both); allocates the maps. */
PM_API pm_status pm_set_scene(pm_ctx *ctx, const pm_scene *scene, const pm_config *cfg);
/* Replaces the scene of the next frame (geometry, materials, light, medium
 * coefficients, camera) without reallocating: sphere and plane counts may
 * change, het_res may not. The per-frame counterpart of the reference's
 * positionObjects(animTime) (photonMappingKernel.cu:1380-1404). */
PM_API pm_status pm_update_scene(pm_ctx *ctx, const pm_scene *scene);
/* Traces photon paths until both maps reach their targets. Synchronises
 * the stream once to learn the map sizes. */
PM_API pm_status pm_emit(pm_ctx *ctx, cudaStream_t stream);
/* Builds the kd-tree of each map: level-by-level median splits along each
 * cell's longest axis (stable radix sort per level) and tight node boxes. */
PM_API pm_status pm_build(pm_ctx *ctx, cudaStream_t stream);
/* Renders one frame: eye rays, specular chains, the volume march and the
 * surface radiance estimate. radiance (nullable, device): width*height
 * float4 (rgb, alpha = 1); rgba (nullable, device): width*height uchar4. */
PM_API pm_status pm_render(pm_ctx *ctx, float4 *radiance, uchar4 *rgba, cudaStream_t stream);
/* The same image from one kernel launch (a warp per pixel marching its eye
 * path, each k-NN warm-started from the previous march sample), without the
 * query list: no host synchronisation, slower on large frames. pm_render
 * builds the frame's query list (one stream synchronisation to size it),
 * estimates the queries in spatial order from one shared candidate set per
 * group of 32 neighbours, and sums them per pixel with this kernel's
 * arithmetic; the k-NN sets are exact and the estimate sum is independent
 * of the order of the records, so the two are bit-identical. */
PM_API pm_status pm_render_single_kernel(pm_ctx *ctx, float4 *radiance, uchar4 *rgba,
                                         cudaStream_t stream);
/* Counters of the last pm_render's k-NN estimates (n <= 7 of them):
 * [0] queries estimated from a shared candidate set, [1] by the list
 * search, [2] single queries whose radius was narrowed to fit their set,
 * [3] results that contradicted their upper bound and were redone by the
 * list search (0 while the bounds hold), [4] candidate sets collected,
 * [5] candidates collected, [6] segments halved because their set did not
 * fit in shared memory. */
PM_API pm_status pm_get_gather_stats(pm_ctx *ctx, uint64_t *out, int n);
/* k nearest photons of map `map` for nq query points (device float4
 * xyz), within radius; idx_out / d2_out (device, nq*k) receive photon
 * indices and squared distances sorted by (distance, index); missing
 * neighbours are 0xFFFFFFFF / radius^2. Needs pm_build. */
PM_API pm_status pm_knn(pm_ctx *ctx, int map, const float4 *queries, uint32_t nq, int k,
                        float radius, uint32_t *idx_out, float *d2_out, cudaStream_t stream);
/* The reference's record-list radius gather (kernelPBO.cu:165-182,
 * "photonMappingKernel - Copy.cu":191-208) over map `map`: for each of nq
 * points (device float4 xyz) with normal (device float4 xyz), the sum over
 * photons with squared distance <= sq_radius of energy * max(0, -N.dir) *
 * (1 - distance) / exposure, into out (device float4 rgb). Unlike the
 * reference, photons are not restricted to the queried object. Needs
 * pm_build. */
PM_API pm_status pm_radius_gather(pm_ctx *ctx, int map, const float4 *points,
                                  const float4 *normals, uint32_t nq, float sq_radius,
                                  float exposure, float4 *out, cudaStream_t stream);
/* Synchronous copy of a map in index order, in the reference's record
 * layout (cap records at most); *count receives the map size. */
PM_API pm_status pm_get_photons(pm_ctx *ctx, int map, pm_photon_record *out, uint32_t cap,
                                uint32_t *count);
/* Synchronous copy of a map's raw SoA records in index order: pos = xyz +
 * index bits, pow = rgb flux + octahedral direction bits. */
PM_API pm_status pm_get_photons_soa(pm_ctx *ctx, int map, float4 *pos, float4 *pow,
                                    uint32_t cap, uint32_t *count);
PM_API pm_status pm_get_stats(pm_ctx *ctx, pm_frame_stats *out);
/* Replaces map `map` with n host records in the SoA layout of
 * pm_get_photons_soa (pos.w is overwritten with the record index); used to
 * load a saved map or to query an arbitrary point set. Needs pm_set_scene
 * (its box is the tree's root cell); follow with pm_build. */
PM_API pm_status pm_set_photons(pm_ctx *ctx, int map, const float4 *pos, const float4 *pow,
                                uint32_t n);

/* ---- 4. allocation-free k-NN ------------------------------------------------
 *
 * No counterpart in the reference. For callers that cannot allocate device
 * memory -- code running inside another framework's memory pool or
 * stream-ordered allocator, plug-ins whose host forbids device allocation
 * after start-up, real-time loops that must not risk an allocation stall or
 * failure -- pm_knn_noalloc answers the same queries as pm_set_photons +
 * pm_build + pm_knn over n caller-provided points (device float4, xyz; the
 * point's position in the array is its index for ties and in idx_out) and
 * calls no cudaMalloc, cudaFree or other allocating routine. Its temporary
 * memory is one fixed file-scope device array of
 * PM_KNN_NOALLOC_SCRATCH_BYTES (about 7.3 MiB) that every GPU loading the
 * library holds until the process exits; n above PM_KNN_NOALLOC_MAX_POINTS
 * returns PM_ERR_LIMIT.
 *
 * The first call on each device looks up that array's device address
 * (cudaGetSymbolAddress) with the device current; make that first call
 * before any stream capture. All calls share the array and it keeps the
 * last call's contents, so calls that overlap on the GPU (other streams,
 * other host threads on the same device) race and must be serialised by the
 * caller. Needs no pm_ctx. */
#define PM_KNN_NOALLOC_MAX_POINTS (1u << 17)
#define PM_KNN_NOALLOC_SCRATCH_BYTES 7635456u
PM_API pm_status pm_knn_noalloc(const float4 *points, uint32_t n, const float4 *queries,
                                uint32_t nq, int k, float radius, uint32_t *idx_out,
                                float *d2_out, cudaStream_t stream);

/* ---- 5. host utilities ------------------------------------------------------- */

/* Saves map `map` in index order: one JSON header line, then the records'
 * float4 pos array and float4 pow array (the layout of pm_get_photons_soa). */
PM_API pm_status pm_save_map(pm_ctx *ctx, int map, const char *path);
/* Loads a file written by pm_save_map into map `map` (as pm_set_photons;
 * follow with pm_build). */
PM_API pm_status pm_load_map(pm_ctx *ctx, int map, const char *path);
/* Writes width*height host RGBA8 pixels as a binary PPM (RGB, row 0 on top):
 * the headless stand-in for the reference's GL blit (callbacksPBO.cpp:65-92). */
PM_API pm_status pm_write_ppm(const char *path, const uchar4 *rgba, unsigned width,
                              unsigned height);
/* The same pixels as an 8-bit RGB PNG (row 0 on top; the zlib stream in
 * stored deflate blocks, so the file is about the size of a PPM). */
PM_API pm_status pm_write_png(const char *path, const uchar4 *rgba, unsigned width,
                              unsigned height);

/* Headless frame driver with the reference's frame loop and keys
 * (callbacksPBO.cpp:19-27 state, :47-101 display, :104-143 keyboard): the
 * first display runs initCuda's early emission, then the random table; each
 * display emits when emit_flag is set, renders into `pos` (device,
 * width*height uchar4), and advances anim_time by anim_inc when anim_flag is
 * set. Key 27 sets quit instead of exiting the process. */
typedef struct pm_viewer pm_viewer;
typedef struct pm_viewer_state {
    unsigned width, height;
    int anim_flag, emit_flag, interpolate, media;
    int iter, quit;
    float anim_time, anim_inc;
    unsigned long long frames;
} pm_viewer_state;
PM_API pm_status pm_viewer_create(pm_viewer **out, unsigned width, unsigned height);
PM_API void pm_viewer_destroy(pm_viewer *v);
PM_API void pm_viewer_key(pm_viewer *v, unsigned char key);
PM_API pm_status pm_viewer_state_get(const pm_viewer *v, pm_viewer_state *out);
PM_API pm_status pm_viewer_display(pm_viewer *v, uchar4 *pos);

/* Physically based frame driver: the reference's frame loop
 * (callbacksPBO.cpp:47-101) over pm_emit / pm_build / pm_render, with
 * temporal reuse. pm_phys_viewer_create installs the scene (pm_set_scene) on
 * ctx. Each display: with anim_flag set, sphere 0 moves to x + anim_radius *
 * sin(anim_time) (clamped inside the box; pm_update_scene); the photon maps
 * are re-emitted and their kd-trees rebuilt only when the scene changed
 * since the last emission, emit_flag is set, or no maps exist yet -- an
 * unchanged scene gives the same maps, so they are reused; with use_cache
 * set and the radiance cache enabled (pm_cache_enable) the network takes
 * cache_frames online training frames on the current maps and renders the
 * frame (pm_render_cached; the network carries over from frame to frame),
 * else pm_render; anim_time then advances by anim_inc when anim_flag is set.
 * Keys as the reference's keyboard() (callbacksPBO.cpp:104-143): 'a'
 * animation, 'e' re-emission every frame, '+' / '-' / 'r' anim_inc, 27 quit;
 * plus 'c' for the cache. The context must outlive the driver. */
typedef struct pm_phys_viewer pm_phys_viewer;
typedef struct pm_phys_viewer_state {
    int anim_flag, emit_flag, use_cache, cache_frames;
    float anim_time, anim_inc, anim_radius;
    int quit;
    unsigned long long frames, emissions, reuses, cached_frames;
} pm_phys_viewer_state;
PM_API pm_status pm_phys_viewer_create(pm_ctx *ctx, const pm_scene *scene, const pm_config *cfg,
                                       pm_phys_viewer **out);
PM_API void pm_phys_viewer_destroy(pm_phys_viewer *v);
PM_API void pm_phys_viewer_key(pm_phys_viewer *v, unsigned char key);
PM_API pm_status pm_phys_viewer_state_get(const pm_phys_viewer *v, pm_phys_viewer_state *out);
PM_API pm_status pm_phys_viewer_display(pm_phys_viewer *v, float4 *radiance, uchar4 *rgba,
                                        cudaStream_t stream);

/* ---- 6. learned radiance cache ------------------------------------------------
 * No counterpart in the reference, whose render always gathers photons. A
 * frame is split into radiance queries -- every volume march sample and the
 * diffuse hit of each pixel's eye path, as pm_render visits them -- whose
 * k-NN estimates a small network learns: a multiresolution hash-grid
 * encoding of the position (fp16 table), spherical harmonics of the view
 * direction, the facing normal, and a 4 x 64 ReLU MLP run in bf16 on the
 * tensor cores with fp32 accumulation. pm_cache_train fits it online to
 * k-NN estimates at random queries of the current frame; pm_render_cached
 * sums the network's predictions per pixel (source 0) or, as its fallback
 * and yardstick, the k-NN estimates of every query (source 1, equal to
 * pm_render up to summation rounding). The cache lives in the context and
 * survives pm_set_scene. */
typedef struct pm_cache_config {
    int levels;              /* hash-grid levels, 1..16 */
    int log2_table;          /* entries per level = 2^log2_table, 8..22 */
    int base_res, max_res;   /* coarsest and finest grid resolution */
    uint32_t train_samples;  /* k-NN samples per training frame, <= 2^24 */
    uint32_t batch;          /* samples per Adam step, a multiple of 128 */
    float lr, beta1, beta2, eps;  /* Adam */
    float lr_min;            /* learning rate decays toward lr_min ... */
    float lr_half_life;      /* ... halving the gap every lr_half_life steps (0: constant) */
    float loss_eps;          /* relative L2 denominator y^2 + loss_eps (targets have mean 1) */
    float surface_fraction;  /* share of each frame's samples drawn from the diffuse queries */
    uint64_t seed;
} pm_cache_config;

typedef struct pm_cache_stats {
    unsigned long long queries;      /* queries of the last cached frame */
    unsigned long long train_steps;  /* Adam steps so far */
    unsigned long long train_frames;
    float loss;                      /* mean loss of the last training frame */
    float target_scale;              /* targets are divided by this before the loss */
    float ms_queries;                /* last query-list build */
    float ms_values;                 /* last per-query values (network or k-NN) */
    float ms_composite;
    float ms_targets, ms_train;      /* last training frame: k-NN targets, steps */
    int tc_status;                   /* nonzero: a tensor-core wait ran out */
} pm_cache_stats;

#define PM_CACHE_WEIGHTS (4 * 64 * 64 + 64 * 16)
PM_API void pm_cache_default_config(pm_cache_config *cfg);
/* Allocates and initialises the cache (cfg NULL: defaults). Re-enabling
 * resets the network. */
PM_API pm_status pm_cache_enable(pm_ctx *ctx, const pm_cache_config *cfg);
PM_API pm_status pm_cache_disable(pm_ctx *ctx);
/* `frames` training frames on the built photon maps and the current camera:
 * each draws train_samples queries, estimates them with the k-NN gather and
 * takes train_samples / batch Adam steps. */
PM_API pm_status pm_cache_train(pm_ctx *ctx, int frames, cudaStream_t stream);
/* Renders through the query list: source 0 = network, 1 = k-NN estimates.
 * radiance / rgba as pm_render (either nullable). */
PM_API pm_status pm_render_cached(pm_ctx *ctx, float4 *radiance, uchar4 *rgba, int source,
                                  cudaStream_t stream);
PM_API pm_status pm_cache_get_stats(pm_ctx *ctx, pm_cache_stats *out);
/* Diagnostics of the tensor-core kernels' bounded waits. Every mbarrier
 * wait of the training and inference kernels (the weight copy, each MMA
 * round) polls at most `polls` times before it gives up (polls < 0: the
 * default, 2^24); a wait that gives up sets tc_status, keeps waiting under
 * the default bound so that no copy or MMA is left in flight, and its CTA
 * stops after the current tile of 128 samples. A low bound makes that path
 * run without a hang (0: give up without polling). pm_cache_clear_status
 * zeroes tc_status (synchronises the device). */
PM_API pm_status pm_cache_set_wait_limit(pm_ctx *ctx, int polls);
PM_API pm_status pm_cache_clear_status(pm_ctx *ctx);
/* Host copies of the fp32 weights (PM_CACHE_WEIGHTS: four [64 in][64 out]
 * layers, then [64][16]), the fp32 table (levels * 2^log2_table * 2,
 * nullable) and the grid resolutions (levels ints, nullable). */
PM_API pm_status pm_cache_get_params(pm_ctx *ctx, float *weights, float *table, int *res);
PM_API pm_status pm_cache_set_params(pm_ctx *ctx, const float *weights, const float *table);
/* Forward and backward of the loss over n host queries (qa, qd as the query
 * list stores them; target = k-NN values), without an update. Outputs, all
 * host and nullable: x (n x 64 encoded features), y (n x 4), *loss, weight
 * gradients (PM_CACHE_WEIGHTS), table gradients (table size). */
PM_API pm_status pm_cache_debug_step(pm_ctx *ctx, const float4 *qa, const float4 *qd,
                                     const float4 *target, uint32_t n, float target_scale,
                                     float *x, float *y, float *loss, float *w_grad,
                                     float *table_grad);
/* Query list of the current camera (host copies, nullable; *count always). */
PM_API pm_status pm_cache_get_queries(pm_ctx *ctx, float4 *qa, float4 *qd, uint32_t cap,
                                      uint32_t *count);
/* Per-query values of the last pm_render_cached, host copy. Source 0: the
 * network's radiance before the transmittance and albedo factors. Source 1:
 * the k-NN flux sum (xyz) and the squared gather radius (w; -1 where no
 * record was found). PM_ERR_STATE after a pm_render, which reuses them. */
PM_API pm_status pm_cache_get_values(pm_ctx *ctx, float4 *val, uint32_t cap, uint32_t *count);
/* The k-NN targets of the next training frame, as pm_cache_train computes
 * them (spatially sorted, warm-started runs), without training: host copies
 * of train_samples targets and the query index of each (both nullable).
 * For checking the targets against per-query k-NN values. */
PM_API pm_status pm_cache_debug_targets(pm_ctx *ctx, float4 *targets, uint32_t *query);
/* Network + table + Adam state to a file (JSON header line, then raw fp32
 * arrays) and back; load requires the same levels and log2_table. */
PM_API pm_status pm_cache_save(pm_ctx *ctx, const char *path);
PM_API pm_status pm_cache_load(pm_ctx *ctx, const char *path);

/* ---- 7. batched scenes ---------------------------------------------------------
 * No counterpart in the reference, which renders one scene. A batch holds
 * many independent scenes (own maps, trees, images, k and resolution) and
 * runs a frame of all of them in shared launches:
 *  - one persistent trace launch over every scene's photon paths (counting
 *    pass);
 *  - every map's record extent from one segmented scan of all path counts;
 *  - one persistent trace launch (writing pass);
 *  - the kd-trees of all maps, level by level and finish by finish;
 *  - the render. Every query-list scene's query list (counts, scans,
 *    records, spatial sort) is built into one arena sized at creation, with
 *    every count kept on the device. Then one persistent shared-candidate
 *    estimate launch per k-list width and one composite launch. The scenes
 *    in per-pixel mode go through one persistent launch that hands out
 *    pixel chunks of all of them dynamically.
 * The number of launches does not grow with the number of scenes. No step
 * reads a count back to the host, so the whole frame can be captured as a
 * CUDA graph (pm_batch_capture) and replayed (pm_batch_launch). Every
 * scene's image is bit-identical to a single-scene pm_emit + pm_build +
 * pm_render with the same scene, config and path cap. */
typedef struct pm_batch pm_batch;
/* Search knobs of one scene that change speed, never results: records per
 * kd leaf (32, 64, 128); query_list 1: render through the query list with
 * shared candidate sets (the default), 0: in the persistent per-pixel
 * launch, where the rest apply -- pixels per warp per work chunk (1..64),
 * records collected before the first k-list sort (32, 64, 128), and the
 * leaf candidates at or above which insertion is one bulk merge (1..33). */
typedef struct pm_batch_tune {
    int leaf_size, tile, collect_max, merge_min, query_list;
} pm_batch_tune;
/* Scene `index` of the batched benchmark workload: 2..32 seeded spheres,
 * sigma_s in [0, 0.2], photons log-uniform in [1e5, 4e6] (half per map),
 * 256^2 / 512^2 / 1024^2 pixels, k of 32 / 64 / 128; scene_id = index. */
PM_API pm_status pm_batch_scene(int index, uint64_t seed, pm_scene *scene, pm_config *cfg);
/* cfg[i].max_paths = 0 caps scene i at 8 x its larger map target. */
PM_API pm_status pm_batch_create(pm_ctx *ctx, int n, const pm_scene *scenes, const pm_config *cfgs,
                                 pm_batch **out);
PM_API void pm_batch_destroy(pm_batch *b);
PM_API pm_status pm_batch_frame(pm_batch *b, cudaStream_t stream);
/* Records one frame as a CUDA graph (the stream must not be capturing). */
PM_API pm_status pm_batch_capture(pm_batch *b, cudaStream_t stream);
/* Replays the captured frame. */
PM_API pm_status pm_batch_launch(pm_batch *b, cudaStream_t stream);
/* Device pointers of scene i's radiance (float4) and image (uchar4). */
PM_API pm_status pm_batch_image(pm_batch *b, int scene, float4 **radiance, uchar4 **rgba);
/* Host copies of scene i's radiance and image (nullable; synchronises). */
PM_API pm_status pm_batch_read(pm_batch *b, int scene, float4 *radiance, uchar4 *rgba);
/* Scene i's map sizes, paths and gathers of the last frame (synchronises). */
PM_API pm_status pm_batch_stats(pm_batch *b, int scene, pm_frame_stats *out);
PM_API pm_status pm_batch_set_tune(pm_batch *b, int scene, const pm_batch_tune *tune);
PM_API pm_status pm_batch_get_tune(pm_batch *b, int scene, pm_batch_tune *tune);
/* Autotuner: for each k of the batch, times the render of its largest scene
 * over leaf size x tile, then collect_max x merge_min at the best of those,
 * applies the fastest setting to every scene with that k and writes every
 * trial and choice to json_path (nullable). Rebuilds the trees it changes;
 * a captured graph is dropped (capture again). */
PM_API pm_status pm_batch_autotune(pm_batch *b, const char *json_path, cudaStream_t stream);
/* Per-scene learned radiance caches (NULL config: pm_cache_default_config;
 * scene i's network starts from seed cfg.seed + i, its grid spans its own
 * scene box). From the next frame on, each scene's frame trains its network
 * on cfg.train_samples k-NN targets of its query list (Adam steps of
 * cfg.batch samples) and then renders every query of the list through the
 * network instead of the k-NN estimate. The learning-rate schedule, the
 * target scale and the frame counter live in device memory, so a captured
 * frame keeps training when it is replayed. Every scene is switched to the
 * query-list render (pm_batch_set_tune then refuses query_list 0, and
 * pm_batch_autotune refuses to run); a captured frame is dropped. */
PM_API pm_status pm_batch_cache_enable(pm_batch *b, const pm_cache_config *cfg);
/* Frees the caches: frames render through the k-NN estimates again. */
PM_API pm_status pm_batch_cache_disable(pm_batch *b);

/* Kernels this library has launched since it was loaded (all contexts). */
PM_API unsigned long long pm_kernel_launches(void);

/* sizeof of the ABI structs as this library was compiled (0 = pm_scene,
 * 1 = pm_config, 2 = pm_photon_record, 3 = pm_frame_stats,
 * 4 = pm_cache_config, 5 = pm_cache_stats), for bindings in other
 * languages to check their struct layouts against. */
PM_API size_t pm_abi_struct_size(int which);

#ifdef __cplusplus
}
#endif
#endif /* PM_H */
