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

#ifdef __cplusplus
}
#endif
#endif /* PM_H */
