/*
 * ref_harness.cpp -- runs the reference's own device code serially on the
 * host, to generate golden vectors and to pin the C restatement in
 * oracle/legacy_oracle.c.
 *
 * TEST INFRASTRUCTURE ONLY: built by oracle/ref.mk into
 * oracle/_ref/libpmref.so from photonMappingKernel.cu (lines 6-1521, the
 * scene, photon map and every __device__/__global__ function; the
 * `extern "C"` launchers after line 1521 use <<<>>> and are mirrored here
 * instead). Only tests/golden/make_golden.py loads the result.
 *
 * Serial execution defines the order of the reference's racy `+=` into
 * the photon grid (photonMappingKernel.cu:1068,1158,1177) and of its
 * shared Marsaglia generator (:1029-1036): photon 0 runs to completion,
 * then photon 1, and so on. That is the order the product reproduces.
 */
#include "ref_shim.h"

dim3 blockIdx, blockDim, threadIdx;

#include "ref_body.inc"

namespace {
/* The launch shapes of launch_emit_photons_kernel
 * (photonMappingKernel.cu:1523-1546). */
const int kEmitThreads = 256;
const int kEmitBlocks = (nrPhotons + kEmitThreads - 1) / kEmitThreads;

/* Pixel conversion of photon_mapping_kernel (photonMappingKernel.cu:1451-1459)
 * with the GPU's float-to-integer rule: NaN and negatives give 0, values
 * are truncated toward zero, the reference already clamps above at 255. */
unsigned char to_u8(double v) {
    double c = v > 255.0 ? 255.0 : v;
    if (!(c > 0.0)) return 0;
    return (unsigned char)(int)c;
}
}  // namespace

#define REF_API __attribute__((visibility("default")))

extern "C" {

/* Restores every module-level global the reference initialises statically
 * and later mutates, as a fresh process would see them. */
REF_API void ref_reset(void) {
    m_w = 6548;
    m_z = 316;
    memset(randomNumbers, 0, sizeof(randomNumbers));
    memset(photons, 0, sizeof(photons));
    spheres[0] = make_float4(1.0f, -1.0f, 1.0f, 0.4f);
    spheres[1] = make_float4(-0.6f, -1.0f, 4.5f, 0.4f);
    spheres[2] = make_float4(0.0f, 0.0f, 1.5f, 1.0f);
    gOrigin = make_float3(0.0f, 0.0f, 0.0f);
}

/* launch_init_random_numbers_kernel (photonMappingKernel.cu:1569-1582). */
REF_API void ref_init_random_numbers(void) { init_random_numbers_kernel(); }

/* launch_emit_photons_kernel (photonMappingKernel.cu:1523-1546). */
REF_API void ref_emit(float animTime, int interpolateFlag, int participatingMediaFlag) {
    for (unsigned bx = 0; bx < NR_PHOTONS_X; ++bx)
        for (unsigned by = 0; by < NR_PHOTONS_Y; ++by)
            for (unsigned tx = 0; tx < NR_PHOTONS_Z; ++tx) {
                blockIdx.x = bx; blockIdx.y = by; threadIdx.x = tx;
                init_photons_kernel(animTime);
            }
    blockDim.x = kEmitThreads;
    for (int b = 0; b < kEmitBlocks; ++b)
        for (int t = 0; t < kEmitThreads; ++t) {
            blockIdx.x = b; blockIdx.y = 0; threadIdx.x = t;
            emit_photons_kernel(animTime, interpolateFlag != 0, participatingMediaFlag != 0);
        }
}

/* photon_mapping_kernel (photonMappingKernel.cu:1409-1462), one pixel at a
 * time; rgb_out (optional) receives the float radiance before conversion. */
REF_API void ref_render(unsigned width, unsigned height, float animTime, int interpolateFlag,
                int participatingMediaFlag, unsigned char *rgba_out, float *rgb_out) {
    gOrigin = make_float3(0.0f, 0.0f, 0.0f);
    positionObjects(animTime);
    for (unsigned index = 0; index < width * height; ++index) {
        unsigned x = index % width, y = index / width;
        bool gIntersect = false;
        int gType = 0, gIndex = 0;
        float gSqDist = 0.0f, gDist = -1.0f;
        float3 gPoint = make_float3(0.0f, 0.0f, 0.0f);
        float3 c = computePixelColor(x, y, gDist, gType, gIndex, gIntersect, gPoint, gSqDist,
                                     interpolateFlag != 0, participatingMediaFlag != 0);
        if (rgb_out) {
            rgb_out[3 * index + 0] = c.x;
            rgb_out[3 * index + 1] = c.y;
            rgb_out[3 * index + 2] = c.z;
        }
        rgba_out[4 * index + 0] = to_u8(c.x * 255.0);
        rgba_out[4 * index + 1] = to_u8(c.y * 255.0);
        rgba_out[4 * index + 2] = to_u8(c.z * 255.0);
        rgba_out[4 * index + 3] = 0;
    }
}

REF_API void ref_get_grid(float *out) { memcpy(out, photons, sizeof(photons)); }
REF_API void ref_get_random_numbers(float *out) { memcpy(out, randomNumbers, sizeof(randomNumbers)); }
REF_API void ref_get_rng_state(unsigned *out) { out[0] = m_z; out[1] = m_w; }
REF_API void ref_get_spheres(float *out) { memcpy(out, spheres, sizeof(spheres)); }
REF_API int ref_num_photons(void) { return nrPhotons; }

}  // extern "C"
