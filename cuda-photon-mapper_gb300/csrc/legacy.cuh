// legacy.cuh -- the reference's voxel photon mapper (photonMappingKernel.cu)
// as sm_103a kernels: random table, photon emission into the 32^3 grid,
// and the per-pixel render.
//
// The reference accumulates into the grid with unsynchronised `+=` from
// 10,000 threads (photonMappingKernel.cu:1068,1158,1177), so its GPU output
// changes from run to run. Here every deposit is recorded as
// (voxel, value) in photon order, stably sorted by voxel and summed in that
// order, which reproduces the serial execution of the reference's code bit
// for bit, on every run.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace pm {

constexpr int kLegacyGrid = 32;                       // NR_PHOTONS_X/Y/Z (:15-17)
constexpr int kLegacyVoxels = kLegacyGrid * kLegacyGrid * kLegacyGrid;
constexpr int kLegacyPhotons = 10000;                 // nrPhotons (:28)
// Upper bound of grid deposits one photon makes: 3 volume deposits plus,
// per bounce (5), a direct deposit and up to 36 splats for the photon and
// the same for its shadow photon.
constexpr int kLegacyMaxDepositsPerPhoton = 376;
constexpr uint32_t kLegacyMaxDeposits = (uint32_t)kLegacyPhotons * kLegacyMaxDepositsPerPhoton;

enum LegacyFlags { kLegacyInterpolate = 1, kLegacyMedia = 2 };

struct LegacyState {
    float4 *table = nullptr;      // randomNumbers (:78), xyz used
    float *grid3 = nullptr;       // photons[32][32][32] float3 (:76), reference layout
    float4 *grid4 = nullptr;      // same grid padded to float4
    float4 *vol_win = nullptr;    // the render's window sums of the grid (media march)
    float4 *slab_win = nullptr;   // (wall slabs)
    uint32_t *counts = nullptr;   // deposits per photon
    uint32_t *offsets = nullptr;  // exclusive scan of counts
    uint32_t *total = nullptr;    // total deposits (device scalar)
    uint32_t *keys = nullptr, *keys_tmp = nullptr;
    uint32_t *idx = nullptr, *idx_tmp = nullptr;
    float4 *dep = nullptr;        // deposit values in photon order
    float4 *sdep = nullptr;       // the same, in (voxel, photon order) order
    uint32_t *hist = nullptr;
    uint64_t rng_draws = 0;       // draws taken from the shared generator so far
    bool table_written = false;
};

// Marsaglia multiply-with-carry halves (:1029-1036). z' = a(z mod 2^16) +
// floor(z / 2^16) equals a*z mod (a*2^16 - 1) for every reachable state,
// so the state after n draws is a^n * z0 mod (a*2^16 - 1).
constexpr uint32_t kMwcAz = 36969u, kMwcAw = 18000u;
constexpr uint64_t kMwcMz = (uint64_t)kMwcAz * 65536u - 1u;
constexpr uint64_t kMwcMw = (uint64_t)kMwcAw * 65536u - 1u;
constexpr uint32_t kMwcSeedZ = 316u, kMwcSeedW = 6548u;   // m_z, m_w (:1026-1027)

uint32_t mwc_jump_host(uint32_t state, uint64_t a, uint64_t m, uint64_t n);

cudaError_t legacy_alloc(LegacyState &st);
void legacy_free(LegacyState &st);
cudaError_t legacy_init_random(LegacyState &st, cudaStream_t s);
cudaError_t legacy_emit(LegacyState &st, float anim_time, int flags, cudaStream_t s);
cudaError_t legacy_render(const LegacyState &st, uchar4 *out, unsigned width, unsigned height,
                          float anim_time, int flags, float *rgb_out, cudaStream_t s);
// Replaces the grid with a host copy in the reference layout
// (float[32][32][32][3]); used to render a grid produced elsewhere.
cudaError_t legacy_upload_grid(LegacyState &st, const float *host_grid3, cudaStream_t s);
// Sphere placement for animTime (positionObjects, :1380-1404), on the host.
void legacy_position_spheres(float anim_time, float out[2][4]);

}  // namespace pm
