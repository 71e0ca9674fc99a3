/*
 * ref_gpu_runner.cpp -- the reference's own GPU kernels, timed headless:
 * the measured reference-GPU bar of the legacy frame.
 *
 * MEASUREMENT INFRASTRUCTURE ONLY (bench.py's legacy baseline). The
 * kernels are the reference's photonMappingKernel.cu compiled unmodified
 * for sm_103a into oracle/_ref/ref_kernels.cubin (build.py, from the
 * reference checkout, behind the cutil shims in oracle/ref_gpu/); this
 * file only loads that module and replays the reference's three host
 * launch wrappers with their launch shapes and synchronisations:
 *   launch_init_random_numbers_kernel (photonMappingKernel.cu:1569-1583):
 *     init_random_numbers_kernel<<<1, 1>>>, synchronise;
 *   launch_emit_photons_kernel (:1523-1545): init_photons_kernel<<<(32,
 *     32), 32>>>, synchronise, emit_photons_kernel<<<ceil(10000/256),
 *     256>>>, synchronise;
 *   launch_photon_mapping_kernel (:1549-1566): photon_mapping_kernel<<<
 *     ceil(w*h/256), 256>>>, synchronise.
 * The GL pixel buffer the reference writes into is replaced by a device
 * buffer of w*h uchar4.
 *
 * The reference's kernels share one generator and add into the voxel grid
 * without atomics, so their output is not deterministic; they are timed
 * here, never compared. Every index they compute was checked by reading:
 * grid writes clamp to the grid (:1150-1173), gather loops bound their
 * ranges (:314-389, :831-870) and photon indices are tested against the
 * photon count (:1229).
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>

namespace {

CUmodule g_mod = nullptr;
CUfunction g_init_rng = nullptr, g_init_ph = nullptr, g_emit = nullptr, g_render = nullptr;
uchar4 *g_pos = nullptr;
size_t g_pos_bytes = 0;
cudaEvent_t g_ev[2] = {nullptr, nullptr};

int fail(const char *what, int code) {
    std::fprintf(stderr, "ref_gpu_runner: %s failed (%d)\n", what, code);
    return code ? code : -1;
}

#define RG_DRV(x) do { CUresult r_ = (x); if (r_ != CUDA_SUCCESS) return fail(#x, (int)r_); } while (0)
#define RG_RT(x) do { cudaError_t r_ = (x); if (r_ != cudaSuccess) return fail(#x, (int)r_); } while (0)

int launch(CUfunction f, unsigned gx, unsigned gy, unsigned bx, void **args) {
    RG_DRV(cuLaunchKernel(f, gx, gy, 1, bx, 1, 1, 0, nullptr, args, nullptr));
    RG_RT(cudaDeviceSynchronize());
    return 0;
}

}  // namespace

extern "C" {

int pmref_gpu_load(const char *cubin) {
    if (g_mod) return 0;
    RG_RT(cudaFree(nullptr));  // the runtime's primary context becomes current
    RG_DRV(cuModuleLoad(&g_mod, cubin));
    RG_DRV(cuModuleGetFunction(&g_init_rng, g_mod, "_Z26init_random_numbers_kernelv"));
    RG_DRV(cuModuleGetFunction(&g_init_ph, g_mod, "_Z19init_photons_kernelf"));
    RG_DRV(cuModuleGetFunction(&g_emit, g_mod, "_Z19emit_photons_kernelfbb"));
    RG_DRV(cuModuleGetFunction(&g_render, g_mod, "_Z21photon_mapping_kernelP6uchar4jjfbb"));
    RG_RT(cudaEventCreate(&g_ev[0]));
    RG_RT(cudaEventCreate(&g_ev[1]));
    return 0;
}

/* launch_init_random_numbers_kernel; *ms: its device time. */
int pmref_gpu_init_rng(float *ms) {
    if (!g_mod) return -1;
    RG_RT(cudaEventRecord(g_ev[0], 0));
    if (int e = launch(g_init_rng, 1, 1, 1, nullptr)) return e;
    RG_RT(cudaEventRecord(g_ev[1], 0));
    RG_RT(cudaEventSynchronize(g_ev[1]));
    RG_RT(cudaEventElapsedTime(ms, g_ev[0], g_ev[1]));
    return 0;
}

/* One frame: launch_emit_photons_kernel when emit is set, then
 * launch_photon_mapping_kernel into a w*h uchar4 device buffer; the device
 * time of each call (launches and synchronisations) in *ms_emit and
 * *ms_render. */
int pmref_gpu_frame(unsigned w, unsigned h, float anim_time, int interpolate, int media, int emit,
                    float *ms_emit, float *ms_render) {
    if (!g_mod) return -1;
    const size_t bytes = (size_t)w * h * sizeof(uchar4);
    if (bytes > g_pos_bytes) {
        cudaFree(g_pos);
        g_pos = nullptr;
        g_pos_bytes = 0;
        RG_RT(cudaMalloc(&g_pos, bytes));
        g_pos_bytes = bytes;
    }
    bool ib = interpolate != 0, mb = media != 0;
    *ms_emit = 0.0f;
    if (emit) {
        void *a_init[] = {&anim_time};
        void *a_emit[] = {&anim_time, &ib, &mb};
        const unsigned blocks = (10000u + 255u) / 256u;
        RG_RT(cudaEventRecord(g_ev[0], 0));
        if (int e = launch(g_init_ph, 32, 32, 32, a_init)) return e;
        if (int e = launch(g_emit, blocks, 1, 256, a_emit)) return e;
        RG_RT(cudaEventRecord(g_ev[1], 0));
        RG_RT(cudaEventSynchronize(g_ev[1]));
        RG_RT(cudaEventElapsedTime(ms_emit, g_ev[0], g_ev[1]));
    }
    uchar4 *pos = g_pos;
    void *a_render[] = {&pos, &w, &h, &anim_time, &ib, &mb};
    const unsigned blocks = (unsigned)(((size_t)w * h + 255u) / 256u);
    RG_RT(cudaEventRecord(g_ev[0], 0));
    if (int e = launch(g_render, blocks, 1, 256, a_render)) return e;
    RG_RT(cudaEventRecord(g_ev[1], 0));
    RG_RT(cudaEventSynchronize(g_ev[1]));
    RG_RT(cudaEventElapsedTime(ms_render, g_ev[0], g_ev[1]));
    return 0;
}

void pmref_gpu_unload(void) {
    if (g_pos) cudaFree(g_pos);
    g_pos = nullptr;
    g_pos_bytes = 0;
    if (g_ev[0]) cudaEventDestroy(g_ev[0]);
    if (g_ev[1]) cudaEventDestroy(g_ev[1]);
    g_ev[0] = g_ev[1] = nullptr;
    if (g_mod) cuModuleUnload(g_mod);
    g_mod = nullptr;
}

}  // extern "C"
