/*
 * physical_oracle.h -- CPU restatements of the physically based mode.
 * TEST INFRASTRUCTURE ONLY (tests, smoke check, benchmark CPU baseline).
 *
 * pmo_scene / pmo_config have the memory layout of include/pm.h's
 * pm_scene / pm_config (float4 members 16-byte aligned, float2 8-byte), so
 * the same bytes can be handed to the product and to the oracle.
 */
#ifndef PM_PHYSICAL_ORACLE_H
#define PM_PHYSICAL_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { PMO_MAT_DIFFUSE = 0, PMO_MAT_MIRROR = 1, PMO_MAT_DIELECTRIC = 2 };

typedef struct pmo_material {
    int kind;
    float albedo[3];
    float ior;
} pmo_material;

typedef struct pmo_scene {
    int num_spheres;
    float spheres[64][4] __attribute__((aligned(16)));
    pmo_material sphere_mat[64];
    int num_planes;
    float planes[8][2] __attribute__((aligned(8)));
    pmo_material plane_mat[8];
    float box_min[3], box_max[3];
    float light[3];
    float light_power;
    float sigma_s, sigma_a, hg_g;
    int het_res;
    float het_min, het_max;
    float cam_pos[3];
    float focal;
} __attribute__((aligned(16))) pmo_scene;

typedef struct pmo_config {
    uint64_t seed;
    uint32_t scene_id;
    uint32_t surface_photons;
    uint32_t volume_photons;
    uint32_t max_paths;
    int max_bounces;
    float rr_survival;
    int width, height;
    int k;
    float radius;
    float march_step;
    int leaf_size;
    float exposure;
} pmo_config;

typedef struct pmo_grid pmo_grid;
typedef struct pmo_kd pmo_kd;

/* The benchmark presets 1-3 (preset_oracle.c; the bytes pm_preset writes). */
int pmo_preset(int which, uint64_t seed, pmo_scene *scene, pmo_config *cfg);

/* kd-tree k nearest neighbours (kdtree_oracle.c), pmo_grid_knn's contract. */
pmo_kd *pmo_kd_build(const float (*pos)[4], uint32_t n);
void pmo_kd_free(pmo_kd *t);
int pmo_kd_knn(const pmo_kd *t, const float q[3], int k, float r2, uint64_t *keys);
void pmo_knn_kd(const float (*pos)[4], uint32_t n, const float (*queries)[4], uint32_t nq, int k,
                float radius, uint32_t *idx_out, float *d2_out);
/* The neighbour index pmo_render's gathers use: a kd-tree per map (the
 * default) or a uniform grid of cell = radius. The k-NN sets are the same. */
enum { PMO_GATHER_GRID = 0, PMO_GATHER_KDTREE = 1 };
void pmo_set_gather_index(int which);

/* single precision, bit-exact with the GPU (physical_oracle.c) */
void pmo_trace_path(const pmo_scene *scene, const pmo_config *cfg, const float *het, uint32_t id,
                    float (*spos)[4], float (*spow)[4], uint32_t *ns_out, float (*vpos)[4],
                    float (*vpow)[4], uint32_t *nv_out);
int pmo_emit(const pmo_scene *scene, const pmo_config *cfg, const float *het, float (*spos)[4],
             float (*spow)[4], float (*vpos)[4], float (*vpow)[4], uint32_t *sizes, uint32_t *paths);
pmo_grid *pmo_grid_build(const float (*pos)[4], uint32_t n, float radius);
void pmo_grid_free(pmo_grid *g);
int pmo_grid_knn(const pmo_grid *g, const float q[3], int k, float r2, uint64_t *keys);
/* The estimate sum: order-independent fixed-point sum of n >= 0 float terms. */
float pmo_fixed_sum(const float *t, int n);
void pmo_knn(const float (*pos)[4], uint32_t n, const float (*queries)[4], uint32_t nq, int k,
             float radius, uint32_t *idx_out, float *d2_out);
void pmo_render(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                const float (*spos)[4], const float (*spow)[4], uint32_t ns,
                const float (*vpos)[4], const float (*vpow)[4], uint32_t nv,
                const uint32_t *pixels, uint32_t npix, float (*out)[4], uint64_t *gathers);
/* pmo_render with seconds[0] = neighbour-index build time (kd-trees or
 * grids of both maps), seconds[1] = shading time (all threads). */
void pmo_render_timed(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                      const float (*spos)[4], const float (*spow)[4], uint32_t ns,
                      const float (*vpos)[4], const float (*vpow)[4], uint32_t nv,
                      const uint32_t *pixels, uint32_t npix, float (*out)[4], uint64_t *gathers,
                      double *seconds);
/* A render context that keeps its neighbour indexes (built once) for
 * repeated pixel samples; pmo_render_pixels runs on all threads. The maps
 * must outlive the context. */
typedef struct pmo_render_ctx pmo_render_ctx;
pmo_render_ctx *pmo_render_create(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                                  const float (*spos)[4], const float (*spow)[4], uint32_t ns,
                                  const float (*vpos)[4], const float (*vpow)[4], uint32_t nv);
void pmo_render_pixels(const pmo_render_ctx *x, const uint32_t *pixels, uint32_t npix,
                       float (*out)[4], uint64_t *gathers);
void pmo_render_free(pmo_render_ctx *x);
/* Traces paths first .. first + count - 1 on all threads without keeping
 * their records (a timing sample of the emission); returns the records the
 * paths produced. */
uint64_t pmo_trace_sample(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                          uint32_t first, uint32_t count);
void pmo_noise_grid(float *grid, int res, uint64_t seed, float lo, float hi);
void pmo_philox(uint64_t seed, const uint32_t *ctr, uint32_t *out);
float pmo_logf(float x);
float pmo_expf(float x);
void pmo_sincos2pi(float u, float *s, float *c);
uint32_t pmo_oct_encode(const float *d);
void pmo_oct_decode(uint32_t e, float *d);
/* which: 0 uniform sphere, 1 cosine hemisphere around dir, 2 HG(g) around dir */
void pmo_sample(int which, const float *dir, float g, float u1, float u2, float *out);
float pmo_fresnel(float ci, float eta);
float pmo_hg_phase(float g, float c);
size_t pmo_sizeof_scene(void);
size_t pmo_sizeof_config(void);

/* double precision restatement (physical_oracle64.c): the same methods in
 * float64 with libm, used to measure the GPU's float32 error. */
int pmo64_emit(const pmo_scene *scene, const pmo_config *cfg, const float *het, double *spos,
               double *spow, double *vpos, double *vpow, uint32_t *sizes, uint32_t *paths);
void pmo64_render(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                  const double *spos, const double *spow, uint32_t ns, const double *vpos,
                  const double *vpow, uint32_t nv, const uint32_t *pixels, uint32_t npix,
                  double *out);

void pmo64_radius_gather(const float (*pos)[4], const float (*pw)[4], const float (*dirs)[3],
                         uint32_t n, const float (*pts)[4], const float (*nrm)[4], uint32_t nq,
                         float sq_radius, float exposure, double (*out)[3]);

#ifdef __cplusplus
}
#endif
#endif
