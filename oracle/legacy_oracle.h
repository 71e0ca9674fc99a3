/*
 * legacy_oracle.h -- CPU restatement of the reference's voxel photon mapper
 * (photonMappingKernel.cu). TEST INFRASTRUCTURE ONLY: tests, the smoke
 * check and the benchmark's CPU-baseline leg use it as the checker.
 */
#ifndef PM_LEGACY_ORACLE_H
#define PM_LEGACY_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct pmo_legacy pmo_legacy;

pmo_legacy *pmo_legacy_create(void);
void pmo_legacy_destroy(pmo_legacy *s);
void pmo_legacy_reset(pmo_legacy *s);
void pmo_legacy_position_spheres(float animTime, float out[2][4]);
void pmo_legacy_init_random(pmo_legacy *s);
void pmo_legacy_emit(pmo_legacy *s, float animTime, int interp, int media);
void pmo_legacy_render(pmo_legacy *s, unsigned width, unsigned height, float animTime, int interp,
                       int media, unsigned char *rgba, float *rgb);
void pmo_legacy_get_grid(const pmo_legacy *s, float *out);
void pmo_legacy_set_grid(pmo_legacy *s, const float *in);
void pmo_legacy_get_table(const pmo_legacy *s, float *out);
void pmo_legacy_get_rng(const pmo_legacy *s, unsigned *out);

#ifdef __cplusplus
}
#endif
#endif
