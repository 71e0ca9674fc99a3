/*
 * physical_oracle.c -- CPU restatement of the physically based photon
 * mapper in single precision, operation for operation as the GPU kernels
 * compute it, so photon records, k-NN sets and pixel radiance can be
 * compared bit for bit.
 *
 * TEST INFRASTRUCTURE ONLY. Used by tests/, __graft_entry__.smoke() and the
 * benchmark's CPU-baseline leg as the checker; the product never calls it.
 *
 * Parity unpinned by the reference: the reference has no physically based
 * tracer, kd-tree or k-NN code (its only gather is a fixed voxel window,
 * photonMappingKernel.cu:314-389). This restatement follows the published
 * methods named in each function and shares only the scene layout with the
 * reference (float4 spheres, float2 axis planes, photonMappingKernel.cu:59-73).
 * It is pinned instead by known-answer tests (tests/test_physical_oracle.py)
 * and by the double-precision restatement in physical_oracle64.c.
 *
 * Build with -ffp-contract=off: one rounding per operation; fused
 * multiply-adds appear only where written as fmaf, as on the GPU.
 */
#include "physical_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "../include/pm_math.h"

typedef struct { float x, y, z; } v3;

static v3 mk(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 scl(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 nrm(v3 v) { float inv = 1.0f / sqrtf(dot3(v, v)); return scl(v, inv); }
static float vget(v3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
static void vset(v3 *v, int a, float s) { if (a == 0) v->x = s; else if (a == 1) v->y = s; else v->z = s; }

#define RAY_EPS 1e-4f
#define OFFSET 1e-4f
#define NONE 0x7fffffff

/* ---- scene ------------------------------------------------------------- */

typedef struct {
    const pmo_scene *s;
    const float *het;
    float sigma_max, inv_sigma_max, het_scale[3];
} scn;

static scn make_scn(const pmo_scene *s, const float *het) {
    scn c;
    c.s = s;
    c.het = het;
    c.sigma_max = (s->het_res > 0 ? s->het_max : s->sigma_s) + s->sigma_a;
    c.inv_sigma_max = c.sigma_max > 0.0f ? 1.0f / c.sigma_max : 0.0f;
    for (int a = 0; a < 3; ++a)
        c.het_scale[a] = s->het_res > 0 ? (float)s->het_res / (s->box_max[a] - s->box_min[a]) : 0.0f;
    return c;
}

typedef struct { float t; int obj; } hitr;

/* Nearest sphere or bounded wall hit with t in (RAY_EPS, tmax). */
static hitr intersect(const scn *S, v3 o, v3 d, float tmax) {
    const pmo_scene *s = S->s;
    hitr h;
    h.t = tmax;
    h.obj = NONE;
    for (int i = 0; i < s->num_spheres; ++i) {
        const float *sp = s->spheres[i];
        /* the GPU's sphere_t (phys_common.cuh): the same fused multiply-adds */
        const float ox = o.x - sp[0], oy = o.y - sp[1], oz = o.z - sp[2];
        float b = fmaf(oz, d.z, fmaf(oy, d.y, ox * d.x));
        float c = fmaf(oz, oz, fmaf(oy, oy, fmaf(ox, ox, -(sp[3] * sp[3]))));
        float disc = fmaf(b, b, -c);
        if (disc > 0.0f) {
            float sq = sqrtf(disc);
            float t = -b - sq;
            if (!(t > RAY_EPS)) t = -b + sq;
            if (t > RAY_EPS && t < h.t) { h.t = t; h.obj = i; }
        }
    }
    for (int i = 0; i < s->num_planes; ++i) {
        int a = (int)s->planes[i][0];
        float da = vget(d, a);
        if (da != 0.0f) {
            float t = (s->planes[i][1] - vget(o, a)) / da;
            if (t > RAY_EPS && t < h.t) {
                v3 p = add(o, scl(d, t));
                int a1 = a == 0 ? 1 : 0, a2 = a == 2 ? 1 : 2;
                float p1 = vget(p, a1), p2 = vget(p, a2);
                if (p1 >= s->box_min[a1] && p1 <= s->box_max[a1] && p2 >= s->box_min[a2] &&
                    p2 <= s->box_max[a2]) {
                    h.t = t;
                    h.obj = -1 - i;
                }
            }
        }
    }
    return h;
}

static float box_exit(const pmo_scene *s, v3 o, v3 d) {
    float t = 3.0e38f;
    for (int a = 0; a < 3; ++a) {
        float da = vget(d, a);
        if (da > 0.0f) t = fminf(t, (s->box_max[a] - vget(o, a)) / da);
        else if (da < 0.0f) t = fminf(t, (s->box_min[a] - vget(o, a)) / da);
    }
    return t;
}

static void box_span(const pmo_scene *s, v3 o, v3 d, float *t0, float *t1) {
    float lo = 0.0f, hi = 3.0e38f;
    for (int a = 0; a < 3; ++a) {
        float da = vget(d, a), oa = vget(o, a);
        if (da != 0.0f) {
            float ta = (s->box_min[a] - oa) / da, tb = (s->box_max[a] - oa) / da;
            lo = fmaxf(lo, fminf(ta, tb));
            hi = fminf(hi, fmaxf(ta, tb));
        } else if (oa < s->box_min[a] || oa > s->box_max[a]) {
            lo = 1.0f; hi = 0.0f;
        }
    }
    *t0 = lo;
    *t1 = hi;
}

static v3 outward_normal(const pmo_scene *s, int obj, v3 p) {
    if (obj >= 0) {
        const float *sp = s->spheres[obj];
        return nrm(mk(p.x - sp[0], p.y - sp[1], p.z - sp[2]));
    }
    v3 n = mk(0.0f, 0.0f, 0.0f);
    vset(&n, (int)s->planes[-1 - obj][0], 1.0f);
    return n;
}

static const pmo_material *mat_of(const pmo_scene *s, int obj) {
    return obj >= 0 ? &s->sphere_mat[obj] : &s->plane_mat[-1 - obj];
}

/* sigma_s at x: nearest voxel of the noise grid (x fastest). */
static float sigma_s_at(const scn *S, v3 x) {
    const pmo_scene *s = S->s;
    if (s->het_res <= 0) return s->sigma_s;
    int r = s->het_res, i[3];
    for (int a = 0; a < 3; ++a) {
        float f = (vget(x, a) - s->box_min[a]) * S->het_scale[a];
        int q = (int)f;
        i[a] = q < 0 ? 0 : (q >= r ? r - 1 : q);
    }
    return S->het[(i[2] * r + i[1]) * r + i[0]];
}

/* ---- sampling ------------------------------------------------------------ */

/* Duff et al., "Building an Orthonormal Basis, Revisited", JCGT 2017. */
static v3 from_local(v3 n, float x, float y, float z) {
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float bb = n.x * n.y * a;
    v3 t = mk(1.0f + sign * n.x * n.x * a, sign * bb, -sign * n.x);
    v3 b = mk(bb, sign + n.y * n.y * a, -n.y);
    return mk(t.x * x + b.x * y + n.x * z, t.y * x + b.y * y + n.y * z, t.z * x + b.z * y + n.z * z);
}

static v3 sample_sphere(float u1, float u2) {
    float z = 1.0f - 2.0f * u1;
    float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float s, c;
    pm_sincos2pi(u2, &s, &c);
    return mk(r * c, r * s, z);
}

static v3 sample_cosine(v3 n, float u1, float u2) {
    float r = sqrtf(u1);
    float s, c;
    pm_sincos2pi(u2, &s, &c);
    return nrm(from_local(n, r * c, r * s, sqrtf(fmaxf(0.0f, 1.0f - u1))));
}

/* Henyey and Greenstein 1941, inverted cumulative distribution. */
static v3 sample_hg(v3 d, float g, float u1, float u2) {
    float ct;
    if (fabsf(g) < 1e-3f) {
        ct = 1.0f - 2.0f * u1;
    } else {
        float sq = (1.0f - g * g) / (1.0f - g + 2.0f * g * u1);
        ct = (1.0f + g * g - sq * sq) / (2.0f * g);
    }
    ct = fminf(1.0f, fmaxf(-1.0f, ct));
    float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    float s, c;
    pm_sincos2pi(u2, &s, &c);
    return nrm(from_local(d, st * c, st * s, ct));
}

static float hg_phase(float g, float cos_t) {
    float den = 1.0f + g * g - 2.0f * g * cos_t;
    return (1.0f - g * g) / (12.566370614f * den * sqrtf(den));
}

static float fresnel(float ci, float eta, float *ct_out) {
    float s2 = eta * eta * (1.0f - ci * ci);
    if (s2 >= 1.0f) { *ct_out = 0.0f; return 1.0f; }
    float ct = sqrtf(1.0f - s2);
    float rs = (eta * ci - ct) / (eta * ci + ct);
    float rp = (ci - eta * ct) / (ci + eta * ct);
    *ct_out = ct;
    return 0.5f * (rs * rs + rp * rp);
}

static uint32_t oct_encode(v3 d) {
    float l1 = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    float px = d.x / l1, py = d.y / l1;
    if (d.z < 0.0f) {
        float qx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
        float qy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
        px = qx; py = qy;
    }
    int ix = (int)rintf(fminf(1.0f, fmaxf(-1.0f, px)) * 32767.0f);
    int iy = (int)rintf(fminf(1.0f, fmaxf(-1.0f, py)) * 32767.0f);
    return ((uint32_t)(ix & 0xFFFF)) | ((uint32_t)(iy & 0xFFFF) << 16);
}

static v3 oct_decode(uint32_t e) {
    float px = (float)(int16_t)(e & 0xFFFF) / 32767.0f;
    float py = (float)(int16_t)(e >> 16) / 32767.0f;
    float pz = 1.0f - fabsf(px) - fabsf(py);
    if (pz < 0.0f) {
        float qx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
        float qy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
        px = qx; py = qy;
    }
    return nrm(mk(px, py, pz));
}

static pm_u32x4 philox(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
    pm_u32x4 c;
    c.v[0] = c0; c.v[1] = c1; c.v[2] = c2; c.v[3] = c3;
    return pm_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

static float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* ---- photon paths (GPU: trace.cu) --------------------------------------- */

#define MAX_DELTA_STEPS 4096u

typedef struct {
    float (*spos)[4], (*spow)[4], (*vpos)[4], (*vpow)[4];  /* per-path slots (max_bounces each) */
} slots;

static void store(float (*pos)[4], float (*pw)[4], int k, v3 x, v3 thr, v3 d) {
    pos[k][0] = x.x; pos[k][1] = x.y; pos[k][2] = x.z; pos[k][3] = 0.0f;
    pw[k][0] = thr.x; pw[k][1] = thr.y; pw[k][2] = thr.z; pw[k][3] = u2f(oct_encode(d));
}

/* One photon path: emission from the point light (uniform sphere), then up
 * to max_bounces interactions -- free flight in the medium (homogeneous:
 * exponential distance; heterogeneous: delta tracking, Woodcock et al.
 * 1965), Henyey-Greenstein scattering, Lambertian diffuse bounce,
 * mirror reflection, Fresnel-weighted dielectric reflection/refraction, and
 * Russian roulette with survival probability rr at diffuse and medium
 * events. Records (position, direction, throughput) at every diffuse and
 * medium event. */
void pmo_trace_path(const pmo_scene *scene, const pmo_config *cfg, const float *het, uint32_t id,
                    float (*spos)[4], float (*spow)[4], uint32_t *ns_out, float (*vpos)[4],
                    float (*vpow)[4], uint32_t *nv_out) {
    scn S = make_scn(scene, het);
    const pmo_scene *s = scene;
    const int mb = cfg->max_bounces;
    const float rr = cfg->rr_survival;
    pm_u32x4 r0 = philox(cfg->seed, id, 0u, 0u, cfg->scene_id);
    v3 o = mk(s->light[0], s->light[1], s->light[2]);
    v3 d = sample_sphere(pm_u01(r0.v[0]), pm_u01(r0.v[1]));
    v3 thr = mk(1.0f, 1.0f, 1.0f);
    int glass = 0;
    uint32_t ns = 0, nv = 0;
    for (int ev = 1; ev <= mb; ++ev) {
        pm_u32x4 r = philox(cfg->seed, id, (uint32_t)ev, 0u, cfg->scene_id);
        float u0 = pm_u01(r.v[0]), u1 = pm_u01(r.v[1]), u2 = pm_u01(r.v[2]), u3 = pm_u01(r.v[3]);
        hitr h = intersect(&S, o, d, 3.0e38f);
        float seg = h.obj != NONE ? h.t : box_exit(s, o, d);
        int vol = 0;
        v3 x = o;
        float ss = 0.0f, st = 1.0f;
        if (S.sigma_max > 0.0f && !glass) {
            if (s->het_res <= 0) {
                st = s->sigma_s + s->sigma_a;
                if (s->sigma_s > 0.0f) {
                    float t = -pm_logf(1.0f - u0) / st;
                    if (t < seg) { vol = 1; x = add(o, scl(d, t)); ss = s->sigma_s; }
                }
            } else {
                float t = 0.0f;
                pm_u32x4 q;
                for (uint32_t j = 0; j < MAX_DELTA_STEPS; ++j) {
                    /* two tentative collisions per Philox block (GPU: trace.cu step_path) */
                    if ((j & 1u) == 0u) q = philox(cfg->seed, id, (uint32_t)ev, 1u + (j >> 1), cfg->scene_id);
                    const uint32_t ua = (j & 1u) ? q.v[2] : q.v[0], ub = (j & 1u) ? q.v[3] : q.v[1];
                    t += -pm_logf(1.0f - pm_u01(ua)) * S.inv_sigma_max;
                    if (!(t < seg)) break;
                    v3 y = add(o, scl(d, t));
                    float sv = sigma_s_at(&S, y);
                    float sty = sv + s->sigma_a;
                    if (pm_u01(ub) * S.sigma_max < sty) { vol = 1; x = y; ss = sv; st = sty; break; }
                }
            }
        }
        if (vol) {
            if (nv < (uint32_t)mb) store(vpos, vpow, (int)nv, x, thr, d);
            nv++;
            if (!(u1 < rr)) break;
            float f = (ss / st) / rr;
            thr = scl(thr, f);
            d = sample_hg(d, s->hg_g, u2, u3);
            o = x;
            continue;
        }
        if (h.obj == NONE) break;
        v3 hp = add(o, scl(d, h.t));
        v3 n = outward_normal(s, h.obj, hp);
        const pmo_material *m = mat_of(s, h.obj);
        float dn = dot3(n, d);
        v3 nf = dn < 0.0f ? n : scl(n, -1.0f);
        if (m->kind == PMO_MAT_DIFFUSE) {
            if (ns < (uint32_t)mb) store(spos, spow, (int)ns, hp, thr, d);
            ns++;
            if (!(u1 < rr)) break;
            thr = mk(thr.x * m->albedo[0] / rr, thr.y * m->albedo[1] / rr, thr.z * m->albedo[2] / rr);
            d = sample_cosine(nf, u2, u3);
            o = add(hp, scl(nf, OFFSET));
        } else if (m->kind == PMO_MAT_MIRROR) {
            d = nrm(sub(d, scl(n, 2.0f * dn)));
            o = add(hp, scl(nf, OFFSET));
        } else {
            float ci = -dn;
            int entering = ci > 0.0f;
            float eta = entering ? 1.0f / m->ior : m->ior;
            v3 nn = entering ? n : scl(n, -1.0f);
            ci = fabsf(ci);
            float ct;
            float F = fresnel(ci, eta, &ct);
            if (u1 < F) {
                d = nrm(add(d, scl(nn, 2.0f * ci)));
                o = add(hp, scl(nn, OFFSET));
            } else {
                d = nrm(add(scl(d, eta), scl(nn, eta * ci - ct)));
                o = sub(hp, scl(nn, OFFSET));
                glass = entering;
            }
        }
    }
    *ns_out = ns < (uint32_t)mb ? ns : (uint32_t)mb;
    *nv_out = nv < (uint32_t)mb ? nv : (uint32_t)mb;
}

/* Traces paths 0, 1, 2, ... until each map holds its target (or max_paths
 * paths are spent) and fills the maps exactly as the GPU's compaction does:
 * records in path order, truncated at the target, index in pos[3], power
 * scaled by light_power / (paths the map drew from). Paths are traced in
 * parallel rounds of PMO_EMIT_ROUND (each into its own slots) and merged in
 * path order, so the maps equal a serial run's. */
#define PMO_EMIT_ROUND 32768u
int pmo_emit(const pmo_scene *scene, const pmo_config *cfg, const float *het, float (*spos)[4],
             float (*spow)[4], float (*vpos)[4], float (*vpow)[4], uint32_t *sizes,
             uint32_t *paths) {
    const int mb = cfg->max_bounces > 0 ? cfg->max_bounces : 1;
    const size_t slots = (size_t)PMO_EMIT_ROUND * (size_t)mb;
    float(*a)[4] = malloc(sizeof(float) * 4 * slots);
    float(*b)[4] = malloc(sizeof(float) * 4 * slots);
    float(*c)[4] = malloc(sizeof(float) * 4 * slots);
    float(*e)[4] = malloc(sizeof(float) * 4 * slots);
    uint32_t *ncs = malloc(sizeof(uint32_t) * PMO_EMIT_ROUND);
    uint32_t *ncv = malloc(sizeof(uint32_t) * PMO_EMIT_ROUND);
    if (!a || !b || !c || !e || !ncs || !ncv) {
        free(a); free(b); free(c); free(e); free(ncs); free(ncv);
        return -1;
    }
    uint32_t targets[2] = {cfg->surface_photons, cfg->volume_photons};
    uint32_t n[2] = {0, 0}, np[2] = {0, 0};
    int done[2] = {targets[0] == 0, targets[1] == 0};
    uint32_t tmax = targets[0] > targets[1] ? targets[0] : targets[1];
    uint64_t cap64 = cfg->max_paths ? cfg->max_paths : (uint64_t)tmax * 16u;
    if (cap64 < 1024) cap64 = 1024;
    uint32_t cap = (uint32_t)cap64;
    for (uint32_t base = 0; base < cap && !(done[0] && done[1]); base += PMO_EMIT_ROUND) {
        const uint32_t m = cap - base < PMO_EMIT_ROUND ? cap - base : PMO_EMIT_ROUND;
#pragma omp parallel for schedule(dynamic, 256)
        for (long j = 0; j < (long)m; ++j)
            pmo_trace_path(scene, cfg, het, base + (uint32_t)j, a + (size_t)j * mb, b + (size_t)j * mb,
                           &ncs[j], c + (size_t)j * mb, e + (size_t)j * mb, &ncv[j]);
        for (uint32_t j = 0; j < m && !(done[0] && done[1]); ++j) {
            const uint32_t id = base + j;
            uint32_t cnt[2] = {ncs[j], ncv[j]};
            float(*src_pos[2])[4] = {a + (size_t)j * mb, c + (size_t)j * mb};
            float(*src_pow[2])[4] = {b + (size_t)j * mb, e + (size_t)j * mb};
            float(*dst_pos[2])[4] = {spos, vpos};
            float(*dst_pow[2])[4] = {spow, vpow};
            for (int mm = 0; mm < 2; ++mm) {
                if (done[mm]) continue;
                np[mm] = id + 1;
                for (uint32_t k = 0; k < cnt[mm] && n[mm] < targets[mm]; ++k) {
                    memcpy(dst_pos[mm][n[mm]], src_pos[mm][k], sizeof(float) * 4);
                    memcpy(dst_pow[mm][n[mm]], src_pow[mm][k], sizeof(float) * 4);
                    dst_pos[mm][n[mm]][3] = u2f(n[mm]);
                    n[mm]++;
                }
                if (n[mm] >= targets[mm]) done[mm] = 1;
            }
        }
    }
    for (int mm = 0; mm < 2; ++mm) {
        float(*pw)[4] = mm == 0 ? spow : vpow;
        float scale = scene->light_power / (float)np[mm];
        for (uint32_t i = 0; i < n[mm]; ++i) {
            pw[i][0] = pw[i][0] * scale;
            pw[i][1] = pw[i][1] * scale;
            pw[i][2] = pw[i][2] * scale;
        }
        sizes[mm] = n[mm];
        paths[mm] = np[mm];
    }
    free(a); free(b); free(c); free(e); free(ncs); free(ncv);
    return 0;
}

/* ---- exact k nearest neighbours (uniform grid of cell = radius) --------- */

struct pmo_grid {
    float lo[3], cell;
    int dim[3];
    uint32_t *start, *items;
    const float (*pos)[4];
    uint32_t n;
};

static int cell_of(const pmo_grid *g, int a, float v) {
    int c = (int)floorf((v - g->lo[a]) / g->cell);
    return c < 0 ? 0 : (c >= g->dim[a] ? g->dim[a] - 1 : c);
}

pmo_grid *pmo_grid_build(const float (*pos)[4], uint32_t n, float radius) {
    pmo_grid *g = calloc(1, sizeof(pmo_grid));
    float hi[3];
    for (int a = 0; a < 3; ++a) { g->lo[a] = 3.0e38f; hi[a] = -3.0e38f; }
    for (uint32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            g->lo[a] = fminf(g->lo[a], pos[i][a]);
            hi[a] = fmaxf(hi[a], pos[i][a]);
        }
    if (n == 0) for (int a = 0; a < 3; ++a) { g->lo[a] = 0.0f; hi[a] = 0.0f; }
    g->cell = radius;
    long total = 1;
    for (int a = 0; a < 3; ++a) {
        long d = (long)((hi[a] - g->lo[a]) / radius) + 1;
        if (d > 512) { d = 512; }
        g->dim[a] = (int)d;
        total *= d;
    }
    /* widen the cells when the box would need more than 512 per axis */
    for (int a = 0; a < 3; ++a) {
        float need = (hi[a] - g->lo[a]) / (float)g->dim[a];
        if (need > g->cell) g->cell = need * 1.0001f;
    }
    g->start = calloc((size_t)total + 1, sizeof(uint32_t));
    g->items = malloc(sizeof(uint32_t) * (n ? n : 1));
    g->pos = pos;
    g->n = n;
    for (uint32_t i = 0; i < n; ++i) {
        int c = (cell_of(g, 2, pos[i][2]) * g->dim[1] + cell_of(g, 1, pos[i][1])) * g->dim[0] + cell_of(g, 0, pos[i][0]);
        g->start[c + 1]++;
    }
    for (long c = 0; c < total; ++c) g->start[c + 1] += g->start[c];
    uint32_t *fill = calloc((size_t)total, sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) {
        int c = (cell_of(g, 2, pos[i][2]) * g->dim[1] + cell_of(g, 1, pos[i][1])) * g->dim[0] + cell_of(g, 0, pos[i][0]);
        g->items[g->start[c] + fill[c]++] = i;
    }
    free(fill);
    return g;
}

void pmo_grid_free(pmo_grid *g) {
    if (!g) return;
    free(g->start);
    free(g->items);
    free(g);
}

/* k smallest (d2, index) with d2 <= r2, ascending; returns the count.
 * d2 = (p.x-q.x)^2 + (p.y-q.y)^2 + (p.z-q.z)^2 in single precision. */
int pmo_grid_knn(const pmo_grid *g, const float q[3], int k, float r2, uint64_t *keys) {
    int cnt = 0;
    float r = sqrtf(r2);
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = cell_of(g, a, q[a] - r) - 1;
        hi[a] = cell_of(g, a, q[a] + r) + 1;
        if (lo[a] < 0) lo[a] = 0;
        if (hi[a] >= g->dim[a]) hi[a] = g->dim[a] - 1;
    }
    for (int z = lo[2]; z <= hi[2]; ++z)
        for (int y = lo[1]; y <= hi[1]; ++y)
            for (int x = lo[0]; x <= hi[0]; ++x) {
                int c = (z * g->dim[1] + y) * g->dim[0] + x;
                for (uint32_t it = g->start[c]; it < g->start[c + 1]; ++it) {
                    uint32_t i = g->items[it];
                    const float *p = g->pos[i];
                    float dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
                    float d2 = dx * dx + dy * dy + dz * dz;
                    if (!(d2 <= r2)) continue;
                    uint64_t key = ((uint64_t)f2u(d2) << 32) | f2u(p[3]);
                    if (cnt == k && key >= keys[k - 1]) continue;
                    int j = cnt < k ? cnt++ : k - 1;
                    while (j > 0 && keys[j - 1] > key) { keys[j] = keys[j - 1]; --j; }
                    keys[j] = key;
                }
            }
    return cnt;
}

void pmo_knn(const float (*pos)[4], uint32_t n, const float (*queries)[4], uint32_t nq, int k,
             float radius, uint32_t *idx_out, float *d2_out) {
    float r2 = radius * radius;
    pmo_grid *g = pmo_grid_build(pos, n, radius);
#pragma omp parallel for schedule(dynamic, 64)
    for (long qi = 0; qi < (long)nq; ++qi) {
        uint64_t keys[128];
        int c = pmo_grid_knn(g, queries[qi], k, r2, keys);
        for (int j = 0; j < k; ++j) {
            idx_out[qi * k + j] = j < c ? (uint32_t)keys[j] : 0xffffffffu;
            d2_out[qi * k + j] = j < c ? u2f((uint32_t)(keys[j] >> 32)) : r2;
        }
    }
    pmo_grid_free(g);
}

/* ---- radiance estimate (GPU: gather.cu flux_sum) ------------------------ */

/* Order-independent sum of non-negative float terms (GPU: knn_core.cuh
 * warp_fixed_sum). With E the largest exponent field of the terms (at least
 * 1), each term becomes floor(t * 2^(182 - E)): its 24-bit significand
 * shifted left by 32 - (E - e) bits, or right (truncating) when that is
 * negative. The integers add exactly in 64 bits and the total times
 * 2^(E - 182) is rounded to float once (nearest even); the power-of-two
 * scale is split in two steps when it is below 2^-126. */
static float scale_pow2(float f, int n) {
    if (n < -126) {
        f *= u2f((uint32_t)(127 - 64) << 23);
        n += 64;
    }
    return f * u2f((uint32_t)(n + 127) << 23);
}

static float fixed_sum(const float *t, int n) {
    uint32_t emax = 1;
    for (int i = 0; i < n; ++i) {
        const uint32_t e = f2u(t[i]) >> 23;
        if (e > emax) emax = e;
    }
    uint64_t acc = 0;
    for (int i = 0; i < n; ++i) {
        const uint32_t b = f2u(t[i]);
        const uint32_t e = b >> 23;
        const uint32_t m = (b & 0x7fffffu) | (e ? 0x800000u : 0u);
        const int sh = 32 - (int)(emax - (e ? e : 1u));
        if (sh >= 0) acc += (uint64_t)m << sh;
        else if (sh > -24) acc += (uint64_t)(m >> -sh);
    }
    return scale_pow2((float)acc, (int)emax - 182);
}

float pmo_fixed_sum(const float *t, int n) { return fixed_sum(t, n); }

static v3 flux_sum(const uint64_t *keys, int cnt, int k, const float (*pow)[4], int mode, v3 dirv,
                   float g, float r2cap, int *found, float *r2) {
    float tx[128], ty[128], tz[128];
    const int n = cnt < k ? cnt : k;
    for (int j = 0; j < n; ++j) {
        const float *pw = pow[(uint32_t)keys[j]];
        v3 dir = oct_decode(f2u(pw[3]));
        float w;
        if (mode == 0) w = dot3(dirv, dir) < 0.0f ? 1.0f : 0.0f;
        else w = hg_phase(g, dot3(dir, dirv));
        tx[j] = pw[0] * w;
        ty[j] = pw[1] * w;
        tz[j] = pw[2] * w;
    }
    *found = cnt;
    *r2 = cnt == k ? u2f((uint32_t)(keys[k - 1] >> 32)) : r2cap;
    return mk(fixed_sum(tx, n), fixed_sum(ty, n), fixed_sum(tz, n));
}

/* ---- render (GPU: gather.cu render_kernel) ------------------------------ */

#define MAX_SPECULAR 8
#define EYE_SALT 0xE7E5A17Bu

typedef struct {
    const pmo_scene *s;
    const pmo_config *c;
    scn S;
    const float (*spos)[4], (*spow)[4], (*vpos)[4], (*vpow)[4];
    uint32_t ns, nv;
    pmo_grid *gs, *gv;  /* neighbour grids, or */
    pmo_kd *ks, *kv;    /* kd-trees (pmo_set_gather_index) */
} render_ctx;

static int g_gather_index = PMO_GATHER_KDTREE;

void pmo_set_gather_index(int which) { g_gather_index = which; }

static int render_knn(const render_ctx *R, int vol, const float q[3], int k, float r2, uint64_t *keys) {
    if (vol) return R->kv ? pmo_kd_knn(R->kv, q, k, r2, keys) : pmo_grid_knn(R->gv, q, k, r2, keys);
    return R->ks ? pmo_kd_knn(R->ks, q, k, r2, keys) : pmo_grid_knn(R->gs, q, k, r2, keys);
}

static v3 shade(const render_ctx *R, uint32_t pix, uint64_t *counts) {
    const pmo_scene *s = R->s;
    const pmo_config *c = R->c;
    const float aspect = c->height > 0 ? (float)c->width / (float)c->height : 1.0f;
    const float r2cap = c->radius * c->radius;
    uint32_t px = pix % (uint32_t)c->width, py = pix / (uint32_t)c->width;
    float u = ((float)px / (float)c->width - 0.5f) * aspect;
    float v = -((float)py / (float)c->height - 0.5f);
    v3 o = mk(s->cam_pos[0], s->cam_pos[1], s->cam_pos[2]);
    v3 d = nrm(mk(u, v, s->focal));
    v3 L = mk(0.0f, 0.0f, 0.0f);
    float tau = 0.0f;
    int glass = 0;
    uint64_t keys[128];
    for (int depth = 0; depth < MAX_SPECULAR; ++depth) {
        hitr h = intersect(&R->S, o, d, 3.0e38f);
        float tend = h.obj != NONE ? h.t : 3.0e38f;
        if (c->march_step > 0.0f && R->S.sigma_max > 0.0f && !glass) {
            float t0, t1;
            box_span(s, o, d, &t0, &t1);
            t1 = fminf(t1, tend);
            if (t0 < t1) {
                int nst = (int)fminf(ceilf((t1 - t0) / c->march_step), 65536.0f);
                v3 wo = scl(d, -1.0f);
                for (int j = 0; j < nst; ++j) {
                    float ta = t0 + (float)j * c->march_step;
                    float tb = fminf(t0 + (float)(j + 1) * c->march_step, t1);
                    float dt = tb - ta;
                    float tm = 0.5f * (ta + tb);
                    v3 x = add(o, scl(d, tm));
                    float ss = s->het_res > 0 ? sigma_s_at(&R->S, x) : s->sigma_s;
                    float st = ss + s->sigma_a;
                    float tau_mid = tau + st * (0.5f * dt);
                    if (R->nv > 0) {
                        float q[3] = {x.x, x.y, x.z};
                        int cnt = render_knn(R, 1, q, c->k, r2cap, keys);
                        int found;
                        float r2;
                        v3 e = flux_sum(keys, cnt, c->k, R->vpow, 1, wo, s->hg_g, r2cap, &found, &r2);
                        counts[1]++;
                        if (found > 0) {
                            float scale = pm_expf(-tau_mid) * dt * (1.0f / (4.18879020f * r2 * sqrtf(r2)));
                            L = add(L, scl(e, scale));
                        }
                    }
                    tau = tau + st * dt;
                }
            }
        }
        if (h.obj == NONE) break;
        v3 hp = add(o, scl(d, h.t));
        v3 n = outward_normal(s, h.obj, hp);
        const pmo_material *m = mat_of(s, h.obj);
        float dn = dot3(n, d);
        v3 nf = dn < 0.0f ? n : scl(n, -1.0f);
        if (m->kind == PMO_MAT_DIFFUSE) {
            if (R->ns > 0) {
                float q[3] = {hp.x, hp.y, hp.z};
                int cnt = render_knn(R, 0, q, c->k, r2cap, keys);
                int found;
                float r2;
                v3 e = flux_sum(keys, cnt, c->k, R->spow, 0, nf, 0.0f, r2cap, &found, &r2);
                counts[0]++;
                if (found > 0) {
                    float scale = pm_expf(-tau) * (1.0f / (3.14159265f * r2)) * 0.318309886f;
                    L = add(L, mk(m->albedo[0] * (e.x * scale), m->albedo[1] * (e.y * scale),
                                  m->albedo[2] * (e.z * scale)));
                }
            }
            break;
        }
        if (m->kind == PMO_MAT_MIRROR) {
            d = nrm(sub(d, scl(n, 2.0f * dn)));
            o = add(hp, scl(nf, OFFSET));
        } else {
            float ci = -dn;
            int entering = ci > 0.0f;
            float eta = entering ? 1.0f / m->ior : m->ior;
            v3 nn = entering ? n : scl(n, -1.0f);
            ci = fabsf(ci);
            float ct;
            float F = fresnel(ci, eta, &ct);
            pm_u32x4 r = philox(c->seed, pix, (uint32_t)depth, EYE_SALT, c->scene_id);
            if (pm_u01(r.v[0]) < F) {
                d = nrm(add(d, scl(nn, 2.0f * ci)));
                o = add(hp, scl(nn, OFFSET));
            } else {
                d = nrm(add(scl(d, eta), scl(nn, eta * ci - ct)));
                o = sub(hp, scl(nn, OFFSET));
                glass = entering;
            }
        }
    }
    return L;
}

void pmo_render(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                const float (*spos)[4], const float (*spow)[4], uint32_t ns,
                const float (*vpos)[4], const float (*vpow)[4], uint32_t nv,
                const uint32_t *pixels, uint32_t npix, float (*out)[4], uint64_t *gathers) {
    pmo_render_timed(scene, cfg, het, spos, spow, ns, vpos, vpow, nv, pixels, npix, out, gathers, NULL);
}

struct pmo_render_ctx {
    render_ctx R;
    pmo_scene scene;
    pmo_config cfg;
};

pmo_render_ctx *pmo_render_create(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                                  const float (*spos)[4], const float (*spow)[4], uint32_t ns,
                                  const float (*vpos)[4], const float (*vpow)[4], uint32_t nv) {
    pmo_render_ctx *x = calloc(1, sizeof(pmo_render_ctx));
    if (!x) return NULL;
    x->scene = *scene;
    x->cfg = *cfg;
    render_ctx *R = &x->R;
    R->s = &x->scene;
    R->c = &x->cfg;
    R->S = make_scn(&x->scene, het);
    R->spos = spos; R->spow = spow; R->vpos = vpos; R->vpow = vpow;
    R->ns = ns; R->nv = nv;
    if (g_gather_index == PMO_GATHER_KDTREE) {
        R->ks = pmo_kd_build(spos, ns);
        R->kv = pmo_kd_build(vpos, nv);
    } else {
        R->gs = pmo_grid_build(spos, ns, cfg->radius);
        R->gv = pmo_grid_build(vpos, nv, cfg->radius);
    }
    return x;
}

void pmo_render_pixels(const pmo_render_ctx *x, const uint32_t *pixels, uint32_t npix,
                       float (*out)[4], uint64_t *gathers) {
    uint64_t total[2] = {0, 0};
#pragma omp parallel
    {
        uint64_t local[2] = {0, 0};
#pragma omp for schedule(dynamic, 16)
        for (long i = 0; i < (long)npix; ++i) {
            v3 L = shade(&x->R, pixels[i], local);
            out[i][0] = L.x; out[i][1] = L.y; out[i][2] = L.z; out[i][3] = 1.0f;
        }
#pragma omp critical
        { total[0] += local[0]; total[1] += local[1]; }
    }
    if (gathers) { gathers[0] = total[0]; gathers[1] = total[1]; }
}

void pmo_render_free(pmo_render_ctx *x) {
    if (!x) return;
    pmo_grid_free(x->R.gs);
    pmo_grid_free(x->R.gv);
    pmo_kd_free(x->R.ks);
    pmo_kd_free(x->R.kv);
    free(x);
}

void pmo_render_timed(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                      const float (*spos)[4], const float (*spow)[4], uint32_t ns,
                      const float (*vpos)[4], const float (*vpow)[4], uint32_t nv,
                      const uint32_t *pixels, uint32_t npix, float (*out)[4], uint64_t *gathers,
                      double *seconds) {
    double t0 = omp_get_wtime();
    pmo_render_ctx *x = pmo_render_create(scene, cfg, het, spos, spow, ns, vpos, vpow, nv);
    double t1 = omp_get_wtime();
    pmo_render_pixels(x, pixels, npix, out, gathers);
    if (seconds) { seconds[0] = t1 - t0; seconds[1] = omp_get_wtime() - t1; }
    pmo_render_free(x);
}

uint64_t pmo_trace_sample(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                          uint32_t first, uint32_t count) {
    const int mb = cfg->max_bounces > 0 ? cfg->max_bounces : 1;
    uint64_t records = 0;
#pragma omp parallel reduction(+ : records)
    {
        float(*a)[4] = malloc(sizeof(float) * 4 * mb);
        float(*b)[4] = malloc(sizeof(float) * 4 * mb);
        float(*c)[4] = malloc(sizeof(float) * 4 * mb);
        float(*e)[4] = malloc(sizeof(float) * 4 * mb);
#pragma omp for schedule(dynamic, 256)
        for (long j = 0; j < (long)count; ++j) {
            uint32_t cs = 0, cv = 0;
            if (a && b && c && e) pmo_trace_path(scene, cfg, het, first + (uint32_t)j, a, b, &cs, c, e, &cv);
            records += cs + cv;
        }
        free(a); free(b); free(c); free(e);
    }
    return records;
}

/* Value-noise grid of the heterogeneous medium (GPU: scene.cu). */
static float lattice(uint64_t seed, uint32_t oct, uint32_t i, uint32_t j, uint32_t k) {
    pm_u32x4 r = philox(seed, i, j, k, 0x4E015E00u + oct);
    return pm_u01(r.v[0]);
}

static float value_noise(uint64_t seed, uint32_t oct, int lat, float x, float y, float z) {
    float fx = x * lat, fy = y * lat, fz = z * lat;
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    if (ix > lat - 1) ix = lat - 1;
    if (iy > lat - 1) iy = lat - 1;
    if (iz > lat - 1) iz = lat - 1;
    float tx = fx - ix, ty = fy - iy, tz = fz - iz;
    float c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int e = 0; e < 2; ++e) c[a][b][e] = lattice(seed, oct, ix + a, iy + b, iz + e);
    float x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * tx;
    float x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * tx;
    float x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * tx;
    float x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * tx;
    float y0 = x00 + (x10 - x00) * ty, y1 = x01 + (x11 - x01) * ty;
    return y0 + (y1 - y0) * tz;
}

void pmo_noise_grid(float *grid, int res, uint64_t seed, float lo, float hi) {
    for (int v = 0; v < res * res * res; ++v) {
        int x = v % res, y = (v / res) % res, z = v / (res * res);
        float px = (x + 0.5f) / res, py = (y + 0.5f) / res, pz = (z + 0.5f) / res;
        float n = 0.6666667f * value_noise(seed, 0, 8, px, py, pz) +
                  0.3333333f * value_noise(seed, 1, 16, px, py, pz);
        grid[v] = lo + (hi - lo) * n;
    }
}

void pmo_philox(uint64_t seed, const uint32_t *ctr, uint32_t *out) {
    pm_u32x4 r = philox(seed, ctr[0], ctr[1], ctr[2], ctr[3]);
    memcpy(out, r.v, 16);
}

float pmo_logf(float x) { return pm_logf(x); }
float pmo_expf(float x) { return pm_expf(x); }
void pmo_sincos2pi(float u, float *s, float *c) { pm_sincos2pi(u, s, c); }
uint32_t pmo_oct_encode(const float *d) { return oct_encode(mk(d[0], d[1], d[2])); }
void pmo_oct_decode(uint32_t e, float *d) { v3 v = oct_decode(e); d[0] = v.x; d[1] = v.y; d[2] = v.z; }
size_t pmo_sizeof_scene(void) { return sizeof(pmo_scene); }
size_t pmo_sizeof_config(void) { return sizeof(pmo_config); }

/* Samplers exposed for distribution tests. */
void pmo_sample(int which, const float *dir, float g, float u1, float u2, float *out) {
    v3 r;
    if (which == 0) r = sample_sphere(u1, u2);
    else if (which == 1) r = sample_cosine(mk(dir[0], dir[1], dir[2]), u1, u2);
    else r = sample_hg(mk(dir[0], dir[1], dir[2]), g, u1, u2);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

float pmo_fresnel(float ci, float eta) {
    float ct;
    return fresnel(ci, eta, &ct);
}

float pmo_hg_phase(float g, float c) { return hg_phase(g, c); }
