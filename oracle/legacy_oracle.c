/*
 * legacy_oracle.c -- CPU restatement of the reference's voxel photon mapper
 * (photonMappingKernel.cu), used as the parity oracle for the product's
 * legacy-mode kernels.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load the library built from this file; the
 * product never calls it.
 *
 * Pinning: tests/test_oracle_golden.py checks this restatement bit for bit
 * against golden vectors produced by the reference's own code
 * (oracle/ref.mk + tests/golden/make_golden.py).
 *
 * Semantics restated here, each from the cited reference lines:
 *  - serial photon order: photon 0 runs to completion, then photon 1, ...;
 *    this fixes the order of the grid's `+=` and of the shared generator;
 *  - IEEE single precision with one rounding per operation (build with
 *    -ffp-contract=off), and double precision exactly where the reference's
 *    double literals promote an expression;
 *  - vector helpers as the reference's cutil host path defines them
 *    (scalar division as multiplication by 1.0f/s, normalize as
 *    v * (1.0f/sqrtf(dot(v,v)))).
 */
#include "legacy_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define G 32                 /* NR_PHOTONS_X/Y/Z, photonMappingKernel.cu:15-17 */
#define N_PHOTONS 10000      /* nrPhotons, :28 */
#define N_CAUSTIC 100        /* CAUSTICS_PHOTONS, :13 */
#define N_BOUNCES 5          /* nrBounces, :80 */

typedef struct { float x, y, z; } v3;

struct pmo_legacy {
    unsigned rng_z, rng_w;         /* m_z, m_w (:1026-1027) */
    v3 table[N_PHOTONS];           /* randomNumbers (:78) */
    v3 grid[G][G][G];              /* photons (:76) */
    float sph[2][4];               /* the two traced spheres (:61,66) */
};

/* ---- vector helpers (cutil host-path semantics) ------------------------ */
static v3 mk(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 scl(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static v3 subs(v3 a, float s) { return mk(a.x - s, a.y - s, a.z - s); }
static v3 divs(v3 a, float s) { float inv = 1.0f / s; return scl(a, inv); }
static float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 nrm(v3 v) { float inv = 1.0f / sqrtf(dot3(v, v)); return scl(v, inv); }
static float comp(v3 v, int axis) { return axis == 0 ? v.x : (axis == 1 ? v.y : v.z); }

/* Double-to-int conversion as the GPU performs it: NaN -> 0, saturating. */
static int d2i(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return 2147483647;
    if (v <= -2147483648.0) return (-2147483647 - 1);
    return (int)v;
}

/* ---- scene (:58-73) ---------------------------------------------------- */
static const int kPlaneAxis[5] = {0, 1, 0, 1, 2};
static const float kPlaneOff[5] = {1.5f, -1.5f, -1.5f, 1.5f, 6.0f};
static v3 light_pos(void) { return mk(0.0f, 1.4f, 3.5f); }

/* positionObjects (:1380-1404), with the host's libm. */
void pmo_legacy_position_spheres(float animTime, float out[2][4]) {
    out[0][0] = (float)(1.0 * (double)cosf(animTime));
    out[0][1] = (float)(0.5 * sin(2.0 * (double)animTime));
    out[0][2] = (float)((double)sinf(animTime) + 3.5);
    out[0][3] = 0.4f;
    out[1][0] = 0.0f;
    out[1][1] = (float)(sin(0.5 * (double)animTime + 5.0) - 0.25);
    out[1][2] = 3.5f;
    out[1][3] = 0.4f;
}

/* ---- Marsaglia multiply-with-carry generator (:1026-1051) -------------- */
static unsigned mwc_next(pmo_legacy *s) {
    s->rng_z = 36969u * (s->rng_z & 65535u) + (s->rng_z >> 16);
    s->rng_w = 18000u * (s->rng_w & 65535u) + (s->rng_w >> 16);
    return (s->rng_z << 16) + s->rng_w;
}

/* randFloat (:1038-1051): uniform-ish value in [-max, max] scaled by 32768. */
static float rand_float(pmo_legacy *s, float max) {
    unsigned u = mwc_next(s);
    float r = (float)(int)u / 65535.0f;
    r = (r * 2.0f) * max;
    return r - max;
}

/* ---- intersection (:100-165, 223-241) ---------------------------------- */
typedef struct { float dist; int type, idx, hit; } hitrec;

static void consider(hitrec *h, float t, int type, int idx) {   /* checkDistance :100-103 */
    if (t < h->dist && t > 0.0f) { h->type = type; h->idx = idx; h->dist = t; h->hit = 1; }
}

static void trace(const pmo_legacy *s, v3 r, v3 o, hitrec *h) {   /* raytrace :223-241 */
    h->hit = 0;
    h->dist = 999999.9f;
    for (int i = 0; i < 2; ++i) {                                    /* raySphere :105-126 */
        v3 sc = sub(mk(s->sph[i][0], s->sph[i][1], s->sph[i][2]), o);
        float rad = s->sph[i][3];
        float A = dot3(r, r);
        float B = (float)(-2.0 * (double)dot3(sc, r));
        float C = dot3(sc, sc) - rad * rad;
        float D = B * B - (4.0f * A) * C;
        if (D > 0.0f) {
            float sign = ((double)C < -0.00001) ? 1.0f : -1.0f;
            consider(h, (-B + sign * sqrtf(D)) / (2.0f * A), 0, i);
        }
    }
    for (int i = 0; i < 5; ++i) {                                    /* rayPlane :130-157 */
        float ra = comp(r, kPlaneAxis[i]);
        if (ra != 0.0f) consider(h, (kPlaneOff[i] - comp(o, kPlaneAxis[i])) / ra, 1, i);
    }
}

/* surfaceNormal (:178-201): a sphere's outward normal, or an axis-aligned
 * plane's normal pointing toward `from`. */
static v3 normal_at(const pmo_legacy *s, int type, int idx, v3 p, v3 from) {
    if (type == 0) return nrm(sub(p, mk(s->sph[idx][0], s->sph[idx][1], s->sph[idx][2])));
    v3 n = mk(0.0f, 0.0f, 0.0f);
    float d = comp(from, kPlaneAxis[idx]) - kPlaneOff[idx];
    if (kPlaneAxis[idx] == 0) n.x = d; else if (kPlaneAxis[idx] == 1) n.y = d; else n.z = d;
    return nrm(n);
}

/* reflect3 (:663-668) with factor 1. */
static v3 reflect_ray(const pmo_legacy *s, v3 ray, v3 from, int type, int idx, v3 p) {
    v3 n = scl(normal_at(s, type, idx, p, from), 1.0f);
    return nrm(sub(ray, scl(n, 2.0f * dot3(ray, n))));
}

/* refract3 (:620-659): entering (factor 1, n = 1/1.3) or leaving (factor -1, n = 1). */
static v3 refract_ray(const pmo_legacy *s, v3 ray, int type, int idx, v3 p, float factor) {
    v3 n = scl(normal_at(s, type, idx, p, p), factor);
    float eta = 1.0f / 1.3f;
    if (factor == -1.0f) eta = 1.0f;
    float cos_i = -dot3(n, ray);
    float cos_t2 = (float)(1.0 - (double)(eta * eta) * (1.0 - (double)(cos_i * cos_i)));
    if (cos_t2 > 0.0f) return add(scl(ray, eta), scl(n, eta * cos_i - sqrtf(cos_t2)));
    return mk(0.0f, 0.0f, 0.0f);
}

/* ---- specular chains (:673-827) ----------------------------------------
 * The reference unrolls recursion into handleReflection{,2,3,4} and
 * handleRefraction{,2,3,4}. Numbering those stages 1..8 in call order
 * (Reflection = 1,3,5,7; Refraction = 2,4,6,8), a reflection stage moves on
 * to the next stage when it lands on the glass sphere, a refraction stage
 * when its exit ray lands on the mirror sphere; stage 8 ends the chain. */
typedef struct { v3 ray, point; hitrec h; } chainstate;

static int stage_reflect(const pmo_legacy *s, chainstate *c, v3 from) {
    c->ray = reflect_ray(s, c->ray, from, c->h.type, c->h.idx, c->point);
    trace(s, c->ray, c->point, &c->h);
    if (!c->h.hit) return 0;
    c->point = add(scl(c->ray, c->h.dist), c->point);
    return c->h.type == 0 && c->h.idx == 0;
}

static int stage_refract(const pmo_legacy *s, chainstate *c) {
    c->ray = refract_ray(s, c->ray, c->h.type, c->h.idx, c->point, 1.0f);
    c->point = add(scl(c->ray, 0.00001f), c->point);
    trace(s, c->ray, c->point, &c->h);
    c->point = add(scl(c->ray, c->h.dist), c->point);
    if (!(c->h.hit && c->h.type == 0 && c->h.idx == 0)) return 0;
    c->ray = refract_ray(s, c->ray, c->h.type, c->h.idx, c->point, -1.0f);
    c->point = add(scl(c->ray, 0.00001f), c->point);
    trace(s, c->ray, c->point, &c->h);
    c->point = add(scl(c->ray, c->h.dist), c->point);
    return c->h.type == 0 && c->h.idx == 1;
}

static void run_chain(const pmo_legacy *s, chainstate *c, int first_stage, v3 from) {
    for (int st = first_stage; st <= 8; ++st) {
        int more = (st & 1) ? stage_reflect(s, c, from) : stage_refract(s, c);
        if (!more) break;
    }
}

/* ---- voxel helpers (:254-268, 392-439) --------------------------------- */
typedef struct { int x, y, z; } i3;

static i3 voxel_of(v3 p) {                                          /* getVoxelCoordinates */
    i3 v;
    v.x = d2i((((double)p.x + 1.5) / 3.0) * 32.0);
    v.y = d2i((((double)p.y + 1.5) / 3.0) * 32.0);
    v.z = d2i(((double)p.z / 6.0) * 32.0);
    return v;
}

static v3 voxel_corner(i3 v) {                                      /* getWorldCoordinates */
    return mk((float)((double)((float)v.x / 32.0f) * 3.0 - 1.5),
              (float)((double)((float)v.y / 32.0f) * 3.0 - 1.5),
              (float)((double)((float)v.z / 32.0f) * 6.0));
}

static v3 voxel_center(v3 p) {                                      /* centerPoint */
    v3 c = voxel_corner(voxel_of(p));
    return add(c, mk(0.046875f, 0.046875f, 0.09375f));
}

static const float kVoxDim[3] = {0.09375f, 0.09375f, 0.1875f};    /* getVoxelDim */

static float alpha_of(v3 p, v3 a, v3 b, int axis) {                 /* getAlpha */
    int ax = axis == 0 ? 0 : (axis == 1 ? 1 : 2);
    return (comp(p, ax) - comp(a, ax)) / (comp(b, ax) - comp(a, ax));
}

static v3 lerp3(v3 a, v3 b, float t) {                              /* interpolate3f */
    return add(scl(a, (float)(1.0 - (double)t)), scl(b, t));
}

static int lo_edge(int c, int r, int lo) { return (c - r >= lo) ? c - r : lo; }
static int hi_edge(int c, int r, int hi) { return (c + r <= hi) ? c + r : hi; }

/* integrate (:314-389): sum of a <=6x6 window of the wall slab the plane
 * `id` lies on, times ENERGY_WEIGHT. Spheres gather nothing. */
static v3 integrate_slab(const pmo_legacy *s, v3 e, i3 wp, int type, int id) {
    v3 acc = e;
    if (type != 1) return acc;
    int x0 = lo_edge(wp.x, 3, 0), y0 = lo_edge(wp.y, 3, 0), z0 = lo_edge(wp.z, 3, 0);
    int x1 = hi_edge(wp.x, 3, G), y1 = hi_edge(wp.y, 3, G), z1 = hi_edge(wp.z, 3, G);
    if (id == 0 || id == 2) {
        int i = id == 0 ? G - 1 : 0;
        for (int j = y0; j < y1; ++j)
            for (int k = z0; k < z1; ++k) acc = add(acc, scl(s->grid[i][j][k], 0.0005f));
    } else if (id == 1 || id == 3) {
        int j = id == 1 ? 0 : G - 1;
        for (int i = x0; i < x1; ++i)
            for (int k = z0; k < z1; ++k) acc = add(acc, scl(s->grid[i][j][k], 0.0005f));
    } else if (id == 4) {
        int k = G - 1;
        for (int i = x0; i < x1; ++i)
            for (int j = y0; j < y1; ++j) acc = add(acc, scl(s->grid[i][j][k], 0.0005f));
    }
    return acc;
}

/* bilinearInterpolate (:442-471). */
static v3 bilinear(const pmo_legacy *s, v3 p, v3 p1, v3 p2, v3 p3, v3 p4, v3 e, int type, int id,
                   int ax1, int ax2) {
    v3 c1 = integrate_slab(s, e, voxel_of(p1), type, id);
    v3 c2 = integrate_slab(s, e, voxel_of(p2), type, id);
    v3 c3 = integrate_slab(s, e, voxel_of(p3), type, id);
    v3 c4 = integrate_slab(s, e, voxel_of(p4), type, id);
    float a = alpha_of(p, p1, p2, ax1);
    v3 p12 = lerp3(p1, p2, a), c12 = lerp3(c1, c2, a);
    a = alpha_of(p, p3, p4, ax1);
    v3 p34 = lerp3(p3, p4, a), c34 = lerp3(c3, c4, a);
    a = alpha_of(p, p12, p34, ax2);
    return lerp3(c12, c34, a);
}

/* Sets component `axis` of the three neighbour points: the first two step
 * across the cell along `axis` when `along_first`, otherwise the last two. */
static void set_axis(v3 *q, int axis, float v) {
    if (axis == 0) q->x = v; else if (axis == 1) q->y = v; else q->z = v;
}

/* interpolateEnergy (:475-583): four slab windows around the voxel centre,
 * blended bilinearly. The first listed axis steps p2,p3; the second p3,p4. */
static v3 interpolate_slab(const pmo_legacy *s, v3 p, v3 e, int type, int id) {
    if (type != 1) return e;
    int a1, a2;
    if (id == 0 || id == 2) { a1 = 2; a2 = 1; }
    else if (id == 1 || id == 3) { a1 = 0; a2 = 2; }
    else if (id == 4) { a1 = 0; a2 = 1; }
    else return e;
    v3 p1 = voxel_center(p);
    v3 p2 = mk(0.0f, 0.0f, 0.0f), p3 = p2, p4 = p2;
    float c1 = comp(p1, a1), d1 = kVoxDim[a1];
    float s1 = comp(p, a1) > c1 ? c1 + d1 : c1 - d1;
    set_axis(&p2, a1, s1); set_axis(&p3, a1, s1); set_axis(&p4, a1, c1);
    float c2 = comp(p1, a2), d2 = kVoxDim[a2];
    float s2 = comp(p, a2) > c2 ? c2 + d2 : c2 - d2;
    set_axis(&p2, a2, c2); set_axis(&p3, a2, s2); set_axis(&p4, a2, s2);
    return bilinear(s, p, p1, p2, p3, p4, e, type, id, a1, a2);
}

/* integrateVolumePhotons (:831-870): plain sum of a <=6x6x6 window,
 * clamped to [1,31). */
static v3 integrate_volume(const pmo_legacy *s, v3 p) {
    v3 acc = mk(0.0f, 0.0f, 0.0f);
    i3 wp = voxel_of(p);
    int x0 = lo_edge(wp.x, 3, 1), y0 = lo_edge(wp.y, 3, 1), z0 = lo_edge(wp.z, 3, 1);
    int x1 = hi_edge(wp.x, 3, G - 1), y1 = hi_edge(wp.y, 3, G - 1), z1 = hi_edge(wp.z, 3, G - 1);
    for (int i = x0; i < x1; ++i)
        for (int j = y0; j < y1; ++j)
            for (int k = z0; k < z1; ++k) acc = add(acc, s->grid[i][j][k]);
    return acc;
}

/* ---- photon deposit (:1059-1183) --------------------------------------- */
static i3 clamp_voxel(i3 v) {
    v.x = v.x < G ? v.x : G - 1; v.x = v.x < 0 ? 0 : v.x;
    v.y = v.y < G ? v.y : G - 1; v.y = v.y < 0 ? 0 : v.y;
    v.z = v.z < G ? v.z : G - 1; v.z = v.z < 0 ? 0 : v.z;
    return v;
}

static void splat_one(pmo_legacy *s, v3 e, i3 c, int i, int j, int k) {   /* storeNeighborPhoton */
    if (c.x == i && c.y == j && c.z == k) return;
    int dx = c.x - i, dy = c.y - j, dz = c.z - k;
    float dist = sqrtf((float)(dx * dx + dy * dy + dz * dz));
    v3 *g = &s->grid[i][j][k];
    *g = add(*g, divs(scl(e, 0.05f), dist));
}

static void splat(pmo_legacy *s, i3 c, v3 e, int type, int id) {          /* splatEnergy */
    if (type != 1) return;
    int x0 = lo_edge(c.x, 3, 0), y0 = lo_edge(c.y, 3, 0), z0 = lo_edge(c.z, 3, 0);
    int x1 = hi_edge(c.x, 3, G), y1 = hi_edge(c.y, 3, G), z1 = hi_edge(c.z, 3, G);
    if (id == 0 || id == 2) {
        int i = id == 0 ? G - 1 : 0;
        for (int j = y0; j < y1; ++j) for (int k = z0; k < z1; ++k) splat_one(s, e, c, i, j, k);
    } else if (id == 1 || id == 3) {
        int j = id == 1 ? 0 : G - 1;
        for (int i = x0; i < x1; ++i) for (int k = z0; k < z1; ++k) splat_one(s, e, c, i, j, k);
    } else if (id == 4) {
        int k = G - 1;
        for (int i = x0; i < x1; ++i) for (int j = y0; j < y1; ++j) splat_one(s, e, c, i, j, k);
    }
}

static void store_surface(pmo_legacy *s, int type, int id, v3 loc, v3 e) {  /* storePhoton */
    i3 c = clamp_voxel(voxel_of(loc));
    if (type != 0) { v3 *g = &s->grid[c.x][c.y][c.z]; *g = add(*g, e); }
    splat(s, c, e, type, id);
}

static void store_volume(pmo_legacy *s, v3 loc, v3 e) {                    /* storeVolumePhoton */
    i3 c = clamp_voxel(voxel_of(loc));
    v3 *g = &s->grid[c.x][c.y][c.z];
    *g = add(*g, e);
}

/* getColor/filterColor (:605-617): plane 0 passes green, plane 2 red. */
static v3 surface_color(v3 in, int type, int idx) {
    v3 f = mk(1.0f, 1.0f, 1.0f);
    if (type == 1 && idx == 0) f = mk(0.0f, 1.0f, 0.0f);
    else if (type == 1 && idx == 2) f = mk(1.0f, 0.0f, 0.0f);
    return mk(fminf(f.x, in.x), fminf(f.y, in.y), fminf(f.z, in.z));
}

/* ---- one photon path (emitPhotons :1215-1375) -------------------------- */
static void emit_one(pmo_legacy *s, int index, int media) {
    int bounces = 1;
    v3 rgb = mk(10.0f, 10.0f, 10.0f);
    v3 ray = nrm(s->table[index]);
    v3 first_ray = ray;
    v3 prev = light_pos();
    chainstate c;
    c.point = mk(0.0f, 0.0f, 0.0f);
    if (media) {                                     /* three fixed medium steps :1230-1268 */
        for (int i = 0; i < 3; ++i) {
            rgb = subs(rgb, 1.0f);
            c.point = add(scl(ray, 1.0f), prev);
            store_volume(s, c.point, scl(rgb, 0.00005f));
            v3 q = s->table[i];
            v3 rnd;
            rnd.x = rand_float(s, q.x);
            rnd.y = rand_float(s, q.y);
            rnd.z = rand_float(s, q.z);
            ray = nrm(rnd);
            prev = c.point;
        }
        ray = first_ray;
        prev = light_pos();
    }
    if (index < N_CAUSTIC) {                          /* caustic photons aim at sphere 0 :1274-1278 */
        ray = nrm(sub(mk(s->sph[0][0], s->sph[0][1], s->sph[0][2]), light_pos()));
        ray = add(ray, scl(nrm(s->table[index]), 0.01f));
    }
    c.ray = ray;
    trace(s, c.ray, prev, &c.h);
    int caustic = 0, new_point = 1;
    while (c.h.hit && bounces <= N_BOUNCES) {        /* bounce loop :1289-1373 */
        if (new_point) c.point = add(scl(c.ray, c.h.dist), prev);
        if (caustic) {
            rgb = scl(mk(1.0f, 1.0f, 1.0f), 10.0f);
            store_surface(s, c.h.type, c.h.idx, c.point, rgb);
        } else {
            rgb = scl(divs(scl(surface_color(rgb, c.h.type, c.h.idx), 1.0f), sqrtf((float)bounces)), 5.0f);
            store_surface(s, c.h.type, c.h.idx, c.point, rgb);
            /* shadowPhoton (:1185-1196): continue through the surface and
             * deposit -0.25 where the ray lands next. */
            hitrec saved = c.h;
            v3 bumped = add(c.point, scl(c.ray, 0.00001f));
            trace(s, c.ray, bumped, &c.h);
            v3 sp = add(scl(c.ray, c.h.dist), bumped);
            store_surface(s, c.h.type, c.h.idx, sp, mk(-0.25f, -0.25f, -0.25f));
            c.h.type = saved.type;
            c.h.idx = saved.idx;
        }
        prev = c.point;
        if (c.h.type == 0 && c.h.idx == 1) {
            run_chain(s, &c, 1, prev);
            caustic = 0; new_point = 0;
        } else if (c.h.type == 0 && c.h.idx == 0) {
            run_chain(s, &c, 2, prev);
            caustic = 1; new_point = 0;
        } else {
            c.ray = reflect_ray(s, c.ray, prev, c.h.type, c.h.idx, c.point);
            trace(s, c.ray, c.point, &c.h);
            caustic = 0; new_point = 1;
        }
        ++bounces;
    }
}

/* ---- one pixel (computePixelColor :926-1017) --------------------------- */
static v3 shade_pixel(const pmo_legacy *s, float x, float y, int interp, int media) {
    v3 rgb = mk(0.0f, 0.0f, 0.0f);
    v3 origin = mk(0.0f, 0.0f, 0.0f);
    chainstate c;
    c.ray = mk((float)((double)(x / 512.0f) - 0.5), (float)(-((double)(y / 512.0f) - 0.5)), 1.0f);
    c.h.hit = 0;
    if (media) {                                      /* ten fixed march steps :940-961 */
        v3 at = origin;
        float step = 0.6f;
        for (int i = 0; i < 10; ++i) {
            at = add(scl(c.ray, step), at);
            rgb = add(rgb, integrate_volume(s, at));
        }
    }
    trace(s, c.ray, origin, &c.h);
    if (!c.h.hit) return rgb;
    c.point = scl(c.ray, c.h.dist);
    if (c.h.type == 0 && c.h.idx == 1) run_chain(s, &c, 1, origin);
    else if (c.h.type == 0 && c.h.idx == 0) run_chain(s, &c, 2, origin);
    if (!c.h.hit) return rgb;
    v3 zero = mk(0.0f, 0.0f, 0.0f);
    v3 g = interp ? interpolate_slab(s, c.point, zero, c.h.type, c.h.idx)
                  : integrate_slab(s, zero, voxel_of(c.point), c.h.type, c.h.idx);
    if (media) g = scl(g, 0.15f);
    return add(rgb, g);
}

/* Pixel conversion (:1451-1459) as the GPU performs it. */
static unsigned char to_u8(double v) {
    double c = v > 255.0 ? 255.0 : v;
    if (!(c > 0.0)) return 0;
    return (unsigned char)(int)c;
}

/* ---- public entry points ----------------------------------------------- */
pmo_legacy *pmo_legacy_create(void) {
    pmo_legacy *s = (pmo_legacy *)calloc(1, sizeof(pmo_legacy));
    if (s) pmo_legacy_reset(s);
    return s;
}

void pmo_legacy_destroy(pmo_legacy *s) { free(s); }

void pmo_legacy_reset(pmo_legacy *s) {
    memset(s, 0, sizeof(*s));
    s->rng_z = 316u;
    s->rng_w = 6548u;
    pmo_legacy_position_spheres(0.0f, s->sph);
    s->sph[0][0] = 1.0f; s->sph[0][1] = -1.0f; s->sph[0][2] = 1.0f;
    s->sph[1][0] = -0.6f; s->sph[1][1] = -1.0f; s->sph[1][2] = 4.5f;
}

/* init_random_numbers_kernel (:1483-1498): rand3(1.0) drawn x, y, z in turn. */
void pmo_legacy_init_random(pmo_legacy *s) {
    for (int i = 0; i < N_PHOTONS; ++i) {
        s->table[i].x = rand_float(s, 1.0f);
        s->table[i].y = rand_float(s, 1.0f);
        s->table[i].z = rand_float(s, 1.0f);
    }
}

/* launch_emit_photons_kernel (:1523-1546): clear the grid, place the
 * spheres for animTime, run every photon in index order. */
void pmo_legacy_emit(pmo_legacy *s, float animTime, int interp, int media) {
    (void)interp;
    memset(s->grid, 0, sizeof(s->grid));
    pmo_legacy_position_spheres(animTime, s->sph);
    for (int p = 0; p < N_PHOTONS; ++p) emit_one(s, p, media);
}

/* launch_photon_mapping_kernel (:1549-1566). */
void pmo_legacy_render(pmo_legacy *s, unsigned width, unsigned height, float animTime, int interp,
                       int media, unsigned char *rgba, float *rgb) {
    pmo_legacy_position_spheres(animTime, s->sph);
    long n = (long)width * (long)height;
#pragma omp parallel for schedule(dynamic, 1024)
    for (long idx = 0; idx < n; ++idx) {
        unsigned x = (unsigned)(idx % width), y = (unsigned)(idx / width);
        v3 c = shade_pixel(s, (float)x, (float)y, interp, media);
        if (rgb) { rgb[3 * idx] = c.x; rgb[3 * idx + 1] = c.y; rgb[3 * idx + 2] = c.z; }
        rgba[4 * idx + 0] = to_u8((double)c.x * 255.0);
        rgba[4 * idx + 1] = to_u8((double)c.y * 255.0);
        rgba[4 * idx + 2] = to_u8((double)c.z * 255.0);
        rgba[4 * idx + 3] = 0;
    }
}

void pmo_legacy_get_grid(const pmo_legacy *s, float *out) { memcpy(out, s->grid, sizeof(s->grid)); }
void pmo_legacy_set_grid(pmo_legacy *s, const float *in) { memcpy(s->grid, in, sizeof(s->grid)); }
void pmo_legacy_get_table(const pmo_legacy *s, float *out) { memcpy(out, s->table, sizeof(s->table)); }
void pmo_legacy_get_rng(const pmo_legacy *s, unsigned *out) { out[0] = s->rng_z; out[1] = s->rng_w; }
