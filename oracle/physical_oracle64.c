/*
 * physical_oracle64.c -- the physically based photon mapper restated in
 * double precision with libm, to measure the error of the GPU's single
 * precision: same methods, same Philox streams (each uniform is the same
 * 24-bit value), same k-NN definition, same estimators.
 *
 * TEST INFRASTRUCTURE ONLY (tests, benchmark CPU baseline). Parity
 * unpinned by the reference, which has no physically based mode; the
 * known-answer tests in tests/test_physical_oracle.py pin this file.
 *
 * Records: pos = (x, y, z, index), pow = (r, g, b, dx, dy, dz).
 */
#include "physical_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../include/pm_math.h"

typedef struct { double x, y, z; } d3;

static d3 mk(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
static d3 add(d3 a, d3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static d3 sub(d3 a, d3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static d3 scl(d3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static double dot3(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static d3 nrm(d3 v) { return scl(v, 1.0 / sqrt(dot3(v, v))); }
static double vget(d3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
static void vset(d3 *v, int a, double s) { if (a == 0) v->x = s; else if (a == 1) v->y = s; else v->z = s; }

#define RAY_EPS 1e-4
#define OFFSET 1e-4
#define NONE 0x7fffffff
#define TWO_PI 6.283185307179586

typedef struct { double t; int obj; } hitr;

static double sigma_max(const pmo_scene *s) {
    return (double)(s->het_res > 0 ? s->het_max : s->sigma_s) + (double)s->sigma_a;
}

static hitr intersect(const pmo_scene *s, d3 o, d3 d, double tmax) {
    hitr h;
    h.t = tmax;
    h.obj = NONE;
    for (int i = 0; i < s->num_spheres; ++i) {
        const float *sp = s->spheres[i];
        d3 oc = mk(o.x - sp[0], o.y - sp[1], o.z - sp[2]);
        double b = dot3(oc, d);
        double c = dot3(oc, oc) - (double)sp[3] * sp[3];
        double disc = b * b - c;
        if (disc > 0.0) {
            double sq = sqrt(disc);
            double t = -b - sq;
            if (!(t > RAY_EPS)) t = -b + sq;
            if (t > RAY_EPS && t < h.t) { h.t = t; h.obj = i; }
        }
    }
    for (int i = 0; i < s->num_planes; ++i) {
        int a = (int)s->planes[i][0];
        double da = vget(d, a);
        if (da != 0.0) {
            double t = (s->planes[i][1] - vget(o, a)) / da;
            if (t > RAY_EPS && t < h.t) {
                d3 p = add(o, scl(d, t));
                int a1 = a == 0 ? 1 : 0, a2 = a == 2 ? 1 : 2;
                double p1 = vget(p, a1), p2 = vget(p, a2);
                if (p1 >= s->box_min[a1] && p1 <= s->box_max[a1] && p2 >= s->box_min[a2] && p2 <= s->box_max[a2]) {
                    h.t = t;
                    h.obj = -1 - i;
                }
            }
        }
    }
    return h;
}

static double box_exit(const pmo_scene *s, d3 o, d3 d) {
    double t = 3.0e38;
    for (int a = 0; a < 3; ++a) {
        double da = vget(d, a);
        if (da > 0.0) t = fmin(t, (s->box_max[a] - vget(o, a)) / da);
        else if (da < 0.0) t = fmin(t, (s->box_min[a] - vget(o, a)) / da);
    }
    return t;
}

static void box_span(const pmo_scene *s, d3 o, d3 d, double *t0, double *t1) {
    double lo = 0.0, hi = 3.0e38;
    for (int a = 0; a < 3; ++a) {
        double da = vget(d, a), oa = vget(o, a);
        if (da != 0.0) {
            double ta = (s->box_min[a] - oa) / da, tb = (s->box_max[a] - oa) / da;
            lo = fmax(lo, fmin(ta, tb));
            hi = fmin(hi, fmax(ta, tb));
        } else if (oa < s->box_min[a] || oa > s->box_max[a]) {
            lo = 1.0; hi = 0.0;
        }
    }
    *t0 = lo;
    *t1 = hi;
}

static d3 outward_normal(const pmo_scene *s, int obj, d3 p) {
    if (obj >= 0) {
        const float *sp = s->spheres[obj];
        return nrm(mk(p.x - sp[0], p.y - sp[1], p.z - sp[2]));
    }
    d3 n = mk(0, 0, 0);
    vset(&n, (int)s->planes[-1 - obj][0], 1.0);
    return n;
}

static const pmo_material *mat_of(const pmo_scene *s, int obj) {
    return obj >= 0 ? &s->sphere_mat[obj] : &s->plane_mat[-1 - obj];
}

static double sigma_s_at(const pmo_scene *s, const float *het, d3 x) {
    if (s->het_res <= 0) return s->sigma_s;
    int r = s->het_res, i[3];
    for (int a = 0; a < 3; ++a) {
        double f = (vget(x, a) - s->box_min[a]) / ((double)s->box_max[a] - s->box_min[a]) * r;
        int q = (int)f;
        i[a] = q < 0 ? 0 : (q >= r ? r - 1 : q);
    }
    return het[(i[2] * r + i[1]) * r + i[0]];
}

static d3 from_local(d3 n, double x, double y, double z) {
    double sign = copysign(1.0, n.z);
    double a = -1.0 / (sign + n.z);
    double bb = n.x * n.y * a;
    d3 t = mk(1.0 + sign * n.x * n.x * a, sign * bb, -sign * n.x);
    d3 b = mk(bb, sign + n.y * n.y * a, -n.y);
    return mk(t.x * x + b.x * y + n.x * z, t.y * x + b.y * y + n.y * z, t.z * x + b.z * y + n.z * z);
}

static d3 sample_sphere(double u1, double u2) {
    double z = 1.0 - 2.0 * u1, r = sqrt(fmax(0.0, 1.0 - z * z));
    return mk(r * cos(TWO_PI * u2), r * sin(TWO_PI * u2), z);
}

static d3 sample_cosine(d3 n, double u1, double u2) {
    double r = sqrt(u1);
    return nrm(from_local(n, r * cos(TWO_PI * u2), r * sin(TWO_PI * u2), sqrt(fmax(0.0, 1.0 - u1))));
}

static d3 sample_hg(d3 d, double g, double u1, double u2) {
    double ct;
    if (fabs(g) < 1e-3) ct = 1.0 - 2.0 * u1;
    else {
        double sq = (1.0 - g * g) / (1.0 - g + 2.0 * g * u1);
        ct = (1.0 + g * g - sq * sq) / (2.0 * g);
    }
    ct = fmin(1.0, fmax(-1.0, ct));
    double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    return nrm(from_local(d, st * cos(TWO_PI * u2), st * sin(TWO_PI * u2), ct));
}

static double hg_phase(double g, double c) {
    double den = 1.0 + g * g - 2.0 * g * c;
    return (1.0 - g * g) / (4.0 * M_PI * den * sqrt(den));
}

static double fresnel(double ci, double eta, double *ct_out) {
    double s2 = eta * eta * (1.0 - ci * ci);
    if (s2 >= 1.0) { *ct_out = 0.0; return 1.0; }
    double ct = sqrt(1.0 - s2);
    double rs = (eta * ci - ct) / (eta * ci + ct), rp = (ci - eta * ct) / (ci + eta * ct);
    *ct_out = ct;
    return 0.5 * (rs * rs + rp * rp);
}

static pm_u32x4 philox(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
    pm_u32x4 c;
    c.v[0] = c0; c.v[1] = c1; c.v[2] = c2; c.v[3] = c3;
    return pm_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}
static double u01(uint32_t x) { return (double)(x >> 8) * 5.9604644775390625e-08; }

static void trace_path(const pmo_scene *s, const pmo_config *cfg, const float *het, uint32_t id,
                       double *spos, double *spow, uint32_t *ns_out, double *vpos, double *vpow,
                       uint32_t *nv_out) {
    const int mb = cfg->max_bounces;
    const double rr = cfg->rr_survival, smax = sigma_max(s);
    pm_u32x4 r0 = philox(cfg->seed, id, 0u, 0u, cfg->scene_id);
    d3 o = mk(s->light[0], s->light[1], s->light[2]);
    d3 d = sample_sphere(u01(r0.v[0]), u01(r0.v[1]));
    d3 thr = mk(1, 1, 1);
    int glass = 0;
    uint32_t ns = 0, nv = 0;
    for (int ev = 1; ev <= mb; ++ev) {
        pm_u32x4 r = philox(cfg->seed, id, (uint32_t)ev, 0u, cfg->scene_id);
        double u0 = u01(r.v[0]), u1 = u01(r.v[1]), u2 = u01(r.v[2]), u3 = u01(r.v[3]);
        hitr h = intersect(s, o, d, 3.0e38);
        double seg = h.obj != NONE ? h.t : box_exit(s, o, d);
        int vol = 0;
        d3 x = o;
        double ss = 0.0, st = 1.0;
        if (smax > 0.0 && !glass) {
            if (s->het_res <= 0) {
                st = (double)s->sigma_s + s->sigma_a;
                if (s->sigma_s > 0.0f) {
                    double t = -log(1.0 - u0) / st;
                    if (t < seg) { vol = 1; x = add(o, scl(d, t)); ss = s->sigma_s; }
                }
            } else {
                double t = 0.0;
                pm_u32x4 q;
                for (uint32_t j = 0; j < 4096u; ++j) {
                    /* two tentative collisions per Philox block, as the float32 paths */
                    if ((j & 1u) == 0u) q = philox(cfg->seed, id, (uint32_t)ev, 1u + (j >> 1), cfg->scene_id);
                    const uint32_t ua = (j & 1u) ? q.v[2] : q.v[0], ub = (j & 1u) ? q.v[3] : q.v[1];
                    t += -log(1.0 - u01(ua)) / smax;
                    if (!(t < seg)) break;
                    d3 y = add(o, scl(d, t));
                    double sv = sigma_s_at(s, het, y), sty = sv + s->sigma_a;
                    if (u01(ub) * smax < sty) { vol = 1; x = y; ss = sv; st = sty; break; }
                }
            }
        }
        if (vol) {
            if (nv < (uint32_t)mb) {
                double *p = vpos + 4 * nv, *w = vpow + 6 * nv;
                p[0] = x.x; p[1] = x.y; p[2] = x.z; p[3] = 0;
                w[0] = thr.x; w[1] = thr.y; w[2] = thr.z; w[3] = d.x; w[4] = d.y; w[5] = d.z;
            }
            nv++;
            if (!(u1 < rr)) break;
            thr = scl(thr, (ss / st) / rr);
            d = sample_hg(d, s->hg_g, u2, u3);
            o = x;
            continue;
        }
        if (h.obj == NONE) break;
        d3 hp = add(o, scl(d, h.t));
        d3 n = outward_normal(s, h.obj, hp);
        const pmo_material *m = mat_of(s, h.obj);
        double dn = dot3(n, d);
        d3 nf = dn < 0.0 ? n : scl(n, -1.0);
        if (m->kind == PMO_MAT_DIFFUSE) {
            if (ns < (uint32_t)mb) {
                double *p = spos + 4 * ns, *w = spow + 6 * ns;
                p[0] = hp.x; p[1] = hp.y; p[2] = hp.z; p[3] = 0;
                w[0] = thr.x; w[1] = thr.y; w[2] = thr.z; w[3] = d.x; w[4] = d.y; w[5] = d.z;
            }
            ns++;
            if (!(u1 < rr)) break;
            thr = mk(thr.x * m->albedo[0] / rr, thr.y * m->albedo[1] / rr, thr.z * m->albedo[2] / rr);
            d = sample_cosine(nf, u2, u3);
            o = add(hp, scl(nf, OFFSET));
        } else if (m->kind == PMO_MAT_MIRROR) {
            d = nrm(sub(d, scl(n, 2.0 * dn)));
            o = add(hp, scl(nf, OFFSET));
        } else {
            double ci = -dn;
            int entering = ci > 0.0;
            double eta = entering ? 1.0 / m->ior : m->ior;
            d3 nn = entering ? n : scl(n, -1.0);
            ci = fabs(ci);
            double ct, F = fresnel(ci, eta, &ct);
            if (u1 < F) {
                d = nrm(add(d, scl(nn, 2.0 * ci)));
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

/* Paths traced in parallel rounds, each into its own slots, then merged in
 * path order: the maps equal a serial run's. */
#define PMO64_EMIT_ROUND 32768u
int pmo64_emit(const pmo_scene *scene, const pmo_config *cfg, const float *het, double *spos,
               double *spow, double *vpos, double *vpow, uint32_t *sizes, uint32_t *paths) {
    const int mb = cfg->max_bounces > 0 ? cfg->max_bounces : 1;
    const size_t slots = (size_t)PMO64_EMIT_ROUND * (size_t)mb;
    double *a = malloc(sizeof(double) * 4 * slots), *b = malloc(sizeof(double) * 6 * slots);
    double *c = malloc(sizeof(double) * 4 * slots), *e = malloc(sizeof(double) * 6 * slots);
    uint32_t *ncs = malloc(sizeof(uint32_t) * PMO64_EMIT_ROUND);
    uint32_t *ncv = malloc(sizeof(uint32_t) * PMO64_EMIT_ROUND);
    if (!a || !b || !c || !e || !ncs || !ncv) {
        free(a); free(b); free(c); free(e); free(ncs); free(ncv);
        return -1;
    }
    uint32_t targets[2] = {cfg->surface_photons, cfg->volume_photons};
    uint32_t n[2] = {0, 0}, np[2] = {0, 0};
    int done[2] = {targets[0] == 0, targets[1] == 0};
    uint32_t tmax = targets[0] > targets[1] ? targets[0] : targets[1];
    uint64_t cap = cfg->max_paths ? cfg->max_paths : (uint64_t)tmax * 16u;
    if (cap < 1024) cap = 1024;
    for (uint64_t base = 0; base < cap && !(done[0] && done[1]); base += PMO64_EMIT_ROUND) {
        const uint32_t m = cap - base < PMO64_EMIT_ROUND ? (uint32_t)(cap - base) : PMO64_EMIT_ROUND;
#pragma omp parallel for schedule(dynamic, 256)
        for (long j = 0; j < (long)m; ++j)
            trace_path(scene, cfg, het, (uint32_t)(base + (uint64_t)j), a + (size_t)j * mb * 4,
                       b + (size_t)j * mb * 6, &ncs[j], c + (size_t)j * mb * 4, e + (size_t)j * mb * 6,
                       &ncv[j]);
        for (uint32_t j = 0; j < m && !(done[0] && done[1]); ++j) {
            const uint32_t id = (uint32_t)(base + j);
            uint32_t cnt[2] = {ncs[j], ncv[j]};
            double *sp[2] = {a + (size_t)j * mb * 4, c + (size_t)j * mb * 4};
            double *sw[2] = {b + (size_t)j * mb * 6, e + (size_t)j * mb * 6};
            double *dp[2] = {spos, vpos}, *dw[2] = {spow, vpow};
            for (int mm = 0; mm < 2; ++mm) {
                if (done[mm]) continue;
                np[mm] = id + 1;
                for (uint32_t k = 0; k < cnt[mm] && n[mm] < targets[mm]; ++k) {
                    memcpy(dp[mm] + 4 * n[mm], sp[mm] + 4 * k, sizeof(double) * 4);
                    memcpy(dw[mm] + 6 * n[mm], sw[mm] + 6 * k, sizeof(double) * 6);
                    dp[mm][4 * n[mm] + 3] = n[mm];
                    n[mm]++;
                }
                if (n[mm] >= targets[mm]) done[mm] = 1;
            }
        }
    }
    for (int mm = 0; mm < 2; ++mm) {
        double *w = mm == 0 ? spow : vpow;
        double scale = (double)scene->light_power / np[mm];
        for (uint32_t i = 0; i < n[mm]; ++i) { w[6 * i] *= scale; w[6 * i + 1] *= scale; w[6 * i + 2] *= scale; }
        sizes[mm] = n[mm];
        paths[mm] = np[mm];
    }
    free(a); free(b); free(c); free(e); free(ncs); free(ncv);
    return 0;
}

/* exact k-NN in double: uniform grid, (d2, index) order */
typedef struct { double lo[3], cell; int dim[3]; uint32_t *start, *items; const double *pos; } grid64;

static int cell_of(const grid64 *g, int a, double v) {
    int c = (int)floor((v - g->lo[a]) / g->cell);
    return c < 0 ? 0 : (c >= g->dim[a] ? g->dim[a] - 1 : c);
}

static grid64 *grid_build(const double *pos, uint32_t n, double radius) {
    grid64 *g = calloc(1, sizeof(grid64));
    double hi[3];
    for (int a = 0; a < 3; ++a) { g->lo[a] = n ? 1e300 : 0; hi[a] = n ? -1e300 : 0; }
    for (uint32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) { g->lo[a] = fmin(g->lo[a], pos[4 * i + a]); hi[a] = fmax(hi[a], pos[4 * i + a]); }
    g->cell = radius;
    long total = 1;
    for (int a = 0; a < 3; ++a) {
        long d = (long)((hi[a] - g->lo[a]) / radius) + 1;
        if (d > 512) d = 512;
        g->dim[a] = (int)d;
        total *= d;
        double need = (hi[a] - g->lo[a]) / d;
        if (need > g->cell) g->cell = need * 1.0001;
    }
    g->start = calloc((size_t)total + 1, sizeof(uint32_t));
    g->items = malloc(sizeof(uint32_t) * (n ? n : 1));
    g->pos = pos;
    uint32_t *fill = calloc((size_t)total, sizeof(uint32_t));
    for (int pass = 0; pass < 2; ++pass) {
        for (uint32_t i = 0; i < n; ++i) {
            int c = (cell_of(g, 2, pos[4 * i + 2]) * g->dim[1] + cell_of(g, 1, pos[4 * i + 1])) * g->dim[0] + cell_of(g, 0, pos[4 * i]);
            if (pass == 0) g->start[c + 1]++;
            else g->items[g->start[c] + fill[c]++] = i;
        }
        if (pass == 0) for (long c = 0; c < total; ++c) g->start[c + 1] += g->start[c];
    }
    free(fill);
    return g;
}

static void grid_free(grid64 *g) { free(g->start); free(g->items); free(g); }

typedef struct { double d2; uint32_t i; } cand;

static int grid_knn(const grid64 *g, const double q[3], int k, double r2, cand *out) {
    int cnt = 0, lo[3], hi[3];
    double r = sqrt(r2);
    for (int a = 0; a < 3; ++a) {
        lo[a] = cell_of(g, a, q[a] - r) - 1; if (lo[a] < 0) lo[a] = 0;
        hi[a] = cell_of(g, a, q[a] + r) + 1; if (hi[a] >= g->dim[a]) hi[a] = g->dim[a] - 1;
    }
    for (int z = lo[2]; z <= hi[2]; ++z)
        for (int y = lo[1]; y <= hi[1]; ++y)
            for (int x = lo[0]; x <= hi[0]; ++x) {
                int c = (z * g->dim[1] + y) * g->dim[0] + x;
                for (uint32_t it = g->start[c]; it < g->start[c + 1]; ++it) {
                    uint32_t i = g->items[it];
                    const double *p = g->pos + 4 * i;
                    double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
                    double d2 = dx * dx + dy * dy + dz * dz;
                    if (!(d2 <= r2)) continue;
                    if (cnt == k && (d2 > out[k - 1].d2 || (d2 == out[k - 1].d2 && i > out[k - 1].i))) continue;
                    int j = cnt < k ? cnt++ : k - 1;
                    while (j > 0 && (out[j - 1].d2 > d2 || (out[j - 1].d2 == d2 && out[j - 1].i > i))) { out[j] = out[j - 1]; --j; }
                    out[j].d2 = d2;
                    out[j].i = i;
                }
            }
    return cnt;
}

static d3 shade(const pmo_scene *s, const pmo_config *c, const float *het, const double *spow,
                uint32_t ns, const double *vpow, uint32_t nv, grid64 *gs, grid64 *gv, uint32_t pix) {
    const double aspect = c->height > 0 ? (double)c->width / c->height : 1.0;
    const double r2cap = (double)c->radius * c->radius;
    const double smax = sigma_max(s);
    uint32_t px = pix % (uint32_t)c->width, py = pix / (uint32_t)c->width;
    double u = ((double)px / c->width - 0.5) * aspect, v = -((double)py / c->height - 0.5);
    d3 o = mk(s->cam_pos[0], s->cam_pos[1], s->cam_pos[2]);
    d3 d = nrm(mk(u, v, s->focal));
    d3 L = mk(0, 0, 0);
    double tau = 0.0;
    int glass = 0;
    cand nb[128];
    for (int depth = 0; depth < 8; ++depth) {
        hitr h = intersect(s, o, d, 3.0e38);
        double tend = h.obj != NONE ? h.t : 3.0e38;
        if (c->march_step > 0.0f && smax > 0.0 && !glass) {
            double t0, t1;
            box_span(s, o, d, &t0, &t1);
            t1 = fmin(t1, tend);
            if (t0 < t1) {
                int nst = (int)fmin(ceil((t1 - t0) / c->march_step), 65536.0);
                for (int j = 0; j < nst; ++j) {
                    double ta = t0 + (double)j * c->march_step;
                    double tb = fmin(t0 + (double)(j + 1) * c->march_step, t1);
                    double dt = tb - ta, tm = 0.5 * (ta + tb);
                    d3 x = add(o, scl(d, tm));
                    double ss = s->het_res > 0 ? sigma_s_at(s, het, x) : s->sigma_s, st = ss + s->sigma_a;
                    double tau_mid = tau + st * 0.5 * dt;
                    if (nv > 0) {
                        double q[3] = {x.x, x.y, x.z};
                        int cnt = grid_knn(gv, q, c->k, r2cap, nb);
                        if (cnt > 0) {
                            double r2 = cnt == c->k ? nb[c->k - 1].d2 : r2cap;
                            d3 e = mk(0, 0, 0);
                            for (int i = 0; i < cnt; ++i) {
                                const double *w = vpow + 6 * nb[i].i;
                                double ph = hg_phase(s->hg_g, -(w[3] * d.x + w[4] * d.y + w[5] * d.z));
                                e = add(e, scl(mk(w[0], w[1], w[2]), ph));
                            }
                            L = add(L, scl(e, exp(-tau_mid) * dt / (4.0 / 3.0 * M_PI * r2 * sqrt(r2))));
                        }
                    }
                    tau += st * dt;
                }
            }
        }
        if (h.obj == NONE) break;
        d3 hp = add(o, scl(d, h.t));
        d3 n = outward_normal(s, h.obj, hp);
        const pmo_material *m = mat_of(s, h.obj);
        double dn = dot3(n, d);
        d3 nf = dn < 0.0 ? n : scl(n, -1.0);
        if (m->kind == PMO_MAT_DIFFUSE) {
            if (ns > 0) {
                double q[3] = {hp.x, hp.y, hp.z};
                int cnt = grid_knn(gs, q, c->k, r2cap, nb);
                if (cnt > 0) {
                    double r2 = cnt == c->k ? nb[c->k - 1].d2 : r2cap;
                    d3 e = mk(0, 0, 0);
                    for (int i = 0; i < cnt; ++i) {
                        const double *w = spow + 6 * nb[i].i;
                        if (nf.x * w[3] + nf.y * w[4] + nf.z * w[5] < 0.0) e = add(e, mk(w[0], w[1], w[2]));
                    }
                    double sc = exp(-tau) / (M_PI * r2) / M_PI;
                    L = add(L, mk(m->albedo[0] * e.x * sc, m->albedo[1] * e.y * sc, m->albedo[2] * e.z * sc));
                }
            }
            break;
        }
        if (m->kind == PMO_MAT_MIRROR) {
            d = nrm(sub(d, scl(n, 2.0 * dn)));
            o = add(hp, scl(nf, OFFSET));
        } else {
            double ci = -dn;
            int entering = ci > 0.0;
            double eta = entering ? 1.0 / m->ior : m->ior;
            d3 nn = entering ? n : scl(n, -1.0);
            ci = fabs(ci);
            double ct, F = fresnel(ci, eta, &ct);
            pm_u32x4 r = philox(c->seed, pix, (uint32_t)depth, 0xE7E5A17Bu, c->scene_id);
            if (u01(r.v[0]) < F) {
                d = nrm(add(d, scl(nn, 2.0 * ci)));
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

void pmo64_render(const pmo_scene *scene, const pmo_config *cfg, const float *het,
                  const double *spos, const double *spow, uint32_t ns, const double *vpos,
                  const double *vpow, uint32_t nv, const uint32_t *pixels, uint32_t npix,
                  double *out) {
    grid64 *gs = grid_build(spos, ns, cfg->radius), *gv = grid_build(vpos, nv, cfg->radius);
#pragma omp parallel for schedule(dynamic, 16)
    for (long i = 0; i < (long)npix; ++i) {
        d3 L = shade(scene, cfg, het, spow, ns, vpow, nv, gs, gv, pixels[i]);
        out[4 * i] = L.x; out[4 * i + 1] = L.y; out[4 * i + 2] = L.z; out[4 * i + 3] = 1.0;
    }
    grid_free(gs);
    grid_free(gv);
}

/* The reference's record-list radius gather (kernelPBO.cu:165-182), over
 * the records in index order with the gated squared distance of
 * gatedSqDist3 (:245-257) evaluated in float as the reference does, and the
 * rest in double: energy * max(0, -N.dir) * (1 - distance) / exposure. */
void pmo64_radius_gather(const float (*pos)[4], const float (*pw)[4], const float (*dirs)[3],
                         uint32_t n, const float (*pts)[4], const float (*nrm)[4], uint32_t nq,
                         float sq_radius, float exposure, double (*out)[3]) {
#pragma omp parallel for schedule(dynamic, 16)
    for (long qi = 0; qi < (long)nq; ++qi) {
        double e[3] = {0, 0, 0};
        for (uint32_t i = 0; i < n; ++i) {
            float c = pts[qi][0] - pos[i][0];
            float d = c * c;
            if (d > sq_radius) continue;
            c = pts[qi][1] - pos[i][1];
            d += c * c;
            if (d > sq_radius) continue;
            c = pts[qi][2] - pos[i][2];
            d += c * c;
            if (d > sq_radius) continue;
            double nd = (double)nrm[qi][0] * dirs[i][0] + (double)nrm[qi][1] * dirs[i][1] +
                        (double)nrm[qi][2] * dirs[i][2];
            double w = fmax(0.0, -nd) * (1.0 - sqrt((double)d)) / exposure;
            for (int k = 0; k < 3; ++k) e[k] += pw[i][k] * w;
        }
        for (int k = 0; k < 3; ++k) out[qi][k] = e[k];
    }
}
