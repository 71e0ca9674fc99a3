// phys_common.cuh -- scene, geometry and sampling for the physically based
// mode, shared by the trace, build and render kernels.
//
// All arithmetic is single precision with one rounding per operation (the
// library is compiled with -fmad=false; fused operations are written as
// fmaf) and transcendental functions come from pm_math.h, so the CPU oracle
// (oracle/physical_oracle.c) reproduces every photon bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "pm.h"
#include "pm_math.h"
#include "pm_vec.cuh"

namespace pm {

constexpr float kRayEps = 1e-4f;     // minimum hit distance
constexpr int kGridMax = 8;          // sphere grid cells per axis, at most
constexpr float kOffset = 1e-4f;     // origin offset along the normal after an interaction

// The scene as the kernels read it: passed by value as a kernel parameter
// (lives in the constant bank).
struct PScene {
    int ns, np;
    float4 sph[PM_MAX_SPHERES];
    int sph_kind[PM_MAX_SPHERES];
    float sph_alb[PM_MAX_SPHERES][3];
    float sph_ior[PM_MAX_SPHERES];
    int pl_axis[PM_MAX_PLANES];
    float pl_off[PM_MAX_PLANES];
    int pl_kind[PM_MAX_PLANES];
    float pl_alb[PM_MAX_PLANES][3];
    float pl_ior[PM_MAX_PLANES];
    float bmin[3], bmax[3];
    float light[3];
    float sigma_s, sigma_a, g;
    int het_res;
    float sigma_max;                 // majorant of sigma_t
    float inv_sigma_max;             // 1 / sigma_max (0 without a medium)
    float het_scale[3];              // het_res / box extent per axis (grid cells per unit length)
    const float *het;                // het_res^3 sigma_s values (device)
    float cam[3], focal;
    // Uniform grid over the box for the sphere tests (grid_res = 0: none):
    // bit i of cell_mask[(z * G + y) * G + x] is set when sphere i's
    // bounding box, slightly enlarged, overlaps cell (x, y, z).
    int grid_res;
    float grid_inv[3];                   // G / box extent per axis
    uint64_t cell_mask[kGridMax * kGridMax * kGridMax];
};

struct PHit {
    float t;
    int obj;     // >= 0 sphere index, < 0: plane -1-index, kNone: miss
};
constexpr int kNone = 0x7fffffff;

PM_HD float vget(v3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// Distance to the first crossing of sphere s beyond kRayEps along (o, d),
// or -1 when the line misses it. The quadratic's terms are fused
// multiply-adds (one rounding each; the oracle writes the same fmaf calls):
// the photon tracer spends most of its floating-point instructions in this
// test, over every sphere at every event.
__device__ __forceinline__ float sphere_t(float4 s, v3 o, v3 d) {
    const float ox = o.x - s.x, oy = o.y - s.y, oz = o.z - s.z;
    const float b = __fmaf_rn(oz, d.z, __fmaf_rn(oy, d.y, ox * d.x));
    const float c = __fmaf_rn(oz, oz, __fmaf_rn(oy, oy, __fmaf_rn(ox, ox, -(s.w * s.w))));
    const float disc = __fmaf_rn(b, b, -c);
    if (!(disc > 0.0f)) return -1.0f;
    float sq = sqrtf(disc);
    float t = -b - sq;
    if (!(t > kRayEps)) t = -b + sq;
    return t;
}

__device__ __forceinline__ void plane_hits(const PScene &S, v3 o, v3 d, PHit &h);

// Nearest hit with t in (kRayEps, tmax). d must be unit length. Spheres
// are tested in index order; equal distances keep the lower index.
__device__ __forceinline__ PHit intersect(const PScene &S, v3 o, v3 d, float tmax) {
    PHit h;
    h.t = tmax;
    h.obj = kNone;
    for (int i = 0; i < S.ns; ++i) {
        const float t = sphere_t(S.sph[i], o, d);
        if (t > kRayEps && t < h.t) { h.t = t; h.obj = i; }
    }
    plane_hits(S, o, d, h);
    return h;
}

__device__ __forceinline__ void plane_hits(const PScene &S, v3 o, v3 d, PHit &h) {
    for (int i = 0; i < S.np; ++i) {
        int a = S.pl_axis[i];
        float da = vget(d, a);
        if (da != 0.0f) {
            float t = (S.pl_off[i] - vget(o, a)) / da;
            if (t > kRayEps && t < h.t) {
                v3 p = o + d * t;
                int a1 = a == 0 ? 1 : 0, a2 = a == 2 ? 1 : 2;
                float p1 = vget(p, a1), p2 = vget(p, a2);
                if (p1 >= S.bmin[a1] && p1 <= S.bmax[a1] && p2 >= S.bmin[a2] && p2 <= S.bmax[a2]) {
                    h.t = t;
                    h.obj = -1 - i;
                }
            }
        }
    }
}

PM_HD void box_span(const PScene &S, v3 o, v3 d, float *t0, float *t1);

// The same nearest hit as intersect(), with the spheres found through the
// grid: cells are visited in ray order (3D-DDA from the box entry) and each
// sphere is tested once; the walk stops when the best hit lies before the
// current cell's exit. Sphere bounding boxes are enlarged when binned, so a
// hit near a cell boundary is always in a visited cell. Equal distances keep
// the lower index, as in intersect(). Falls back to intersect() without a
// grid. For warp-uniform rays (one eye ray per warp); lanes that walk
// different rays diverge in the cell and sphere loops.
__device__ __forceinline__ PHit intersect_fast(const PScene &S, v3 o, v3 d, float tmax) {
    const int G = S.grid_res;
    if (G <= 0) return intersect(S, o, d, tmax);
    PHit h;
    h.t = tmax;
    h.obj = kNone;
    float t0, t1;
    box_span(S, o, d, &t0, &t1);
    t1 = fminf(t1, tmax);
    if (t0 < t1) {
        const v3 p = o + d * t0;
        int c[3], step[3];
        float tnext[3], tdelta[3];
        const float dv[3] = {d.x, d.y, d.z}, ov[3] = {o.x, o.y, o.z}, pv[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float cs = (S.bmax[a] - S.bmin[a]) / (float)G;
            int ci = (int)((pv[a] - S.bmin[a]) * S.grid_inv[a]);
            ci = min(max(ci, 0), G - 1);
            c[a] = ci;
            if (dv[a] > 0.0f) {
                step[a] = 1;
                tnext[a] = (S.bmin[a] + (float)(ci + 1) * cs - ov[a]) / dv[a];
                tdelta[a] = cs / dv[a];
            } else if (dv[a] < 0.0f) {
                step[a] = -1;
                tnext[a] = (S.bmin[a] + (float)ci * cs - ov[a]) / dv[a];
                tdelta[a] = -cs / dv[a];
            } else {
                step[a] = 0;
                tnext[a] = 3.0e38f;
                tdelta[a] = 3.0e38f;
            }
        }
        uint64_t tested = 0ull;
        for (int it = 0; it < 3 * kGridMax + 3; ++it) {
            uint64_t mask = S.cell_mask[(c[2] * G + c[1]) * G + c[0]] & ~tested;
            tested |= mask;
            while (mask) {
                const int i = __ffsll((long long)mask) - 1;
                mask &= mask - 1ull;
                const float t = sphere_t(S.sph[i], o, d);
                if (t > kRayEps && (t < h.t || (t == h.t && h.obj != kNone && i < h.obj))) {
                    h.t = t;
                    h.obj = i;
                }
            }
            const int ax = tnext[0] < tnext[1] ? (tnext[0] < tnext[2] ? 0 : 2) : (tnext[1] < tnext[2] ? 1 : 2);
            const float texit = tnext[ax];
            if (h.t <= texit || texit >= t1) break;
            c[ax] += step[ax];
            if (c[ax] < 0 || c[ax] >= G) break;
            tnext[ax] += tdelta[ax];
        }
    }
    plane_hits(S, o, d, h);
    return h;
}

// Distance along (o, d) at which the ray leaves the box (o inside).
PM_HD float box_exit(const PScene &S, v3 o, v3 d) {
    float t = 3.0e38f;
    for (int a = 0; a < 3; ++a) {
        float da = vget(d, a);
        if (da > 0.0f) t = fminf(t, (S.bmax[a] - vget(o, a)) / da);
        else if (da < 0.0f) t = fminf(t, (S.bmin[a] - vget(o, a)) / da);
    }
    return t;
}

// Parametric interval [t0, t1] of (o, d) inside the box; empty if t0 >= t1.
PM_HD void box_span(const PScene &S, v3 o, v3 d, float *t0, float *t1) {
    float lo = 0.0f, hi = 3.0e38f;
    for (int a = 0; a < 3; ++a) {
        float da = vget(d, a), oa = vget(o, a);
        if (da != 0.0f) {
            float ta = (S.bmin[a] - oa) / da, tb = (S.bmax[a] - oa) / da;
            lo = fmaxf(lo, fminf(ta, tb));
            hi = fminf(hi, fmaxf(ta, tb));
        } else if (oa < S.bmin[a] || oa > S.bmax[a]) {
            lo = 1.0f; hi = 0.0f;
        }
    }
    *t0 = lo;
    *t1 = hi;
}

__device__ __forceinline__ v3 outward_normal(const PScene &S, int obj, v3 p) {
    if (obj >= 0) {
        float4 s = S.sph[obj];
        return normalize(mk3(p.x - s.x, p.y - s.y, p.z - s.z));
    }
    v3 n = mk3(0.0f, 0.0f, 0.0f);
    set_axis(n, S.pl_axis[-1 - obj], 1.0f);
    return n;
}

__device__ __forceinline__ int material_kind(const PScene &S, int obj) {
    return obj >= 0 ? S.sph_kind[obj] : S.pl_kind[-1 - obj];
}
__device__ __forceinline__ v3 material_albedo(const PScene &S, int obj) {
    const float *a = obj >= 0 ? S.sph_alb[obj] : S.pl_alb[-1 - obj];
    return mk3(a[0], a[1], a[2]);
}
__device__ __forceinline__ float material_ior(const PScene &S, int obj) {
    return obj >= 0 ? S.sph_ior[obj] : S.pl_ior[-1 - obj];
}

// sigma_s at x (heterogeneous grid: nearest voxel).
__device__ __forceinline__ float sigma_s_at(const PScene &S, v3 x) {
    if (S.het_res <= 0) return S.sigma_s;
    int r = S.het_res;
    int i[3];
    for (int a = 0; a < 3; ++a) {
        float f = (vget(x, a) - S.bmin[a]) * S.het_scale[a];
        int q = (int)f;
        i[a] = q < 0 ? 0 : (q >= r ? r - 1 : q);
    }
    return __ldg(&S.het[(i[2] * r + i[1]) * r + i[0]]);
}

// Orthonormal basis around unit n (Duff et al., "Building an Orthonormal
// Basis, Revisited", JCGT 2017).
PM_HD void onb(v3 n, v3 *t, v3 *b) {
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float bb = n.x * n.y * a;
    *t = mk3(1.0f + sign * n.x * n.x * a, sign * bb, -sign * n.x);
    *b = mk3(bb, sign + n.y * n.y * a, -n.y);
}

PM_HD v3 from_local(v3 n, float x, float y, float z) {
    v3 t, b;
    onb(n, &t, &b);
    return mk3(t.x * x + b.x * y + n.x * z, t.y * x + b.y * y + n.y * z,
               t.z * x + b.z * y + n.z * z);
}

PM_HD v3 sample_sphere(float u1, float u2) {
    float z = 1.0f - 2.0f * u1;
    float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float s, c;
    pm_sincos2pi(u2, &s, &c);
    return mk3(r * c, r * s, z);
}

PM_HD v3 sample_cosine(v3 n, float u1, float u2) {
    float r = sqrtf(u1);
    float s, c;
    pm_sincos2pi(u2, &s, &c);
    return normalize(from_local(n, r * c, r * s, sqrtf(fmaxf(0.0f, 1.0f - u1))));
}

// Henyey-Greenstein direction around the travel direction d.
PM_HD v3 sample_hg(v3 d, float g, float u1, float u2) {
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
    return normalize(from_local(d, st * c, st * s, ct));
}

// HG phase function value for the cosine between the photon's travel
// direction and the direction scattered toward the viewer.
PM_HD float hg_phase(float g, float cos_t) {
    float den = 1.0f + g * g - 2.0f * g * cos_t;
    return (1.0f - g * g) / (12.566370614f * den * sqrtf(den));
}

// Exact dielectric Fresnel reflectance for unpolarised light; ci > 0 is
// the cosine on the incident side, eta = n_incident / n_transmitted.
PM_HD float fresnel(float ci, float eta, float *ct_out) {
    float s2 = eta * eta * (1.0f - ci * ci);
    if (s2 >= 1.0f) { *ct_out = 0.0f; return 1.0f; }
    float ct = sqrtf(1.0f - s2);
    float rs = (eta * ci - ct) / (eta * ci + ct);
    float rp = (ci - eta * ct) / (ci + eta * ct);
    *ct_out = ct;
    return 0.5f * (rs * rs + rp * rp);
}

// Octahedral encoding of a unit direction into two snorm16 values.
PM_HD uint32_t oct_encode(v3 d) {
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

PM_HD v3 oct_decode(uint32_t e) {
    float px = (float)(int16_t)(e & 0xFFFF) / 32767.0f;
    float py = (float)(int16_t)(e >> 16) / 32767.0f;
    float pz = 1.0f - fabsf(px) - fabsf(py);
    if (pz < 0.0f) {
        float qx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
        float qy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
        px = qx; py = qy;
    }
    return normalize(mk3(px, py, pz));
}

PM_HD pm_u32x4 philox(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
    pm_u32x4 c;
    c.v[0] = c0; c.v[1] = c1; c.v[2] = c2; c.v[3] = c3;
    return pm_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

}  // namespace pm
