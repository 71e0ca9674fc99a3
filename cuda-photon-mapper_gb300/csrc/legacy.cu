// legacy.cu -- sm_103a kernels for the reference's voxel photon mapper.
//
// Arithmetic follows photonMappingKernel.cu operation for operation
// (single rounding per float operation, double precision where the
// reference's double literals promote an expression), so the grid and the
// image equal a serial run of the reference's own code. The structure is
// new: the unrolled specular recursion (:673-827) is one bounded loop,
// sphere animation is computed once on the host instead of by every
// thread, the random table is filled in parallel by jumping the generator
// ahead, and grid accumulation is a deterministic sort + ordered sum.
#include "launch_count.cuh"
#include "legacy.cuh"
#include "pm_vec.cuh"
#include "radix_sort.cuh"

#include <cmath>

namespace pm {
namespace {

constexpr int G = kLegacyGrid;

struct Scene {
    float sph[2][4];  // the two traced spheres (nrObjects = {2,5}, :61)
};

__constant__ int c_plane_axis[5] = {0, 1, 0, 1, 2};              // planes[] (:66-72)
__constant__ float c_plane_off[5] = {1.5f, -1.5f, -1.5f, 1.5f, 6.0f};
__constant__ float c_vox_dim[3] = {0.09375f, 0.09375f, 0.1875f};  // getVoxelDim (:426-437)

__device__ __forceinline__ v3 light_pos() { return mk3(0.0f, 1.4f, 3.5f); }  // Light (:64)

struct Hit {
    float dist;
    int type, idx;
    bool hit;
};

__device__ __forceinline__ void consider(Hit &h, float t, int type, int idx) {  // :100-103
    if (t < h.dist && t > 0.0f) { h.type = type; h.idx = idx; h.dist = t; h.hit = true; }
}

// raytrace (:223-241) over the two spheres (:105-126) and five planes (:130-157).
__device__ void trace(const Scene &sc, v3 r, v3 o, Hit &h) {
    h.hit = false;
    h.dist = 999999.9f;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        v3 s = mk3(sc.sph[i][0], sc.sph[i][1], sc.sph[i][2]) - o;
        float rad = sc.sph[i][3];
        float A = dot(r, r);
        float B = (float)(-2.0 * (double)dot(s, r));
        float C = dot(s, s) - rad * rad;
        float D = B * B - (4.0f * A) * C;
        if (D > 0.0f) {
            float sign = ((double)C < -0.00001) ? 1.0f : -1.0f;
            consider(h, (-B + sign * sqrtf(D)) / (2.0f * A), 0, i);
        }
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        float ra = axis_of(r, c_plane_axis[i]);
        if (ra != 0.0f) consider(h, (c_plane_off[i] - axis_of(o, c_plane_axis[i])) / ra, 1, i);
    }
}

// surfaceNormal (:178-201).
__device__ v3 normal_at(const Scene &sc, int type, int idx, v3 p, v3 from) {
    if (type == 0) return normalize(p - mk3(sc.sph[idx][0], sc.sph[idx][1], sc.sph[idx][2]));
    v3 n = mk3(0.0f, 0.0f, 0.0f);
    set_axis(n, c_plane_axis[idx], axis_of(from, c_plane_axis[idx]) - c_plane_off[idx]);
    return normalize(n);
}

__device__ v3 reflect_ray(const Scene &sc, v3 ray, v3 from, int type, int idx, v3 p) {  // :663-668
    v3 n = normal_at(sc, type, idx, p, from) * 1.0f;
    return normalize(ray - n * (2.0f * dot(ray, n)));
}

__device__ v3 refract_ray(const Scene &sc, v3 ray, int type, int idx, v3 p, float factor) {  // :620-659
    v3 n = normal_at(sc, type, idx, p, p) * factor;
    float eta = 1.0f / 1.3f;
    if (factor == -1.0f) eta = 1.0f;
    float cos_i = -dot(n, ray);
    float cos_t2 = (float)(1.0 - (double)(eta * eta) * (1.0 - (double)(cos_i * cos_i)));
    if (cos_t2 > 0.0f) return ray * eta + n * (eta * cos_i - sqrtf(cos_t2));
    return mk3(0.0f, 0.0f, 0.0f);
}

struct Chain {
    v3 ray, point;
    Hit h;
};

// Specular chain (:673-827): stages 1..8 alternate mirror reflection (odd)
// and glass refraction (even); a reflection continues when it lands on the
// glass sphere, a refraction when its exit ray lands on the mirror sphere.
__device__ void run_chain(const Scene &sc, Chain &c, int first, v3 from) {
    for (int st = first; st <= 8; ++st) {
        bool more;
        if (st & 1) {
            c.ray = reflect_ray(sc, c.ray, from, c.h.type, c.h.idx, c.point);
            trace(sc, c.ray, c.point, c.h);
            if (!c.h.hit) break;
            c.point = c.ray * c.h.dist + c.point;
            more = c.h.type == 0 && c.h.idx == 0;
        } else {
            c.ray = refract_ray(sc, c.ray, c.h.type, c.h.idx, c.point, 1.0f);
            c.point = c.ray * 0.00001f + c.point;
            trace(sc, c.ray, c.point, c.h);
            c.point = c.ray * c.h.dist + c.point;
            if (!(c.h.hit && c.h.type == 0 && c.h.idx == 0)) break;
            c.ray = refract_ray(sc, c.ray, c.h.type, c.h.idx, c.point, -1.0f);
            c.point = c.ray * 0.00001f + c.point;
            trace(sc, c.ray, c.point, c.h);
            c.point = c.ray * c.h.dist + c.point;
            more = c.h.type == 0 && c.h.idx == 1;
        }
        if (!more) break;
    }
}

struct I3 {
    int x, y, z;
};

__device__ __forceinline__ I3 voxel_of(v3 p) {  // getVoxelCoordinates (:254-261)
    I3 v;
    v.x = d2i_sat((((double)p.x + 1.5) / 3.0) * 32.0);
    v.y = d2i_sat((((double)p.y + 1.5) / 3.0) * 32.0);
    v.z = d2i_sat(((double)p.z / 6.0) * 32.0);
    return v;
}

__device__ __forceinline__ v3 voxel_center(v3 p) {  // centerPoint + getWorldCoordinates (:263-268, 392-400)
    I3 v = voxel_of(p);
    v3 c = mk3((float)((double)((float)v.x / 32.0f) * 3.0 - 1.5),
               (float)((double)((float)v.y / 32.0f) * 3.0 - 1.5),
               (float)((double)((float)v.z / 32.0f) * 6.0));
    return c + mk3(0.046875f, 0.046875f, 0.09375f);
}

__device__ __forceinline__ int lo_edge(int c, int lo) { return (c - 3 >= lo) ? c - 3 : lo; }
__device__ __forceinline__ int hi_edge(int c, int hi) { return (c + 3 <= hi) ? c + 3 : hi; }
__device__ __forceinline__ int vox_index(int i, int j, int k) { return (i * G + j) * G + k; }

__device__ __forceinline__ v3 grid_at(const float4 *__restrict__ g, int i, int j, int k) {
    float4 q = __ldg(&g[vox_index(i, j, k)]);
    return mk3(q.x, q.y, q.z);
}

// integrate + computeEnergy (:286-389): the plane's wall-slab window.
__device__ v3 integrate_slab(const float4 *__restrict__ g, v3 e, I3 wp, int type, int id) {
    v3 acc = e;
    if (type != 1) return acc;
    int x0 = lo_edge(wp.x, 0), y0 = lo_edge(wp.y, 0), z0 = lo_edge(wp.z, 0);
    int x1 = hi_edge(wp.x, G), y1 = hi_edge(wp.y, G), z1 = hi_edge(wp.z, G);
    if (id == 0 || id == 2) {
        int i = id == 0 ? G - 1 : 0;
        for (int j = y0; j < y1; ++j)
            for (int k = z0; k < z1; ++k) acc = acc + grid_at(g, i, j, k) * 0.0005f;
    } else if (id == 1 || id == 3) {
        int j = id == 1 ? 0 : G - 1;
        for (int i = x0; i < x1; ++i)
            for (int k = z0; k < z1; ++k) acc = acc + grid_at(g, i, j, k) * 0.0005f;
    } else if (id == 4) {
        int k = G - 1;
        for (int i = x0; i < x1; ++i)
            for (int j = y0; j < y1; ++j) acc = acc + grid_at(g, i, j, k) * 0.0005f;
    }
    return acc;
}

__device__ __forceinline__ v3 lerp3(v3 a, v3 b, float t) {  // interpolate3f (:421-423)
    return a * (float)(1.0 - (double)t) + b * t;
}

__device__ __forceinline__ float alpha_of(v3 p, v3 a, v3 b, int ax) {  // getAlpha (:404-418)
    return (axis_of(p, ax) - axis_of(a, ax)) / (axis_of(b, ax) - axis_of(a, ax));
}

// integrateVolumePhotons (:831-870) at voxel wp (getVoxelCoordinates of
// the march point).
__device__ v3 integrate_volume(const float4 *__restrict__ g, I3 wp) {
    v3 acc = mk3(0.0f, 0.0f, 0.0f);
    int x0 = lo_edge(wp.x, 1), y0 = lo_edge(wp.y, 1), z0 = lo_edge(wp.z, 1);
    int x1 = hi_edge(wp.x, G - 1), y1 = hi_edge(wp.y, G - 1), z1 = hi_edge(wp.z, G - 1);
    for (int i = x0; i < x1; ++i)
        for (int j = y0; j < y1; ++j)
            for (int k = z0; k < z1; ++k) acc = acc + grid_at(g, i, j, k);
    return acc;
}

// Both window sums start from zero and depend only on integer voxel
// coordinates, so a frame computes each distinct window once -- in the loop
// order above, so the values are the same bits -- and the render looks them
// up. A coordinate's window is empty outside [kWinLo, kWinLo + kVolN) (volume)
// or [kWinLo, kWinLo + kSlabN) (slab).
constexpr int kWinLo = -2, kVolN = 36, kSlabN = 37;
constexpr int kVolWindows = kVolN * kVolN * kVolN, kSlabWindows = 5 * kSlabN * kSlabN;

__global__ void window_tables_kernel(const float4 *__restrict__ g, float4 *vol, float4 *slab) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < kVolWindows) {
        I3 wp;
        wp.z = t % kVolN + kWinLo;
        wp.y = (t / kVolN) % kVolN + kWinLo;
        wp.x = t / (kVolN * kVolN) + kWinLo;
        const v3 acc = integrate_volume(g, wp);
        vol[t] = make_float4(acc.x, acc.y, acc.z, 0.0f);
    } else if (t < kVolWindows + kSlabWindows) {
        const int u = t - kVolWindows;
        const int id = u / (kSlabN * kSlabN);
        const int a = (u / kSlabN) % kSlabN + kWinLo, b = u % kSlabN + kWinLo;
        // the plane's two free coordinates: (y, z) for 0 and 2, (x, z) for 1
        // and 3, (x, y) for 4; the fixed one does not enter the window
        I3 wp;
        wp.x = id == 0 || id == 2 ? 0 : a;
        wp.y = id == 0 || id == 2 ? a : (id == 4 ? b : 0);
        wp.z = id == 4 ? 0 : b;
        const v3 acc = integrate_slab(g, mk3(0.0f, 0.0f, 0.0f), wp, 1, id);
        slab[u] = make_float4(acc.x, acc.y, acc.z, 0.0f);
    }
}

__device__ __forceinline__ bool in_window_range(int c, int n) { return c >= kWinLo && c < kWinLo + n; }

// integrate_volume through the table.
__device__ __forceinline__ v3 volume_window(const float4 *__restrict__ vol, v3 p) {
    const I3 wp = voxel_of(p);
    if (!in_window_range(wp.x, kVolN) || !in_window_range(wp.y, kVolN) || !in_window_range(wp.z, kVolN))
        return mk3(0.0f, 0.0f, 0.0f);
    const float4 v = __ldg(&vol[((wp.x - kWinLo) * kVolN + (wp.y - kWinLo)) * kVolN + (wp.z - kWinLo)]);
    return mk3(v.x, v.y, v.z);
}

// integrate_slab(g, 0, wp, type, id) through the table.
__device__ __forceinline__ v3 slab_window(const float4 *__restrict__ slab, I3 wp, int type, int id) {
    if (type != 1 || id < 0 || id > 4) return mk3(0.0f, 0.0f, 0.0f);
    const int a = id == 0 || id == 2 ? wp.y : wp.x;
    const int b = id == 4 ? wp.y : wp.z;
    if (!in_window_range(a, kSlabN) || !in_window_range(b, kSlabN)) return mk3(0.0f, 0.0f, 0.0f);
    const float4 v = __ldg(&slab[(id * kSlabN + (a - kWinLo)) * kSlabN + (b - kWinLo)]);
    return mk3(v.x, v.y, v.z);
}

// interpolateEnergy + bilinearInterpolate (:442-583).
__device__ v3 interpolate_slab(const float4 *__restrict__ slab, v3 p, int type, int id) {
    v3 zero = mk3(0.0f, 0.0f, 0.0f);
    if (type != 1) return zero;
    int a1, a2;
    if (id == 0 || id == 2) { a1 = 2; a2 = 1; }
    else if (id == 1 || id == 3) { a1 = 0; a2 = 2; }
    else if (id == 4) { a1 = 0; a2 = 1; }
    else return zero;
    v3 p1 = voxel_center(p);
    v3 p2 = zero, p3 = zero, p4 = zero;
    float c1 = axis_of(p1, a1), d1 = c_vox_dim[a1];
    float s1 = axis_of(p, a1) > c1 ? c1 + d1 : c1 - d1;
    set_axis(p2, a1, s1); set_axis(p3, a1, s1); set_axis(p4, a1, c1);
    float c2 = axis_of(p1, a2), d2 = c_vox_dim[a2];
    float s2 = axis_of(p, a2) > c2 ? c2 + d2 : c2 - d2;
    set_axis(p2, a2, c2); set_axis(p3, a2, s2); set_axis(p4, a2, s2);
    v3 q1 = slab_window(slab, voxel_of(p1), type, id);
    v3 q2 = slab_window(slab, voxel_of(p2), type, id);
    v3 q3 = slab_window(slab, voxel_of(p3), type, id);
    v3 q4 = slab_window(slab, voxel_of(p4), type, id);
    float a = alpha_of(p, p1, p2, a1);
    v3 p12 = lerp3(p1, p2, a), q12 = lerp3(q1, q2, a);
    a = alpha_of(p, p3, p4, a1);
    v3 p34 = lerp3(p3, p4, a), q34 = lerp3(q3, q4, a);
    a = alpha_of(p, p12, p34, a2);
    return lerp3(q12, q34, a);
}

// ---- emission --------------------------------------------------------------

// Records a photon's grid deposits in the order the reference applies them.
// The counting pass only counts; the writing pass stores (voxel, value)
// at this photon's offset.
struct Deposits {
    uint32_t *keys, *idx;
    float4 *vals;
    uint32_t off, n;
    __device__ __forceinline__ void put(int vox, v3 e) {
        if (keys) {
            uint32_t at = off + n;
            keys[at] = (uint32_t)vox;
            idx[at] = at;
            vals[at] = make_float4(e.x, e.y, e.z, 0.0f);
        }
        ++n;
    }
};

__device__ __forceinline__ I3 clamp_voxel(I3 v) {
    v.x = v.x < G ? v.x : G - 1; v.x = v.x < 0 ? 0 : v.x;
    v.y = v.y < G ? v.y : G - 1; v.y = v.y < 0 ? 0 : v.y;
    v.z = v.z < G ? v.z : G - 1; v.z = v.z < 0 ? 0 : v.z;
    return v;
}

__device__ __forceinline__ void splat_one(Deposits &d, v3 e, I3 c, int i, int j, int k) {  // :1059-1071
    if (c.x == i && c.y == j && c.z == k) return;
    int dx = c.x - i, dy = c.y - j, dz = c.z - k;
    float dist = sqrtf((float)(dx * dx + dy * dy + dz * dz));
    d.put(vox_index(i, j, k), div_scalar(e * 0.05f, dist));
}

// storePhoton + splatEnergy (:1074-1144, 1164-1183).
__device__ void store_surface(Deposits &d, int type, int id, v3 loc, v3 e) {
    I3 c = clamp_voxel(voxel_of(loc));
    if (type != 0) d.put(vox_index(c.x, c.y, c.z), e);
    if (type != 1) return;
    int x0 = lo_edge(c.x, 0), y0 = lo_edge(c.y, 0), z0 = lo_edge(c.z, 0);
    int x1 = hi_edge(c.x, G), y1 = hi_edge(c.y, G), z1 = hi_edge(c.z, G);
    if (id == 0 || id == 2) {
        int i = id == 0 ? G - 1 : 0;
        for (int j = y0; j < y1; ++j) for (int k = z0; k < z1; ++k) splat_one(d, e, c, i, j, k);
    } else if (id == 1 || id == 3) {
        int j = id == 1 ? 0 : G - 1;
        for (int i = x0; i < x1; ++i) for (int k = z0; k < z1; ++k) splat_one(d, e, c, i, j, k);
    } else if (id == 4) {
        int k = G - 1;
        for (int i = x0; i < x1; ++i) for (int j = y0; j < y1; ++j) splat_one(d, e, c, i, j, k);
    }
}

__device__ __forceinline__ v3 surface_color(v3 in, int type, int idx) {  // getColor (:605-617)
    v3 f = mk3(1.0f, 1.0f, 1.0f);
    if (type == 1 && idx == 0) f = mk3(0.0f, 1.0f, 0.0f);
    else if (type == 1 && idx == 2) f = mk3(1.0f, 0.0f, 0.0f);
    return mk3(fminf(f.x, in.x), fminf(f.y, in.y), fminf(f.z, in.z));
}

__device__ __forceinline__ uint32_t mulmod(uint64_t a, uint64_t b, uint64_t m) {
    return (uint32_t)((a * b) % m);
}

__host__ __device__ inline uint32_t mwc_jump(uint32_t state, uint64_t a, uint64_t m, uint64_t n) {
    uint64_t r = 1, base = a % m;
    while (n) {
        if (n & 1) r = (r * base) % m;
        base = (base * base) % m;
        n >>= 1;
    }
    return (uint32_t)((r * (uint64_t)state) % m);
}

struct Mwc {
    uint32_t z, w;
    __device__ __forceinline__ uint32_t next() {
        z = kMwcAz * (z & 65535u) + (z >> 16);
        w = kMwcAw * (w & 65535u) + (w >> 16);
        return (z << 16) + w;
    }
    __device__ __forceinline__ float uniform(float max) {  // randFloat (:1038-1051)
        float r = (float)(int)next() / 65535.0f;
        r = (r * 2.0f) * max;
        return r - max;
    }
};

// emitPhotons (:1215-1375) for photon `index`; the medium steps draw from
// the generator positioned at this photon's first draw.
__device__ void emit_one(const Scene &sc, const float4 *__restrict__ table, int index, bool media,
                         Mwc rng, Deposits &d) {
    int bounces = 1;
    v3 rgb = mk3(10.0f, 10.0f, 10.0f);
    float4 t = table[index];
    v3 ray = normalize(mk3(t.x, t.y, t.z));
    v3 first_ray = ray;
    v3 prev = light_pos();
    Chain c;
    c.point = mk3(0.0f, 0.0f, 0.0f);
    if (media) {
        for (int i = 0; i < 3; ++i) {
            rgb = sub_scalar(rgb, 1.0f);
            c.point = ray * 1.0f + prev;
            I3 v = clamp_voxel(voxel_of(c.point));
            d.put(vox_index(v.x, v.y, v.z), rgb * 0.00005f);
            float4 q = table[i];
            v3 rnd;
            rnd.x = rng.uniform(q.x);
            rnd.y = rng.uniform(q.y);
            rnd.z = rng.uniform(q.z);
            ray = normalize(rnd);
            prev = c.point;
        }
        ray = first_ray;
        prev = light_pos();
    }
    if (index < 100) {  // CAUSTICS_PHOTONS aim at the glass sphere (:1274-1278)
        ray = normalize(mk3(sc.sph[0][0], sc.sph[0][1], sc.sph[0][2]) - light_pos());
        ray = ray + normalize(mk3(t.x, t.y, t.z)) * 0.01f;
    }
    c.ray = ray;
    trace(sc, c.ray, prev, c.h);
    bool caustic = false, new_point = true;
    while (c.h.hit && bounces <= 5) {
        if (new_point) c.point = c.ray * c.h.dist + prev;
        if (caustic) {
            rgb = mk3(1.0f, 1.0f, 1.0f) * 10.0f;
            store_surface(d, c.h.type, c.h.idx, c.point, rgb);
        } else {
            rgb = div_scalar(surface_color(rgb, c.h.type, c.h.idx) * 1.0f, sqrtf((float)bounces)) * 5.0f;
            store_surface(d, c.h.type, c.h.idx, c.point, rgb);
            // shadowPhoton (:1185-1196)
            int st = c.h.type, si = c.h.idx;
            v3 bumped = c.point + c.ray * 0.00001f;
            trace(sc, c.ray, bumped, c.h);
            store_surface(d, c.h.type, c.h.idx, c.ray * c.h.dist + bumped, mk3(-0.25f, -0.25f, -0.25f));
            c.h.type = st;
            c.h.idx = si;
        }
        prev = c.point;
        if (c.h.type == 0 && c.h.idx == 1) {
            run_chain(sc, c, 1, prev);
            caustic = false; new_point = false;
        } else if (c.h.type == 0 && c.h.idx == 0) {
            run_chain(sc, c, 2, prev);
            caustic = true; new_point = false;
        } else {
            c.ray = reflect_ray(sc, c.ray, prev, c.h.type, c.h.idx, c.point);
            trace(sc, c.ray, c.point, c.h);
            caustic = false; new_point = true;
        }
        ++bounces;
    }
}

__global__ void __launch_bounds__(256) emit_kernel(Scene sc, const float4 *__restrict__ table,
                                                   bool media, uint32_t z0, uint32_t w0,
                                                   uint32_t *counts, const uint32_t *offsets,
                                                   uint32_t *keys, uint32_t *idx, float4 *vals) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kLegacyPhotons) return;
    Mwc rng;
    rng.z = z0;
    rng.w = w0;
    if (media) {  // each photon's medium loop takes 9 draws, photons in index order
        rng.z = mwc_jump(z0, kMwcAz, kMwcMz, 9ull * (uint64_t)p);
        rng.w = mwc_jump(w0, kMwcAw, kMwcMw, 9ull * (uint64_t)p);
    }
    Deposits d;
    d.keys = offsets ? keys : nullptr;
    d.idx = idx;
    d.vals = vals;
    d.off = offsets ? offsets[p] : 0u;
    d.n = 0;
    emit_one(sc, table, p, media, rng, d);
    if (!offsets) counts[p] = d.n;
}

// Deposit values in sorted order (one parallel gather), so that each
// voxel's sum below streams a contiguous range.
__global__ void gather_deposits_kernel(const uint32_t *__restrict__ sidx,
                                       const float4 *__restrict__ vals, const uint32_t *total,
                                       float4 *sorted) {
    const uint32_t n = *total;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        sorted[j] = vals[sidx[j]];
}

__device__ __forceinline__ uint32_t first_at_least(const uint32_t *__restrict__ keys, uint32_t n,
                                                   uint32_t v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (keys[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Sums each voxel's deposits in photon order and writes both grid layouts;
// one warp per voxel. The lanes load 32 consecutive deposits at a time
// (coalesced, the next 32 already in flight) and the warp adds them in
// order through shuffles: exactly the serial additions, bound by the add
// chain instead of one thread's load latency.
__global__ void __launch_bounds__(256) reduce_kernel(const uint32_t *__restrict__ skeys,
                                                     const float4 *__restrict__ sorted,
                                                     const uint32_t *total, float *grid3,
                                                     float4 *grid4) {
    const int v = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (v >= kLegacyVoxels) return;
    const uint32_t n = *total;
    const uint32_t lo = first_at_least(skeys, n, (uint32_t)v);
    const uint32_t hi = first_at_least(skeys, n, (uint32_t)v + 1u);
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 e = lo + lane < hi ? __ldg(&sorted[lo + lane]) : zero;
    for (uint32_t base = lo; base < hi; base += 32) {
        const uint32_t nb = base + 32;
        const float4 next = nb + lane < hi ? __ldg(&sorted[nb + lane]) : zero;
        const uint32_t cnt = min(32u, hi - base);
        if (cnt == 32) {
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                ax = ax + __shfl_sync(0xffffffffu, e.x, i);
                ay = ay + __shfl_sync(0xffffffffu, e.y, i);
                az = az + __shfl_sync(0xffffffffu, e.z, i);
            }
        } else {
            for (uint32_t i = 0; i < cnt; ++i) {
                ax = ax + __shfl_sync(0xffffffffu, e.x, i);
                ay = ay + __shfl_sync(0xffffffffu, e.y, i);
                az = az + __shfl_sync(0xffffffffu, e.z, i);
            }
        }
        e = next;
    }
    if (lane == 0) {
        grid3[3 * v + 0] = ax;
        grid3[3 * v + 1] = ay;
        grid3[3 * v + 2] = az;
        grid4[v] = make_float4(ax, ay, az, 0.0f);
    }
}

// init_random_numbers_kernel (:1483-1498): entry i holds draws 3i..3i+2
// after `base` earlier draws.
__global__ void table_kernel(float4 *table, uint32_t z0, uint32_t w0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kLegacyPhotons) return;
    Mwc rng;
    rng.z = mwc_jump(z0, kMwcAz, kMwcMz, 3ull * (uint64_t)i);
    rng.w = mwc_jump(w0, kMwcAw, kMwcMw, 3ull * (uint64_t)i);
    float x = rng.uniform(1.0f);
    float y = rng.uniform(1.0f);
    float z = rng.uniform(1.0f);
    table[i] = make_float4(x, y, z, 0.0f);
}

__global__ void grid_from_host_kernel(const float *grid3, float4 *grid4) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < kLegacyVoxels) grid4[v] = make_float4(grid3[3 * v], grid3[3 * v + 1], grid3[3 * v + 2], 0.0f);
}

// ---- render ----------------------------------------------------------------

// computePixelColor (:926-1017).
__device__ v3 shade_pixel(const Scene &sc, const float4 *__restrict__ vol,
                          const float4 *__restrict__ slab, float x, float y, bool interp, bool media) {
    v3 rgb = mk3(0.0f, 0.0f, 0.0f);
    v3 origin = mk3(0.0f, 0.0f, 0.0f);
    Chain c;
    c.ray = mk3((float)((double)(x / 512.0f) - 0.5), (float)(-((double)(y / 512.0f) - 0.5)), 1.0f);
    c.h.hit = false;
    c.h.type = 0;
    c.h.idx = 0;
    if (media) {  // ten fixed steps of 0.6 along the unnormalised ray (:940-961)
        v3 at = origin;
        for (int i = 0; i < 10; ++i) {
            at = c.ray * 0.6f + at;
            rgb = rgb + volume_window(vol, at);
        }
    }
    trace(sc, c.ray, origin, c.h);
    if (!c.h.hit) return rgb;
    c.point = c.ray * c.h.dist;
    if (c.h.type == 0 && c.h.idx == 1) run_chain(sc, c, 1, origin);
    else if (c.h.type == 0 && c.h.idx == 0) run_chain(sc, c, 2, origin);
    if (!c.h.hit) return rgb;
    v3 e = interp ? interpolate_slab(slab, c.point, c.h.type, c.h.idx)
                  : slab_window(slab, voxel_of(c.point), c.h.type, c.h.idx);
    if (media) e = e * 0.15f;
    return rgb + e;
}

__global__ void __launch_bounds__(256) render_kernel(Scene sc, const float4 *__restrict__ vol,
                                                     const float4 *__restrict__ slab, uchar4 *out,
                                                     unsigned width, unsigned height, bool interp,
                                                     bool media, float *rgb_out) {
    unsigned index = blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= width * height) return;
    unsigned x = index % width, y = index / width;
    v3 c = shade_pixel(sc, vol, slab, (float)x, (float)y, interp, media);
    if (rgb_out) {
        rgb_out[3 * index + 0] = c.x;
        rgb_out[3 * index + 1] = c.y;
        rgb_out[3 * index + 2] = c.z;
    }
    out[index] = make_uchar4(to_u8_sat((double)c.x * 255.0), to_u8_sat((double)c.y * 255.0),
                             to_u8_sat((double)c.z * 255.0), 0);
}

Scene make_scene(float anim_time) {
    Scene sc;
    legacy_position_spheres(anim_time, sc.sph);
    return sc;
}

}  // namespace

uint32_t mwc_jump_host(uint32_t state, uint64_t a, uint64_t m, uint64_t n) {
    return mwc_jump(state, a, m, n);
}

void legacy_position_spheres(float t, float out[2][4]) {
    out[0][0] = (float)(1.0 * (double)std::cos(t));
    out[0][1] = (float)(0.5 * std::sin(2.0 * (double)t));
    out[0][2] = (float)((double)std::sin(t) + 3.5);
    out[0][3] = 0.4f;
    out[1][0] = 0.0f;
    out[1][1] = (float)(std::sin(0.5 * (double)t + 5.0) - 0.25);
    out[1][2] = 3.5f;
    out[1][3] = 0.4f;
}

cudaError_t legacy_alloc(LegacyState &st) {
    cudaError_t e;
#define PM_ALLOC(ptr, bytes) \
    if ((e = cudaMalloc((void **)&(ptr), (bytes))) != cudaSuccess) { legacy_free(st); return e; }
    PM_ALLOC(st.table, sizeof(float4) * kLegacyPhotons);
    PM_ALLOC(st.grid3, sizeof(float) * 3 * kLegacyVoxels);
    PM_ALLOC(st.grid4, sizeof(float4) * kLegacyVoxels);
    PM_ALLOC(st.vol_win, sizeof(float4) * kVolWindows);
    PM_ALLOC(st.slab_win, sizeof(float4) * kSlabWindows);
    PM_ALLOC(st.counts, sizeof(uint32_t) * kLegacyPhotons);
    PM_ALLOC(st.offsets, sizeof(uint32_t) * kLegacyPhotons);
    PM_ALLOC(st.total, sizeof(uint32_t));
    PM_ALLOC(st.keys, sizeof(uint32_t) * kLegacyMaxDeposits);
    PM_ALLOC(st.keys_tmp, sizeof(uint32_t) * kLegacyMaxDeposits);
    PM_ALLOC(st.idx, sizeof(uint32_t) * kLegacyMaxDeposits);
    PM_ALLOC(st.idx_tmp, sizeof(uint32_t) * kLegacyMaxDeposits);
    PM_ALLOC(st.dep, sizeof(float4) * kLegacyMaxDeposits);
    PM_ALLOC(st.sdep, sizeof(float4) * kLegacyMaxDeposits);
    PM_ALLOC(st.hist, sizeof(uint32_t) * radix_sort_hist_words(kLegacyMaxDeposits));
#undef PM_ALLOC
    // A fresh module starts with a zero table and grid (static __device__
    // storage in the reference).
    if ((e = cudaMemset(st.table, 0, sizeof(float4) * kLegacyPhotons)) != cudaSuccess) return e;
    if ((e = cudaMemset(st.grid3, 0, sizeof(float) * 3 * kLegacyVoxels)) != cudaSuccess) return e;
    if ((e = cudaMemset(st.grid4, 0, sizeof(float4) * kLegacyVoxels)) != cudaSuccess) return e;
    st.rng_draws = 0;
    return cudaSuccess;
}

void legacy_free(LegacyState &st) {
    cudaFree(st.table); cudaFree(st.grid3); cudaFree(st.grid4); cudaFree(st.counts);
    cudaFree(st.vol_win); cudaFree(st.slab_win);
    cudaFree(st.offsets); cudaFree(st.total); cudaFree(st.keys); cudaFree(st.keys_tmp);
    cudaFree(st.idx); cudaFree(st.idx_tmp); cudaFree(st.dep); cudaFree(st.sdep); cudaFree(st.hist);
    st = LegacyState();
}

cudaError_t legacy_init_random(LegacyState &st, cudaStream_t s) {
    uint32_t z0 = mwc_jump_host(kMwcSeedZ, kMwcAz, kMwcMz, st.rng_draws);
    uint32_t w0 = mwc_jump_host(kMwcSeedW, kMwcAw, kMwcMw, st.rng_draws);
    table_kernel<<<(kLegacyPhotons + 255) / 256, 256, 0, s>>>(st.table, z0, w0); note_launch();
    st.rng_draws += 3ull * kLegacyPhotons;
    st.table_written = true;
    return cudaGetLastError();
}

cudaError_t legacy_emit(LegacyState &st, float anim_time, int flags, cudaStream_t s) {
    Scene sc = make_scene(anim_time);
    bool media = (flags & kLegacyMedia) != 0;
    uint32_t z0 = mwc_jump_host(kMwcSeedZ, kMwcAz, kMwcMz, st.rng_draws);
    uint32_t w0 = mwc_jump_host(kMwcSeedW, kMwcAw, kMwcMw, st.rng_draws);
    const int blocks = (kLegacyPhotons + 255) / 256;
    emit_kernel<<<blocks, 256, 0, s>>>(sc, st.table, media, z0, w0, st.counts, nullptr, nullptr,
                                       nullptr, nullptr); note_launch();
    cudaError_t e = exclusive_scan_u32(st.counts, st.offsets, kLegacyPhotons, st.total, s);
    if (e != cudaSuccess) return e;
    emit_kernel<<<blocks, 256, 0, s>>>(sc, st.table, media, z0, w0, st.counts, st.offsets, st.keys,
                                       st.idx, st.dep); note_launch();
    uint32_t *sk = nullptr, *si = nullptr;
    e = radix_sort_pairs_u32(st.keys, st.idx, st.keys_tmp, st.idx_tmp, st.total, kLegacyMaxDeposits,
                             0, 16, st.hist, s, &sk, &si);
    if (e != cudaSuccess) return e;
    gather_deposits_kernel<<<512, 256, 0, s>>>(si, st.dep, st.total, st.sdep); note_launch();
    reduce_kernel<<<(kLegacyVoxels * 32 + 255) / 256, 256, 0, s>>>(sk, st.sdep, st.total, st.grid3,
                                                                  st.grid4); note_launch();
    if (media) st.rng_draws += 9ull * kLegacyPhotons;
    return cudaGetLastError();
}

cudaError_t legacy_render(const LegacyState &st, uchar4 *out, unsigned width, unsigned height,
                          float anim_time, int flags, float *rgb_out, cudaStream_t s) {
    Scene sc = make_scene(anim_time);
    unsigned n = width * height;
    if (n == 0) return cudaSuccess;
    // the frame's window sums, from the current grid
    window_tables_kernel<<<(kVolWindows + kSlabWindows + 255) / 256, 256, 0, s>>>(st.grid4, st.vol_win,
                                                                                 st.slab_win);
    note_launch();
    render_kernel<<<(n + 255) / 256, 256, 0, s>>>(sc, st.vol_win, st.slab_win, out, width, height,
                                                  (flags & kLegacyInterpolate) != 0,
                                                  (flags & kLegacyMedia) != 0, rgb_out); note_launch();
    return cudaGetLastError();
}

cudaError_t legacy_upload_grid(LegacyState &st, const float *host_grid3, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(st.grid3, host_grid3, sizeof(float) * 3 * kLegacyVoxels,
                                    cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    grid_from_host_kernel<<<(kLegacyVoxels + 255) / 256, 256, 0, s>>>(st.grid3, st.grid4); note_launch();
    return cudaGetLastError();
}

}  // namespace pm
