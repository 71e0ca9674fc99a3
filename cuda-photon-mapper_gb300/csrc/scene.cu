// scene.cu -- benchmark scene presets (host) and the heterogeneous-medium
// noise grid (device).
#include "launch_count.cuh"
#include "pm.h"
#include "phys_common.cuh"
#include "scene.cuh"

#include <cmath>
#include <cstring>

namespace pm {
namespace {

// splitmix64 (Steele, Lea, Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): the seeded stream scene placement draws from.
struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }
    float range(float a, float b) { return a + (b - a) * uniform(); }
};

void set_mat(pm_material &m, int kind, float r, float g, float b, float ior) {
    m.kind = kind;
    m.albedo[0] = r; m.albedo[1] = g; m.albedo[2] = b;
    m.ior = ior;
}

// The Cornell-style box of every preset: floor, ceiling, left (red),
// right (green) and back walls, open toward the camera at z = -0.5.
void base_box(pm_scene &s) {
    s.box_min[0] = -0.5f; s.box_min[1] = 0.0f; s.box_min[2] = -0.5f;
    s.box_max[0] = 0.5f;  s.box_max[1] = 1.0f; s.box_max[2] = 0.5f;
    s.num_planes = 5;
    s.planes[0] = make_float2(1.0f, 0.0f);   // floor
    s.planes[1] = make_float2(1.0f, 1.0f);   // ceiling
    s.planes[2] = make_float2(0.0f, -0.5f);  // left
    s.planes[3] = make_float2(0.0f, 0.5f);   // right
    s.planes[4] = make_float2(2.0f, 0.5f);   // back
    set_mat(s.plane_mat[0], PM_MAT_DIFFUSE, 0.75f, 0.75f, 0.75f, 1.0f);
    set_mat(s.plane_mat[1], PM_MAT_DIFFUSE, 0.75f, 0.75f, 0.75f, 1.0f);
    set_mat(s.plane_mat[2], PM_MAT_DIFFUSE, 0.75f, 0.25f, 0.25f, 1.0f);
    set_mat(s.plane_mat[3], PM_MAT_DIFFUSE, 0.25f, 0.75f, 0.25f, 1.0f);
    set_mat(s.plane_mat[4], PM_MAT_DIFFUSE, 0.75f, 0.75f, 0.75f, 1.0f);
    s.light[0] = 0.0f; s.light[1] = 0.95f; s.light[2] = 0.0f;
    s.light_power = 1.0f;
    s.cam_pos[0] = 0.0f; s.cam_pos[1] = 0.5f; s.cam_pos[2] = -1.5f;
    s.focal = 1.0f;
}

// Seeded spheres: radii uniform in [rmin, rmax], centres uniform in the
// box shrunk by the radius, kept clear of the light and of each other when
// a placement attempt allows (bounded attempts); materials 50 % diffuse
// (seeded colour), 25 % mirror, 25 % dielectric (ior 1.5).
void seeded_spheres(pm_scene &s, int count, float rmin, float rmax, SplitMix &rng) {
    s.num_spheres = 0;
    for (int i = 0; i < count; ++i) {
        float r = rng.range(rmin, rmax), cx = 0, cy = 0, cz = 0;
        for (int attempt = 0; attempt < 64; ++attempt) {
            cx = rng.range(s.box_min[0] + r, s.box_max[0] - r);
            cy = rng.range(s.box_min[1] + r, s.box_max[1] - r);
            cz = rng.range(s.box_min[2] + r, s.box_max[2] - r);
            float lx = cx - s.light[0], ly = cy - s.light[1], lz = cz - s.light[2];
            bool ok = std::sqrt(lx * lx + ly * ly + lz * lz) > r + 0.02f;
            for (int j = 0; ok && j < s.num_spheres; ++j) {
                float dx = cx - s.spheres[j].x, dy = cy - s.spheres[j].y, dz = cz - s.spheres[j].z;
                ok = std::sqrt(dx * dx + dy * dy + dz * dz) > r + s.spheres[j].w;
            }
            if (ok || attempt == 63) {
                if (!ok) {
                    // keep the light outside every sphere whatever happens
                    float lx2 = cx - s.light[0], ly2 = cy - s.light[1], lz2 = cz - s.light[2];
                    if (std::sqrt(lx2 * lx2 + ly2 * ly2 + lz2 * lz2) <= r + 0.02f) cy = s.box_min[1] + r;
                }
                break;
            }
        }
        s.spheres[i] = make_float4(cx, cy, cz, r);
        float pick = rng.uniform();
        if (pick < 0.5f) {
            // red, green, blue drawn in that order (separate statements: the
            // order of a call's argument evaluations is unspecified)
            const float ar = rng.range(0.2f, 0.9f);
            const float ag = rng.range(0.2f, 0.9f);
            const float ab = rng.range(0.2f, 0.9f);
            set_mat(s.sphere_mat[i], PM_MAT_DIFFUSE, ar, ag, ab, 1.0f);
        } else if (pick < 0.75f)
            set_mat(s.sphere_mat[i], PM_MAT_MIRROR, 1.0f, 1.0f, 1.0f, 1.0f);
        else
            set_mat(s.sphere_mat[i], PM_MAT_DIELECTRIC, 1.0f, 1.0f, 1.0f, 1.5f);
        s.num_spheres = i + 1;
    }
}

}  // namespace

pm_status preset(int which, uint64_t seed, pm_scene *scene, pm_config *cfg) {
    if (!scene || !cfg || which < 1 || which > 3) return PM_ERR_INVALID;
    pm_scene s;
    memset(&s, 0, sizeof(s));
    pm_config c;
    memset(&c, 0, sizeof(c));
    base_box(s);
    s.sigma_s = 0.1f;
    s.sigma_a = 0.02f;
    s.hg_g = 0.3f;
    c.seed = seed;
    c.scene_id = 0;
    c.rr_survival = 0.8f;
    c.leaf_size = 32;
    c.exposure = 8.0f;
    SplitMix rng{seed ^ (0xC0FFEEull * (uint64_t)which)};
    if (which == 1) {
        s.num_spheres = 2;
        s.spheres[0] = make_float4(-0.2f, 0.3f, 0.1f, 0.3f);
        set_mat(s.sphere_mat[0], PM_MAT_DIFFUSE, 0.75f, 0.75f, 0.75f, 1.0f);
        s.spheres[1] = make_float4(0.24f, 0.25f, -0.2f, 0.25f);
        set_mat(s.sphere_mat[1], PM_MAT_MIRROR, 1.0f, 1.0f, 1.0f, 1.0f);
        c.surface_photons = 100000;
        c.volume_photons = 100000;
        c.max_bounces = 5;
        c.width = 512; c.height = 512;
        c.k = 64; c.radius = 0.1f;
        c.march_step = 0.01f;
    } else if (which == 2) {
        seeded_spheres(s, 8, 0.05f, 0.3f, rng);
        c.surface_photons = 1000000;
        c.volume_photons = 1000000;
        c.max_bounces = 5;
        c.width = 1024; c.height = 1024;
        c.k = 100; c.radius = 0.05f;
        c.march_step = 0.01f;
    } else {
        seeded_spheres(s, 64, 0.05f, 0.3f, rng);
        s.het_res = 128;
        s.het_min = 0.02f;
        s.het_max = 0.3f;
        c.surface_photons = 8000000;
        c.volume_photons = 8000000;
        c.max_bounces = 8;
        c.width = 1920; c.height = 1080;
        c.k = 128; c.radius = 0.05f;
        c.march_step = 0.01f;
    }
    *scene = s;
    *cfg = c;
    return PM_OK;
}

// Scene `index` of the batched benchmark: the preset box with 2..32 seeded
// spheres, sigma_s uniform in [0, 0.2], a photon count log-uniform in
// [1e5, 4e6] split evenly between the two maps (no volume map without a
// medium), an image of 256^2, 512^2 or 1024^2 and k of 32, 64 or 128.
pm_status batch_scene(int index, uint64_t seed, pm_scene *scene, pm_config *cfg) {
    if (!scene || !cfg || index < 0) return PM_ERR_INVALID;
    pm_scene s;
    memset(&s, 0, sizeof(s));
    pm_config c;
    memset(&c, 0, sizeof(c));
    base_box(s);
    SplitMix rng{seed ^ (0xBA7C4ull * (uint64_t)(index + 1))};
    const int spheres = 2 + (int)(rng.next() % 31u);
    seeded_spheres(s, spheres, 0.05f, 0.3f, rng);
    s.sigma_s = rng.range(0.0f, 0.2f);
    s.sigma_a = 0.02f;
    s.hg_g = 0.3f;
    const double photons = 1e5 * std::exp(std::log(40.0) * (double)rng.uniform());
    const uint32_t half = (uint32_t)(photons * 0.5);
    c.seed = seed;
    c.scene_id = (uint32_t)index;
    c.surface_photons = half;
    c.volume_photons = s.sigma_s > 0.0f ? half : 0u;
    c.max_bounces = 5;
    c.rr_survival = 0.8f;
    const int res = 256 << (int)(rng.next() % 3u);
    c.width = res;
    c.height = res;
    c.k = 32 << (int)(rng.next() % 3u);
    c.radius = 0.05f;
    c.march_step = 0.01f;
    c.leaf_size = 32;
    c.exposure = 8.0f;
    *scene = s;
    *cfg = c;
    return PM_OK;
}

pm_status validate(const pm_scene &s, const pm_config &c, std::string *why) {
    auto bad = [&](const char *m) { *why = m; return PM_ERR_INVALID; };
    if (s.num_spheres < 0 || s.num_spheres > PM_MAX_SPHERES) return bad("num_spheres out of range");
    if (s.num_planes < 0 || s.num_planes > PM_MAX_PLANES) return bad("num_planes out of range");
    for (int i = 0; i < s.num_planes; ++i) {
        float a = s.planes[i].x;
        if (!(a == 0.0f || a == 1.0f || a == 2.0f)) return bad("plane axis must be 0, 1 or 2");
    }
    for (int a = 0; a < 3; ++a)
        if (!(s.box_max[a] > s.box_min[a])) return bad("empty box");
    for (int i = 0; i < s.num_spheres; ++i)
        if (!(s.spheres[i].w > 0.0f)) return bad("sphere radius must be positive");
    if (!(s.sigma_s >= 0.0f) || !(s.sigma_a >= 0.0f)) return bad("negative medium coefficient");
    if (!(s.hg_g > -1.0f && s.hg_g < 1.0f)) return bad("HG g must be in (-1, 1)");
    if (s.het_res < 0 || s.het_res > 512) return bad("het_res must be in [0, 512]");
    if (s.het_res > 0 && !(s.het_max >= s.het_min && s.het_min >= 0.0f)) return bad("bad het range");
    if (c.max_bounces < 1 || c.max_bounces > 16) return bad("max_bounces must be in [1, 16]");
    if (!(c.rr_survival > 0.0f && c.rr_survival <= 1.0f)) return bad("rr_survival must be in (0, 1]");
    if (c.k < 1 || c.k > 128) return bad("k must be in [1, 128]");
    if (!(c.radius > 0.0f)) return bad("radius must be positive");
    if (c.width < 0 || c.height < 0 || (long long)c.width * c.height > (1ll << 28))
        return bad("image size out of range");
    if (c.leaf_size != 32 && c.leaf_size != 64 && c.leaf_size != 128)
        return bad("leaf_size must be 32, 64 or 128");
    if (!(c.march_step >= 0.0f)) return bad("march_step must be >= 0");
    if (c.march_step > 0.0f && c.march_step < 1e-4f) return bad("march_step below 1e-4");
    return PM_OK;
}

PScene to_device_scene(const pm_scene &s, const float *het_dev) {
    PScene d;
    memset(&d, 0, sizeof(d));
    d.ns = s.num_spheres;
    d.np = s.num_planes;
    for (int i = 0; i < s.num_spheres; ++i) {
        d.sph[i] = s.spheres[i];
        d.sph_kind[i] = s.sphere_mat[i].kind;
        for (int c = 0; c < 3; ++c) d.sph_alb[i][c] = s.sphere_mat[i].albedo[c];
        d.sph_ior[i] = s.sphere_mat[i].ior;
    }
    for (int i = 0; i < s.num_planes; ++i) {
        d.pl_axis[i] = (int)s.planes[i].x;
        d.pl_off[i] = s.planes[i].y;
        d.pl_kind[i] = s.plane_mat[i].kind;
        for (int c = 0; c < 3; ++c) d.pl_alb[i][c] = s.plane_mat[i].albedo[c];
        d.pl_ior[i] = s.plane_mat[i].ior;
    }
    for (int a = 0; a < 3; ++a) {
        d.bmin[a] = s.box_min[a];
        d.bmax[a] = s.box_max[a];
        d.light[a] = s.light[a];
        d.cam[a] = s.cam_pos[a];
    }
    d.sigma_s = s.sigma_s;
    d.sigma_a = s.sigma_a;
    d.g = s.hg_g;
    d.het_res = s.het_res;
    d.het = het_dev;
    d.sigma_max = (s.het_res > 0 ? s.het_max : s.sigma_s) + s.sigma_a;
    d.inv_sigma_max = d.sigma_max > 0.0f ? 1.0f / d.sigma_max : 0.0f;
    for (int a = 0; a < 3; ++a)
        d.het_scale[a] = s.het_res > 0 ? (float)s.het_res / (s.box_max[a] - s.box_min[a]) : 0.0f;
    d.focal = s.focal;
    // Sphere grid for scenes with many spheres, all inside the box (the
    // walk only visits the box): G = ceil(1.5 * cbrt(n)) cells per axis,
    // each sphere's bounding box enlarged by 1e-3 of a cell when binned.
    d.grid_res = 0;
    bool inside = s.num_spheres >= 12;
    for (int i = 0; i < s.num_spheres && inside; ++i)
        for (int a = 0; a < 3; ++a) {
            const float c = a == 0 ? s.spheres[i].x : (a == 1 ? s.spheres[i].y : s.spheres[i].z);
            if (c - s.spheres[i].w < s.box_min[a] || c + s.spheres[i].w > s.box_max[a]) inside = false;
        }
    if (inside) {
        int G = (int)std::ceil(1.5 * std::cbrt((double)s.num_spheres));
        G = G < 2 ? 2 : (G > kGridMax ? kGridMax : G);
        d.grid_res = G;
        double cs[3];
        for (int a = 0; a < 3; ++a) {
            d.grid_inv[a] = (float)G / (s.box_max[a] - s.box_min[a]);
            cs[a] = ((double)s.box_max[a] - s.box_min[a]) / G;
        }
        for (int i = 0; i < s.num_spheres; ++i) {
            int lo[3], hi[3];
            for (int a = 0; a < 3; ++a) {
                const double c = a == 0 ? s.spheres[i].x : (a == 1 ? s.spheres[i].y : s.spheres[i].z);
                const double r = s.spheres[i].w + 1e-3 * cs[a];
                lo[a] = (int)std::floor((c - r - s.box_min[a]) / cs[a]);
                hi[a] = (int)std::floor((c + r - s.box_min[a]) / cs[a]);
                lo[a] = lo[a] < 0 ? 0 : (lo[a] > G - 1 ? G - 1 : lo[a]);
                hi[a] = hi[a] < 0 ? 0 : (hi[a] > G - 1 ? G - 1 : hi[a]);
            }
            for (int z = lo[2]; z <= hi[2]; ++z)
                for (int y = lo[1]; y <= hi[1]; ++y)
                    for (int x = lo[0]; x <= hi[0]; ++x) d.cell_mask[(z * G + y) * G + x] |= 1ull << i;
        }
    }
    return d;
}

namespace {

// Value noise: seeded lattice values on a (L+1)^3 grid, trilinearly
// interpolated at voxel centres, two octaves.
__device__ float lattice(uint64_t seed, uint32_t oct, uint32_t i, uint32_t j, uint32_t k) {
    pm_u32x4 r = philox(seed, i, j, k, 0x4E015E00u + oct);
    return pm_u01(r.v[0]);
}

__device__ float value_noise(uint64_t seed, uint32_t oct, int lat, float x, float y, float z) {
    float fx = x * lat, fy = y * lat, fz = z * lat;
    int ix = min((int)fx, lat - 1), iy = min((int)fy, lat - 1), iz = min((int)fz, lat - 1);
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

__global__ void noise_kernel(float *grid, int res, uint64_t seed, float lo, float hi) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= res * res * res) return;
    int x = v % res, y = (v / res) % res, z = v / (res * res);
    float px = (x + 0.5f) / res, py = (y + 0.5f) / res, pz = (z + 0.5f) / res;
    float n = 0.6666667f * value_noise(seed, 0, 8, px, py, pz) +
              0.3333333f * value_noise(seed, 1, 16, px, py, pz);
    grid[v] = lo + (hi - lo) * n;
}

}  // namespace

cudaError_t make_noise_grid(float *grid, int res, uint64_t seed, float lo, float hi,
                            cudaStream_t s) {
    int n = res * res * res;
    noise_kernel<<<(n + 255) / 256, 256, 0, s>>>(grid, res, seed, lo, hi); note_launch();
    return cudaGetLastError();
}

}  // namespace pm

extern "C" pm_status pm_preset(int which, uint64_t seed, pm_scene *scene, pm_config *cfg) {
    return pm::preset(which, seed, scene, cfg);
}

extern "C" pm_status pm_batch_scene(int index, uint64_t seed, pm_scene *scene, pm_config *cfg) {
    return pm::batch_scene(index, seed, scene, cfg);
}
