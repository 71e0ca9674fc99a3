/*
 * preset_oracle.c -- the benchmark scenes (presets 1-3 and the batched
 * scenes) restated for the CPU oracle, so that a CPU-only run (the
 * benchmark's reference arm) builds the same scene bytes without loading the
 * product library. TEST INFRASTRUCTURE ONLY.
 *
 * Follows cuda-photon-mapper_gb300/csrc/scene.cu (preset, batch_scene): the
 * same splitmix64 stream (Steele, Lea, Flood, OOPSLA 2014), the same draws in
 * the same order and the same single-precision expressions (compiled with
 * -ffp-contract=off, like the library's host code), so the structs are equal
 * byte for byte (checked against pm_preset in tests/test_physical_oracle.py).
 */
#include <math.h>
#include <string.h>

#include "physical_oracle.h"

typedef struct {
    uint64_t s;
} splitmix;

static uint64_t sm_next(splitmix *r) {
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static float sm_uniform(splitmix *r) { return (float)(sm_next(r) >> 40) * (1.0f / 16777216.0f); }
static float sm_range(splitmix *r, float a, float b) { return a + (b - a) * sm_uniform(r); }

static void set_mat(pmo_material *m, int kind, float r, float g, float b, float ior) {
    m->kind = kind;
    m->albedo[0] = r;
    m->albedo[1] = g;
    m->albedo[2] = b;
    m->ior = ior;
}

/* Unit box open toward the camera: floor, ceiling, red left wall, green
 * right wall, back wall; point light under the ceiling; pinhole camera. */
static void base_box(pmo_scene *s) {
    s->box_min[0] = -0.5f; s->box_min[1] = 0.0f; s->box_min[2] = -0.5f;
    s->box_max[0] = 0.5f;  s->box_max[1] = 1.0f; s->box_max[2] = 0.5f;
    s->num_planes = 5;
    const float planes[5][2] = {{1.0f, 0.0f}, {1.0f, 1.0f}, {0.0f, -0.5f}, {0.0f, 0.5f}, {2.0f, 0.5f}};
    memcpy(s->planes, planes, sizeof(planes));
    set_mat(&s->plane_mat[0], PMO_MAT_DIFFUSE, 0.75f, 0.75f, 0.75f, 1.0f);
    set_mat(&s->plane_mat[1], PMO_MAT_DIFFUSE, 0.75f, 0.75f, 0.75f, 1.0f);
    set_mat(&s->plane_mat[2], PMO_MAT_DIFFUSE, 0.75f, 0.25f, 0.25f, 1.0f);
    set_mat(&s->plane_mat[3], PMO_MAT_DIFFUSE, 0.25f, 0.75f, 0.25f, 1.0f);
    set_mat(&s->plane_mat[4], PMO_MAT_DIFFUSE, 0.75f, 0.75f, 0.75f, 1.0f);
    s->light[0] = 0.0f; s->light[1] = 0.95f; s->light[2] = 0.0f;
    s->light_power = 1.0f;
    s->cam_pos[0] = 0.0f; s->cam_pos[1] = 0.5f; s->cam_pos[2] = -1.5f;
    s->focal = 1.0f;
}

/* Seeded spheres: radius uniform in [rmin, rmax], centre uniform in the box
 * shrunk by the radius, up to 64 attempts to stay clear of the light and the
 * earlier spheres; 50 % diffuse (seeded albedo), 25 % mirror, 25 %
 * dielectric (ior 1.5). */
static void seeded_spheres(pmo_scene *s, int count, float rmin, float rmax, splitmix *rng) {
    s->num_spheres = 0;
    for (int i = 0; i < count; ++i) {
        float r = sm_range(rng, rmin, rmax), cx = 0, cy = 0, cz = 0;
        for (int attempt = 0; attempt < 64; ++attempt) {
            cx = sm_range(rng, s->box_min[0] + r, s->box_max[0] - r);
            cy = sm_range(rng, s->box_min[1] + r, s->box_max[1] - r);
            cz = sm_range(rng, s->box_min[2] + r, s->box_max[2] - r);
            float lx = cx - s->light[0], ly = cy - s->light[1], lz = cz - s->light[2];
            int ok = sqrtf(lx * lx + ly * ly + lz * lz) > r + 0.02f;
            for (int j = 0; ok && j < s->num_spheres; ++j) {
                float dx = cx - s->spheres[j][0], dy = cy - s->spheres[j][1], dz = cz - s->spheres[j][2];
                ok = sqrtf(dx * dx + dy * dy + dz * dz) > r + s->spheres[j][3];
            }
            if (ok || attempt == 63) {
                if (!ok) {
                    float lx2 = cx - s->light[0], ly2 = cy - s->light[1], lz2 = cz - s->light[2];
                    if (sqrtf(lx2 * lx2 + ly2 * ly2 + lz2 * lz2) <= r + 0.02f) cy = s->box_min[1] + r;
                }
                break;
            }
        }
        s->spheres[i][0] = cx;
        s->spheres[i][1] = cy;
        s->spheres[i][2] = cz;
        s->spheres[i][3] = r;
        float pick = sm_uniform(rng);
        if (pick < 0.5f) {
            float a = sm_range(rng, 0.2f, 0.9f);
            float b = sm_range(rng, 0.2f, 0.9f);
            float c = sm_range(rng, 0.2f, 0.9f);
            set_mat(&s->sphere_mat[i], PMO_MAT_DIFFUSE, a, b, c, 1.0f);
        } else if (pick < 0.75f) {
            set_mat(&s->sphere_mat[i], PMO_MAT_MIRROR, 1.0f, 1.0f, 1.0f, 1.0f);
        } else {
            set_mat(&s->sphere_mat[i], PMO_MAT_DIELECTRIC, 1.0f, 1.0f, 1.0f, 1.5f);
        }
        s->num_spheres = i + 1;
    }
}

int pmo_preset(int which, uint64_t seed, pmo_scene *scene, pmo_config *cfg) {
    if (!scene || !cfg || which < 1 || which > 3) return -1;
    pmo_scene s;
    pmo_config c;
    memset(&s, 0, sizeof(s));
    memset(&c, 0, sizeof(c));
    base_box(&s);
    s.sigma_s = 0.1f;
    s.sigma_a = 0.02f;
    s.hg_g = 0.3f;
    c.seed = seed;
    c.scene_id = 0;
    c.rr_survival = 0.8f;
    c.leaf_size = 32;
    c.exposure = 8.0f;
    splitmix rng = {seed ^ (0xC0FFEEull * (uint64_t)which)};
    if (which == 1) {
        s.num_spheres = 2;
        const float sp[2][4] = {{-0.2f, 0.3f, 0.1f, 0.3f}, {0.24f, 0.25f, -0.2f, 0.25f}};
        memcpy(s.spheres, sp, sizeof(sp));
        set_mat(&s.sphere_mat[0], PMO_MAT_DIFFUSE, 0.75f, 0.75f, 0.75f, 1.0f);
        set_mat(&s.sphere_mat[1], PMO_MAT_MIRROR, 1.0f, 1.0f, 1.0f, 1.0f);
        c.surface_photons = 100000;
        c.volume_photons = 100000;
        c.max_bounces = 5;
        c.width = 512; c.height = 512;
        c.k = 64; c.radius = 0.1f;
        c.march_step = 0.01f;
    } else if (which == 2) {
        seeded_spheres(&s, 8, 0.05f, 0.3f, &rng);
        c.surface_photons = 1000000;
        c.volume_photons = 1000000;
        c.max_bounces = 5;
        c.width = 1024; c.height = 1024;
        c.k = 100; c.radius = 0.05f;
        c.march_step = 0.01f;
    } else {
        seeded_spheres(&s, 64, 0.05f, 0.3f, &rng);
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
    return 0;
}
