// host_tools.cu -- host-side utilities around the photon mapper: photon-map
// files, PPM and PNG image output and a headless frame driver with the reference's
// display()/keyboard() semantics.
#include "pm.h"
#include "pm_ctx.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

const char kMapMagic[] = "{\"format\": \"pm-photon-map\", \"version\": 1";

}  // namespace

extern "C" {

// File = one JSON header line, then `records` float4 pos followed by
// `records` float4 pow (the SoA layout of pm_get_photons_soa).
pm_status pm_save_map(pm_ctx *ctx, int map, const char *path) {
    if (!ctx || !path || map < 0 || map > 1) return PM_ERR_INVALID;
    uint32_t n = 0;
    pm_status s = pm_get_photons_soa(ctx, map, nullptr, nullptr, 0, &n);
    if (s != PM_OK) return s;
    std::vector<float4> pos(n), pw(n);
    s = pm_get_photons_soa(ctx, map, pos.data(), pw.data(), n, &n);
    if (s != PM_OK) return s;
    pm_frame_stats st;
    if (pm_get_stats(ctx, &st) != PM_OK) memset(&st, 0, sizeof(st));
    FILE *f = fopen(path, "wb");
    if (!f) return pm::fail(ctx, PM_ERR_INVALID, std::string("cannot open ") + path);
    fprintf(f,
            "%s, \"map\": \"%s\", \"records\": %u, \"paths\": %u, \"layout\": \"float4 pos (xyz, "
            "index bits) x records, float4 pow (rgb flux, octahedral 16:16 direction) x records\"}\n",
            kMapMagic, map == 0 ? "surface" : "volume", n, st.map_paths[map]);
    bool ok = fwrite(pos.data(), sizeof(float4), n, f) == n && fwrite(pw.data(), sizeof(float4), n, f) == n;
    ok = (fclose(f) == 0) && ok;
    return ok ? PM_OK : pm::fail(ctx, PM_ERR_INVALID, "short write");
}

pm_status pm_load_map(pm_ctx *ctx, int map, const char *path) {
    if (!ctx || !path || map < 0 || map > 1) return PM_ERR_INVALID;
    FILE *f = fopen(path, "rb");
    if (!f) return pm::fail(ctx, PM_ERR_INVALID, std::string("cannot open ") + path);
    char line[1024];
    if (!fgets(line, sizeof(line), f) || strncmp(line, kMapMagic, strlen(kMapMagic)) != 0) {
        fclose(f);
        return pm::fail(ctx, PM_ERR_INVALID, "not a photon-map file");
    }
    const char *r = strstr(line, "\"records\": ");
    unsigned n = 0;
    if (!r || sscanf(r + 11, "%u", &n) != 1) {
        fclose(f);
        return pm::fail(ctx, PM_ERR_INVALID, "header without a record count");
    }
    std::vector<float4> pos(n), pw(n);
    bool ok = fread(pos.data(), sizeof(float4), n, f) == n && fread(pw.data(), sizeof(float4), n, f) == n;
    fclose(f);
    if (!ok) return pm::fail(ctx, PM_ERR_INVALID, "truncated photon-map file");
    return pm_set_photons(ctx, map, pos.data(), pw.data(), n);
}

pm_status pm_write_ppm(const char *path, const uchar4 *rgba, unsigned width, unsigned height) {
    if (!path || (!rgba && width && height)) return PM_ERR_INVALID;
    FILE *f = fopen(path, "wb");
    if (!f) return PM_ERR_INVALID;
    fprintf(f, "P6\n%u %u\n255\n", width, height);
    std::vector<unsigned char> row(3 * (size_t)width);
    bool ok = true;
    for (unsigned y = 0; y < height && ok; ++y) {
        for (unsigned x = 0; x < width; ++x) {
            const uchar4 &p = rgba[(size_t)y * width + x];
            row[3 * x] = p.x;
            row[3 * x + 1] = p.y;
            row[3 * x + 2] = p.z;
        }
        ok = fwrite(row.data(), 1, row.size(), f) == row.size();
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? PM_OK : PM_ERR_INVALID;
}

// ---- PNG (ISO/IEC 15948): RGB 8-bit, the zlib stream in stored deflate blocks ----
// (RFC 1950 / 1951), so no compression library is needed: the file is the
// image's bytes plus framing, readable by any PNG decoder.

namespace {

uint32_t crc32_update(uint32_t crc, const unsigned char *p, size_t n) {
    static uint32_t table[256];
    static bool ready = false;
    if (!ready) {  // the reflected CRC-32 polynomial 0xEDB88320 (ISO 3309)
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        ready = true;
    }
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
    return crc;
}

void put_be32(std::vector<unsigned char> &v, uint32_t x) {
    v.push_back((unsigned char)(x >> 24));
    v.push_back((unsigned char)(x >> 16));
    v.push_back((unsigned char)(x >> 8));
    v.push_back((unsigned char)x);
}

bool write_chunk(FILE *f, const char *type, const std::vector<unsigned char> &data) {
    std::vector<unsigned char> head;
    put_be32(head, (uint32_t)data.size());
    head.insert(head.end(), type, type + 4);
    uint32_t crc = crc32_update(0xffffffffu, head.data() + 4, 4);
    crc = crc32_update(crc, data.data(), data.size()) ^ 0xffffffffu;
    std::vector<unsigned char> tail;
    put_be32(tail, crc);
    return fwrite(head.data(), 1, head.size(), f) == head.size() &&
           (data.empty() || fwrite(data.data(), 1, data.size(), f) == data.size()) &&
           fwrite(tail.data(), 1, 4, f) == 4;
}

}  // namespace

pm_status pm_write_png(const char *path, const uchar4 *rgba, unsigned width, unsigned height) {
    if (!path || !width || !height || !rgba) return PM_ERR_INVALID;
    const size_t row = 1 + 3 * (size_t)width;  // filter byte 0, then RGB
    const size_t raw = row * height;
    if (row > 0x7fffffffu || raw > ((size_t)1 << 31)) return PM_ERR_LIMIT;
    // the scanlines (filter type 0)
    std::vector<unsigned char> img(raw);
    for (unsigned y = 0; y < height; ++y) {
        unsigned char *r = img.data() + y * row;
        r[0] = 0;
        for (unsigned x = 0; x < width; ++x) {
            const uchar4 &p = rgba[(size_t)y * width + x];
            r[1 + 3 * x] = p.x;
            r[2 + 3 * x] = p.y;
            r[3 + 3 * x] = p.z;
        }
    }
    // zlib stream: header 0x78 0x01, stored blocks of <= 65535 bytes, Adler-32
    std::vector<unsigned char> z;
    z.reserve(raw + raw / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    for (size_t at = 0; at < raw || raw == 0;) {
        const size_t len = std::min<size_t>(65535, raw - at);
        const bool last = at + len == raw;
        z.push_back(last ? 1 : 0);
        z.push_back((unsigned char)(len & 0xff));
        z.push_back((unsigned char)(len >> 8));
        z.push_back((unsigned char)(~len & 0xff));
        z.push_back((unsigned char)((~len >> 8) & 0xff));
        z.insert(z.end(), img.begin() + at, img.begin() + at + len);
        at += len;
        if (last) break;
    }
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < raw; ++i) {
        a = (a + img[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);
    std::vector<unsigned char> ihdr;
    put_be32(ihdr, width);
    put_be32(ihdr, height);
    const unsigned char rest[5] = {8, 2, 0, 0, 0};  // 8-bit, truecolour, deflate, filter 0, no interlace
    ihdr.insert(ihdr.end(), rest, rest + 5);
    FILE *f = fopen(path, "wb");
    if (!f) return PM_ERR_INVALID;
    static const unsigned char sig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
    bool ok = fwrite(sig, 1, 8, f) == 8 && write_chunk(f, "IHDR", ihdr) && write_chunk(f, "IDAT", z) &&
              write_chunk(f, "IEND", {});
    ok = (fclose(f) == 0) && ok;
    return ok ? PM_OK : PM_ERR_INVALID;
}

// ---- headless frame driver (callbacksPBO.cpp:19-27, 47-101, 104-143) --------

struct pm_viewer {
    pm_viewer_state s;
    pm_ctx *ctx;
    bool started;
};

pm_status pm_viewer_create(pm_viewer **out, unsigned width, unsigned height) {
    if (!out) return PM_ERR_INVALID;
    pm_viewer *v = new pm_viewer();
    memset(&v->s, 0, sizeof(v->s));
    v->s.width = width;
    v->s.height = height;
    v->s.anim_flag = 0;       // animFlag
    v->s.emit_flag = 1;       // emitFlag
    v->s.interpolate = 0;     // interpolateFlag
    v->s.media = 0;           // participatingMediaFlag
    v->s.iter = 0;
    v->s.anim_time = 0.0f;
    v->s.anim_inc = 0.1f;
    v->ctx = nullptr;
    v->started = false;
    *out = v;
    return PM_OK;
}

void pm_viewer_destroy(pm_viewer *v) {
    if (!v) return;
    pm_destroy(v->ctx);
    delete v;
}

void pm_viewer_key(pm_viewer *v, unsigned char key) {
    if (!v) return;
    pm_viewer_state &s = v->s;
    switch (key) {
        case 27: s.quit = 1; break;  // the reference exits the process here
        case 'a': case 'A': s.anim_flag = s.anim_flag ? 0 : 1; break;
        case 'e': case 'E': s.emit_flag = s.emit_flag ? 0 : 1; break;
        case 'i': case 'I': s.interpolate = !s.interpolate; break;
        case 'p': case 'P': s.media = !s.media; break;
        case '-': s.anim_inc = (float)((double)s.anim_inc - 0.01); break;
        case '+': s.anim_inc = (float)((double)s.anim_inc + 0.01); break;
        case 'r': s.anim_inc = 0.01f; break;
        default: break;
    }
}

pm_status pm_viewer_state_get(const pm_viewer *v, pm_viewer_state *out) {
    if (!v || !out) return PM_ERR_INVALID;
    *out = v->s;
    return PM_OK;
}

pm_status pm_viewer_display(pm_viewer *v, uchar4 *pos) {
    if (!v) return PM_ERR_INVALID;
    pm_status st;
    if (!v->started) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) {
            cudaGetLastError();
            return PM_ERR_CUDA;
        }
        if ((st = pm_create(&v->ctx, dev)) != PM_OK) return st;
        // initCuda runs one emission before the first display
        // (simplePBO.cpp:203), before the random table exists.
        if ((st = pm_legacy_emit(v->ctx, v->s.anim_time, 0, 0)) != PM_OK) return st;
        v->started = true;
    }
    pm_viewer_state &s = v->s;
    const int flags = (s.interpolate ? PM_LEGACY_INTERPOLATE : 0) | (s.media ? PM_LEGACY_MEDIA : 0);
    if (s.iter == 0) {
        if ((st = pm_legacy_init_random(v->ctx, 0)) != PM_OK) return st;
        s.iter++;
    }
    if (s.emit_flag && (st = pm_legacy_emit(v->ctx, s.anim_time, flags, 0)) != PM_OK) return st;
    if ((st = pm_legacy_render(v->ctx, pos, s.width, s.height, s.anim_time, flags, nullptr, 0)) != PM_OK)
        return st;
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        return PM_ERR_CUDA;
    }
    s.frames++;
    if (s.anim_flag) s.anim_time += s.anim_inc;
    return PM_OK;
}

// ---- physically based frame driver (the same loop over pm_emit / pm_build /
// pm_render, with temporal reuse) -------------------------------------------

struct pm_phys_viewer {
    pm_phys_viewer_state s;
    pm_ctx *ctx;
    pm_scene base;       // the scene as installed; animation moves sphere 0 from here
    pm_scene current;    // the scene of the last emission
    bool have_maps;
};

pm_status pm_phys_viewer_create(pm_ctx *ctx, const pm_scene *scene, const pm_config *cfg,
                                pm_phys_viewer **out) {
    if (!ctx || !scene || !cfg || !out) return PM_ERR_INVALID;
    pm_status st = pm_set_scene(ctx, scene, cfg);
    if (st != PM_OK) return st;
    pm_phys_viewer *v = new pm_phys_viewer();
    memset(&v->s, 0, sizeof(v->s));
    v->s.anim_flag = 0;
    v->s.emit_flag = 0;  // an unchanged scene gives the same maps: reuse them
    v->s.use_cache = 1;
    v->s.cache_frames = 1;
    v->s.anim_time = 0.0f;
    v->s.anim_inc = 0.1f;
    v->s.anim_radius = 0.05f;
    v->ctx = ctx;
    v->base = *scene;
    v->current = *scene;
    v->have_maps = false;
    *out = v;
    return PM_OK;
}

void pm_phys_viewer_destroy(pm_phys_viewer *v) { delete v; }

void pm_phys_viewer_key(pm_phys_viewer *v, unsigned char key) {
    if (!v) return;
    pm_phys_viewer_state &s = v->s;
    switch (key) {
        case 27: s.quit = 1; break;
        case 'a': case 'A': s.anim_flag = s.anim_flag ? 0 : 1; break;
        case 'e': case 'E': s.emit_flag = s.emit_flag ? 0 : 1; break;
        case 'c': case 'C': s.use_cache = s.use_cache ? 0 : 1; break;
        case '-': s.anim_inc = (float)((double)s.anim_inc - 0.01); break;
        case '+': s.anim_inc = (float)((double)s.anim_inc + 0.01); break;
        case 'r': s.anim_inc = 0.01f; break;
        default: break;
    }
}

pm_status pm_phys_viewer_state_get(const pm_phys_viewer *v, pm_phys_viewer_state *out) {
    if (!v || !out) return PM_ERR_INVALID;
    *out = v->s;
    return PM_OK;
}

pm_status pm_phys_viewer_display(pm_phys_viewer *v, float4 *radiance, uchar4 *rgba,
                                 cudaStream_t stream) {
    if (!v) return PM_ERR_INVALID;
    pm_phys_viewer_state &s = v->s;
    pm_status st;
    // the frame's scene: sphere 0 displaced along x by anim_radius *
    // sin(anim_time), kept inside the box
    pm_scene sc = v->base;
    if (sc.num_spheres > 0 && s.anim_time != 0.0f) {
        float4 &p = sc.spheres[0];
        const float lo = sc.box_min[0] + p.w, hi = sc.box_max[0] - p.w;
        p.x = fminf(fmaxf(p.x + s.anim_radius * sinf(s.anim_time), lo), hi);
    }
    const bool changed = memcmp(&sc, &v->current, sizeof(sc)) != 0;
    if (changed && (st = pm_update_scene(v->ctx, &sc)) != PM_OK) return st;
    if (!v->have_maps || changed || s.emit_flag) {
        if ((st = pm_emit(v->ctx, stream)) != PM_OK) return st;
        if ((st = pm_build(v->ctx, stream)) != PM_OK) return st;
        v->current = sc;
        v->have_maps = true;
        s.emissions++;
    } else {
        s.reuses++;
    }
    const bool cached = s.use_cache && v->ctx->cache != nullptr;
    if (cached) {
        if (s.cache_frames > 0 && (st = pm_cache_train(v->ctx, s.cache_frames, stream)) != PM_OK) return st;
        if ((st = pm_render_cached(v->ctx, radiance, rgba, 0, stream)) != PM_OK) return st;
        s.cached_frames++;
    } else if ((st = pm_render(v->ctx, radiance, rgba, stream)) != PM_OK) {
        return st;
    }
    s.frames++;
    if (s.anim_flag) s.anim_time += s.anim_inc;
    return PM_OK;
}

}  // extern "C"
