// eye_path.cuh -- the eye path of one pixel as a list of radiance queries.
//
// The render kernel estimates, along the pixel's eye ray and its specular
// continuations, the in-scattered radiance at every march sample of the
// medium and the reflected radiance at the first diffuse hit, each scaled by
// the transmittance in front of it. walk_eye() replays exactly that path --
// the same pixel mapping, intersections, march segments, Fresnel choices
// (same Philox counters) and transmittance updates -- and hands every query
// to a sink instead of gathering photons, so that the frame can be rendered
// as (query list) -> (per-query estimate from the photon map or the learned
// cache) -> (ordered per-pixel sum).
#pragma once
#include "gather.cuh"
#include "phys_common.cuh"

namespace pm {

constexpr int kMaxSpecular = 8;
constexpr uint32_t kEyeSalt = 0xE7E5A17Bu;
constexpr int kMaxMarchSteps = 1 << 16;  // per segment

// Sink interface:
//   void volume(v3 x, v3 wo, float w)         in-scattering query, w = T(mid) * dt
//   void surface(v3 x, int obj, v3 wo, float w) diffuse query,   w = T(hit)
//   static constexpr bool kCountOnly          true: volume_steps(n) replaces the
//   void volume_steps(int n)                  n volume() calls of a march segment
// (the path itself never depends on the transmittance, so a counting sink
// needs no march step).
template <class Sink>
__device__ __forceinline__ void walk_eye(const PScene &Sc, const RenderParams &R, uint32_t pix,
                                         bool vol_on, bool surf_on, Sink &sink) {
    const uint32_t px = pix % (uint32_t)R.width, py = pix / (uint32_t)R.width;
    const float u = ((float)px / (float)R.width - 0.5f) * R.aspect;
    const float v = -((float)py / (float)R.height - 0.5f);
    v3 o = mk3(Sc.cam[0], Sc.cam[1], Sc.cam[2]);
    v3 d = normalize(mk3(u, v, Sc.focal));
    float tau = 0.0f;
    bool glass = false;
    for (int depth = 0; depth < kMaxSpecular; ++depth) {
        PHit h = intersect(Sc, o, d, 3.0e38f);
        const float tend = h.obj != kNone ? h.t : 3.0e38f;
        if (R.step > 0.0f && Sc.sigma_max > 0.0f && !glass) {
            float t0, t1;
            box_span(Sc, o, d, &t0, &t1);
            t1 = fminf(t1, tend);
            if (t0 < t1) {
                const int nst = (int)fminf(ceilf((t1 - t0) / R.step), (float)kMaxMarchSteps);
                const v3 wo = d * -1.0f;
                if constexpr (Sink::kCountOnly) {
                    if (vol_on) sink.volume_steps(nst);
                } else for (int j = 0; j < nst; ++j) {
                    const float ta = t0 + (float)j * R.step;
                    const float tb = fminf(t0 + (float)(j + 1) * R.step, t1);
                    const float dt = tb - ta;
                    const float tm = 0.5f * (ta + tb);
                    const v3 x = o + d * tm;
                    const float ss = Sc.het_res > 0 ? sigma_s_at(Sc, x) : Sc.sigma_s;
                    const float st = ss + Sc.sigma_a;
                    const float tau_mid = tau + st * (0.5f * dt);
                    if (vol_on) sink.volume(x, wo, pm_expf(-tau_mid) * dt);
                    tau = tau + st * dt;
                }
            }
        }
        if (h.obj == kNone) break;
        const v3 hp = o + d * h.t;
        const v3 n = outward_normal(Sc, h.obj, hp);
        const int kind = material_kind(Sc, h.obj);
        const float dn = dot(n, d);
        const v3 nf = dn < 0.0f ? n : n * -1.0f;
        if (kind == PM_MAT_DIFFUSE) {
            if (surf_on) sink.surface(hp, h.obj, d * -1.0f, pm_expf(-tau));
            break;
        }
        if (kind == PM_MAT_MIRROR) {
            d = normalize(d - n * (2.0f * dn));
            o = hp + nf * kOffset;
        } else {
            float ci = -dn;
            const bool entering = ci > 0.0f;
            const float ior = material_ior(Sc, h.obj);
            const float eta = entering ? 1.0f / ior : ior;
            const v3 nn = entering ? n : n * -1.0f;
            ci = fabsf(ci);
            float ct;
            const float F = fresnel(ci, eta, &ct);
            pm_u32x4 r = philox(R.seed, pix, (uint32_t)depth, kEyeSalt, R.scene_id);
            if (pm_u01(r.v[0]) < F) {
                d = normalize(d + nn * (2.0f * ci));
                o = hp + nn * kOffset;
            } else {
                d = normalize(d * eta + nn * (eta * ci - ct));
                o = hp - nn * kOffset;
                glass = entering;
            }
        }
    }
}

// Facing normal of a diffuse query: the render's nf for the hit on `obj`
// at x seen along -wo.
__device__ __forceinline__ v3 facing_normal(const PScene &Sc, int obj, v3 x, v3 wo) {
    const v3 n = outward_normal(Sc, obj, x);
    const v3 d = wo * -1.0f;
    return dot(n, d) < 0.0f ? n : n * -1.0f;
}

}  // namespace pm
