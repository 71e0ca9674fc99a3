// phys_state.cuh -- the physically based mode's per-context state, shared
// by the C ABI implementation files (physical.cu, cache_api.cu).
#pragma once
#include "gather.cuh"
#include "pm.h"

struct PhysicalState {
    pm_scene scene;
    pm_config cfg;
    pm::PScene dscene;
    float *het = nullptr;
    uint32_t path_cap = 0;
    int mb = 0;
    uint32_t *cnt[2] = {nullptr, nullptr};  // records per path, per map
    uint32_t *off[2] = {nullptr, nullptr};  // exclusive scans of cnt
    uint32_t *scan_tmp = nullptr;
    uint32_t *words = nullptr;  // [0] path counter [1] stored_s [2] stored_v [3] total [4..7] extents
    struct Map {
        float4 *pos = nullptr, *pow = nullptr, *tpos = nullptr, *tpow = nullptr;
        float4 *lo = nullptr, *hi = nullptr;
        uint32_t cap = 0, n = 0, paths = 0;
        int depth = 0;
        int leaf_shift = 0;
        bool built = false;
    } map[2];
    uint64_t *keys = nullptr, *keys_tmp = nullptr;
    uint32_t *vals = nullptr, *vals_tmp = nullptr, *hist = nullptr;
    uint32_t sort_cap = 0;
    unsigned long long *gctr = nullptr;
    cudaEvent_t ev[6] = {};  // emit, build, render: start/stop
    pm_frame_stats stats;
    bool emitted = false;
    bool rendered = false;
    int sm_count = 148;
    uint64_t gen = 0;  // bumped whenever the scene or the camera changes
};

namespace pm {

inline MapView view_of(const PhysicalState::Map &m) {
    MapView v;
    v.pos = m.tpos;
    v.pow = m.tpow;
    v.lo = m.lo;
    v.hi = m.hi;
    v.n = m.built ? m.n : 0;
    v.depth = m.depth;
    v.leaf_shift = m.leaf_shift;
    return v;
}

// The render parameters pm_render passes for the installed configuration.
inline RenderParams render_params(const PhysicalState *st) {
    RenderParams R;
    R.width = st->cfg.width;
    R.height = st->cfg.height;
    R.aspect = st->cfg.height > 0 ? (float)st->cfg.width / (float)st->cfg.height : 1.0f;
    R.k = st->cfg.k;
    R.r2cap = st->cfg.radius * st->cfg.radius;
    R.step = st->cfg.march_step;
    R.exposure = st->cfg.exposure;
    R.seed = st->cfg.seed;
    R.scene_id = st->cfg.scene_id;
    R.counters = nullptr;
    return R;
}

}  // namespace pm
