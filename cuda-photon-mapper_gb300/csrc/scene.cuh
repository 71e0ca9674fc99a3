// scene.cuh -- scene presets, validation and the device copy of a scene.
#pragma once
#include <string>

#include "phys_common.cuh"

namespace pm {

pm_status preset(int which, uint64_t seed, pm_scene *scene, pm_config *cfg);
pm_status batch_scene(int index, uint64_t seed, pm_scene *scene, pm_config *cfg);
pm_status validate(const pm_scene &s, const pm_config &c, std::string *why);
PScene to_device_scene(const pm_scene &s, const float *het_dev);
// Fills grid[res^3] (x fastest) with seeded value noise scaled to [lo, hi].
cudaError_t make_noise_grid(float *grid, int res, uint64_t seed, float lo, float hi,
                            cudaStream_t s);

}  // namespace pm
