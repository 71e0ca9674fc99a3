// launch_count.cuh -- process-wide count of kernels this library launched
// (read through pm_kernel_launches), so a benchmark can state how many of
// its kernels ran inside a timed region.
#pragma once
#include <atomic>

namespace pm {

inline std::atomic<unsigned long long> &launch_counter() {
    static std::atomic<unsigned long long> c{0};
    return c;
}

inline void note_launch() { launch_counter().fetch_add(1, std::memory_order_relaxed); }
// Kernels of a replayed CUDA graph (counted when the graph was captured).
inline void note_launches(unsigned long long n) {
    launch_counter().fetch_add(n, std::memory_order_relaxed);
}

}  // namespace pm
