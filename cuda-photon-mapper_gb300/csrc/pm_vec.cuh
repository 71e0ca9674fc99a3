// pm_vec.cuh -- float3 arithmetic shared by the host and device code.
//
// Every operation rounds once (the library is compiled with -fmad=false,
// so no multiply-add is fused unless written as fmaf). The helpers follow
// the vector semantics the reference's kernels were written against
// (cutil_math.h, photonMappingKernel.cu:4): scalar division multiplies by
// 1.0f/s and normalize multiplies by 1.0f/sqrtf(dot(v, v)), with IEEE
// division and square root on both sides.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define PM_HD __host__ __device__ __forceinline__
#else
#define PM_HD inline
#endif

namespace pm {

struct v3 {
    float x, y, z;
};

PM_HD v3 mk3(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
PM_HD v3 operator+(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
PM_HD v3 operator-(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
PM_HD v3 operator*(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
PM_HD v3 sub_scalar(v3 a, float s) { return mk3(a.x - s, a.y - s, a.z - s); }
PM_HD v3 div_scalar(v3 a, float s) { float inv = 1.0f / s; return a * inv; }
PM_HD float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PM_HD v3 normalize(v3 v) { float inv = 1.0f / sqrtf(dot(v, v)); return v * inv; }
PM_HD float axis_of(v3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
PM_HD void set_axis(v3 &v, int a, float s) {
    if (a == 0) v.x = s; else if (a == 1) v.y = s; else v.z = s;
}

// Double to int with the GPU's conversion rule, written out so that host
// and device agree: NaN gives 0, values beyond the int range saturate,
// everything else truncates toward zero.
PM_HD int d2i_sat(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return 2147483647;
    if (v <= -2147483648.0) return -2147483647 - 1;
    return (int)v;
}

// 8-bit channel from a radiance value already scaled by 255: NaN and
// values <= 0 give 0, values above 255 give 255, the rest truncate.
PM_HD unsigned char to_u8_sat(double v) {
    double c = v > 255.0 ? 255.0 : v;
    if (!(c > 0.0)) return 0;
    return (unsigned char)(int)c;
}

}  // namespace pm
