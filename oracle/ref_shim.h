/*
 * ref_shim.h -- lets the reference's device code (photonMappingKernel.cu,
 * lines 6-1521) compile as plain serial C++ on the host.
 *
 * TEST INFRASTRUCTURE ONLY. This header is used by oracle/ref_harness.cpp,
 * which oracle/ref.mk builds into oracle/_ref/libpmref.so from the
 * reference's own source file. Nothing in the product links it.
 *
 * The reference includes the CUDA SDK 3.x `cutil_math.h` for its float3
 * arithmetic (photonMappingKernel.cu:4). cutil is not vendored and not
 * present in this image, so the vector operations below are written from
 * that header's documented host-path behaviour:
 *   - component-wise +, -, * and scalar broadcast,
 *   - float3 / s computed as a * (1.0f / s),
 *   - normalize(v) = v * rsqrtf(dot(v, v)) with the host rsqrtf
 *     defined as 1.0f / sqrtf(x),
 *   - dot(a, b) = a.x*b.x + a.y*b.y + a.z*b.z, evaluated left to right.
 * The product kernels use exactly these definitions, so results agree bit
 * for bit; whether the original cutil agreed in the last ulp is not
 * pinned by any file in the reference.
 *
 * Build with -ffp-contract=off: every float expression must round after
 * each operation (no fused multiply-add), as the product kernels do.
 */
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <climits>

#define __device__
#define __global__
#define __host__
#define __shared__

typedef unsigned int uint;

struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct int3 { int x, y, z; };
struct uchar4 { unsigned char x, y, z, w; };
struct dim3 { unsigned int x, y, z; };

/* CUDA launch coordinates; the harness sets them before calling a
 * __global__ body as an ordinary function. */
extern dim3 blockIdx, blockDim, threadIdx;

static inline void __threadfence() {}

/* checkCUDAError (photonMappingKernel.cu:49-55) needs these names. */
typedef int cudaError_t;
static const cudaError_t cudaSuccess = 0;
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
static inline const char *cudaGetErrorString(cudaError_t) { return "no error"; }

/* Double-to-int conversion with the GPU's defined behaviour (NaN -> 0,
 * saturate at the int range); in range it truncates like a C cast. */
static inline int shim_d2i(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return INT_MAX;
    if (v <= -2147483648.0) return INT_MIN;
    return (int)v;
}

static inline float2 make_float2(float x, float y) { float2 r = {x, y}; return r; }
static inline float3 shim_f3(float x, float y, float z) { float3 r = {x, y, z}; return r; }
static inline float4 make_float4(float x, float y, float z, float w) { float4 r = {x, y, z, w}; return r; }
static inline int3 make_int3(int x, int y, int z) { int3 r = {x, y, z}; return r; }
static inline int3 make_int3(double x, double y, double z) {
    int3 r = {shim_d2i(x), shim_d2i(y), shim_d2i(z)};
    return r;
}

static inline float3 operator+(float3 a, float3 b) { return shim_f3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline float3 operator-(float3 a, float3 b) { return shim_f3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline float3 operator-(float3 a, float b) { return shim_f3(a.x - b, a.y - b, a.z - b); }
static inline float3 operator+(float3 a, float b) { return shim_f3(a.x + b, a.y + b, a.z + b); }
static inline float3 operator*(float3 a, float s) { return shim_f3(a.x * s, a.y * s, a.z * s); }
static inline float3 operator*(float s, float3 a) { return shim_f3(a.x * s, a.y * s, a.z * s); }
static inline float3 operator/(float3 a, float s) { float inv = 1.0f / s; return a * inv; }
static inline void operator+=(float3 &a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
static inline void operator-=(float3 &a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }

static inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float shim_rsqrtf(float x) { return 1.0f / sqrtf(x); }
static inline float3 normalize(float3 v) { float inv = shim_rsqrtf(dot(v, v)); return v * inv; }

/* CUDA's min/max on floats behave like fminf/fmaxf. */
static inline float min(float a, float b) { return fminf(a, b); }
static inline float max(float a, float b) { return fmaxf(a, b); }
static inline double min(double a, float b) { return fmin(a, (double)b); }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }

/* pow(radius, 2.0f) (photonMappingKernel.cu:118): the square of a float,
 * rounded once. */
static inline float shim_powf(float x, float y) {
    if (y == 2.0f) return x * x;
    return powf(x, y);
}
#define pow(a, b) shim_powf((float)(a), (float)(b))

/* make_float3 evaluates its three arguments left to right, as device code
 * built by nvcc does. The order matters only in rand3
 * (photonMappingKernel.cu:1054-1056), whose arguments each draw from the
 * shared generator; g++ would otherwise evaluate them right to left. A
 * braced initialiser list is sequenced left to right by the language. */
#define make_float3(a, b, c) (float3{(float)(a), (float)(b), (float)(c)})

using std::sqrt;
using std::cos;
using std::sin;
