/*
 * cutil_math.h (shim) -- the float3 arithmetic the reference's CUDA file
 * includes (photonMappingKernel.cu:4), for building that file's GPU code
 * here as the measured reference-GPU bar of the legacy frame.
 *
 * TEST / MEASUREMENT INFRASTRUCTURE ONLY: used by the recipe in
 * cuda-photon-mapper_gb300/build.py that compiles the reference's own
 * photonMappingKernel.cu into oracle/_ref/ref_kernels.cubin. Nothing in the
 * product includes it.
 *
 * The CUDA SDK 3.x header is not vendored and not in this image; these
 * are the same definitions as oracle/ref_shim.h (the reference built for
 * the CPU) and the legacy kernels: component-wise +, -, *, scalar
 * broadcast, v / s as v * (1 / s), dot evaluated left to right, and
 * normalize(v) = v * (1 / sqrtf(dot(v, v))).
 */
#pragma once
#include <cuda_runtime.h>

inline __host__ __device__ float3 operator+(float3 a, float3 b) {
    return make_float3(a.x + b.x, a.y + b.y, a.z + b.z);
}
inline __host__ __device__ float3 operator-(float3 a, float3 b) {
    return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
inline __host__ __device__ float3 operator+(float3 a, float b) { return make_float3(a.x + b, a.y + b, a.z + b); }
inline __host__ __device__ float3 operator-(float3 a, float b) { return make_float3(a.x - b, a.y - b, a.z - b); }
inline __host__ __device__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
inline __host__ __device__ float3 operator*(float s, float3 a) { return make_float3(a.x * s, a.y * s, a.z * s); }
inline __host__ __device__ float3 operator/(float3 a, float s) {
    const float inv = 1.0f / s;
    return a * inv;
}
inline __host__ __device__ void operator+=(float3 &a, float3 b) {
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
}
inline __host__ __device__ void operator-=(float3 &a, float3 b) {
    a.x -= b.x;
    a.y -= b.y;
    a.z -= b.z;
}
inline __host__ __device__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline __host__ __device__ float3 normalize(float3 v) {
    const float inv = 1.0f / sqrtf(dot(v, v));
    return v * inv;
}
