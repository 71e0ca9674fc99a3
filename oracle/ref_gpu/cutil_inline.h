/*
 * cutil_inline.h (shim) -- the one name the reference's CUDA file takes
 * from this SDK header: cudaThreadSynchronize (photonMappingKernel.cu:1532,
 * 1543,1563,1579), removed from CUDA 13 and equivalent to
 * cudaDeviceSynchronize. Measurement infrastructure only (see
 * cutil_math.h beside it).
 */
#pragma once
#include <cuda_runtime.h>
#define cudaThreadSynchronize cudaDeviceSynchronize
