/*
 * Force-included header for compiling the reference tracer's frame kernels
 * (src/CUDA/Kernel.cu) with nvcc. TEST INFRASTRUCTURE ONLY (oracle): used by
 * the recipe in oracle/ref_build.py that builds the reference's own GPU frame
 * for a golden fixture; nothing in the product library includes it.
 *
 * The reference was written for MSVC, where std::cosf/std::sinf exist (used by
 * unused helpers in Core/Random.cuh); these forward to the global functions,
 * on the host and on the device.
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
using std::abs;
using std::fabs;
using std::sqrt;
namespace std {
__host__ __device__ inline float cosf(float x) { return ::cosf(x); }
__host__ __device__ inline float sinf(float x) { return ::sinf(x); }
}  // namespace std
