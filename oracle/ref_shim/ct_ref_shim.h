/*
 * Force-included header for compiling the reference tracer's host code with g++.
 *
 * TEST INFRASTRUCTURE ONLY (oracle). Nothing in the product library includes this.
 *
 * The reference was written for MSVC, where `fabs(float)` and friends resolve to
 * the float overloads in the global namespace and `std::cosf/std::sinf` exist.
 * These using-declarations reproduce that overload resolution under libstdc++ so
 * that, e.g., `max(1.0e-8f, fabs(x))` in Core/Microfacet.cuh:434 stays a float
 * expression exactly as MSVC compiles it.
 */
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdint>
using std::abs;
using std::fabs;
using std::sqrt;
namespace std {
inline float cosf(float x) { return ::cosf(x); }
inline float sinf(float x) { return ::sinf(x); }
}  // namespace std

/* Core/Tools.h has __device__-only helpers that use CUDA's bit-cast builtins;
 * under a host compiler they need host definitions to parse (never called). */
#include <cstring>
inline float __uint_as_float(unsigned int u) { float f; std::memcpy(&f, &u, 4); return f; }
inline unsigned int __float_as_uint(float f) { unsigned int u; std::memcpy(&u, &f, 4); return u; }
