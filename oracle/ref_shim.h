// ORACLE - test infrastructure only. Host-side stand-ins for the CUDA
// built-ins that the reference kernels use, so that their source compiles
// with g++ and runs on the CPU (oracle/_ref, built by ref_build.py from the
// reference tree; used here only to generate and check golden vectors).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <cuda_runtime_api.h>
#include <vector_types.h>
#include <cuda_fp16.h>

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

// Block-shared arrays: one copy per OS thread, shared by the fibers that
// emulate the threads of one block.
#undef __shared__
#define __shared__ static thread_local

inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
inline float __sinf(float x) { return std::sin(x); }
inline float __logf(float x) { return std::log(x); }
inline float __expf(float x) { return std::exp(x); }
inline int __float_as_int(float x) { int i; std::memcpy(&i, &x, 4); return i; }
inline float atomicAdd(float* p, float v) { const float o = *p; *p = o + v; return o; }
inline int atomicAdd(int* p, int v) { const int o = *p; *p = o + v; return o; }
inline int atomicMax(int* p, int v) { const int o = *p; if (v > o) *p = v; return o; }
using std::min;
using std::max;
using std::isfinite;

// Barrier of the block being emulated (fiber switch, see ref_fibers.h).
void __syncthreads();

namespace foilcfd {
using FPop = float;
inline float load_f(const FPop* f, long long idx) { return f[idx]; }
inline void store_f(FPop* f, long long idx, float v) { f[idx] = v; }
} // namespace foilcfd
