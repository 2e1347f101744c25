// Shared helpers of libzandgpu: status handling, complex arithmetic on
// double2/float2 (interleaved re, im like numpy complex128/complex64).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string>
#include "../../include/zandgpu.h"

namespace zg {

void set_error(const char* fmt, ...);

#define ZG_CHECK_CUDA(call)                                                        \
  do {                                                                             \
    cudaError_t _e = (call);                                                       \
    if (_e != cudaSuccess) {                                                       \
      zg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(_e)); \
      return _e == cudaErrorMemoryAllocation ? ZG_ENOMEM : ZG_ECUDA;               \
    }                                                                              \
  } while (0)

#define ZG_CHECK_LAUNCH() ZG_CHECK_CUDA(cudaGetLastError())

#define ZG_REQUIRE(cond, ...)        \
  do {                               \
    if (!(cond)) {                   \
      zg::set_error(__VA_ARGS__);    \
      return ZG_EINVAL;              \
    }                                \
  } while (0)

#define ZG_TRY(call)           \
  do {                         \
    int _s = (call);           \
    if (_s != ZG_OK) return _s; \
  } while (0)

// ---------------------------------------------------------------- complex
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// a / b
__host__ __device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
// acc += a*b
__host__ __device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 cdiv(float2 a, float2 b) {
  const float d = b.x * b.x + b.y * b.y;
  return make_float2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__host__ __device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}

// complex type of a real type
template <typename T> struct cx;
template <> struct cx<double> {
  using t = double2;
  __host__ __device__ static double2 make(double a, double b) { return make_double2(a, b); }
};
template <> struct cx<float> {
  using t = float2;
  __host__ __device__ static float2 make(float a, float b) { return make_float2(a, b); }
};

// ------------------------------------------------------- launch helpers
inline int grid_for(int64_t n, int threads, int max_blocks) {
  int64_t b = (n + threads - 1) / threads;
  if (b > max_blocks) b = max_blocks;
  if (b < 1) b = 1;
  return (int)b;
}

// Coefficient list of a stage combination: out = sum_t c[t] * Y[idx[t]]
struct CombineCoefs {
  int n;
  int idx[ZG_MAX_STAGES + 1];
  double c[ZG_MAX_STAGES + 1];
};

}  // namespace zg
