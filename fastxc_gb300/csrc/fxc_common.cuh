// Shared helpers for the fastxc_gb300 C-ABI library: status codes, the
// per-thread last-error string, CUDA error propagation and small math helpers.
//
// The library never calls exit(): every failure is reported as a negative
// status plus a message readable through fxc_last_error(), which replaces the
// reference's CUDACHECK/CUFFTCHECK -> log + exit(EXIT_FAILURE) pattern
// (native/sac2spec/include/cuda.util.cuh:57-93).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>

#include "../../include/fastxc_gb300.h"

namespace fxc {

void set_error(const char* fmt, ...);
void clear_error();

}  // namespace fxc

#define FXC_CUDA_TRY(expr)                                                     \
  do {                                                                         \
    cudaError_t _e = (expr);                                                   \
    if (_e != cudaSuccess) {                                                   \
      fxc::set_error("%s failed at %s:%d: %s (%s)", #expr, __FILE__, __LINE__, \
                     cudaGetErrorName(_e), cudaGetErrorString(_e));            \
      return FXC_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

#define FXC_CHECK_ARG(cond, ...)   \
  do {                             \
    if (!(cond)) {                 \
      fxc::set_error(__VA_ARGS__); \
      return FXC_ERR_INVALID;      \
    }                              \
  } while (0)

#define FXC_TRY(expr)            \
  do {                           \
    int _s = (expr);             \
    if (_s != FXC_OK) return _s; \
  } while (0)

// Launch check: a launch configuration error surfaces here, never later.
#define FXC_LAUNCH_CHECK() FXC_CUDA_TRY(cudaGetLastError())

namespace fxc {

__host__ __device__ inline float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline float2 cadd(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__host__ __device__ inline float2 csub(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}
__host__ __device__ inline float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i
__host__ __device__ inline float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }
// multiply by +i
__host__ __device__ inline float2 mul_pi(float2 a) { return make_float2(-a.y, a.x); }

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

int num_sms();

}  // namespace fxc
