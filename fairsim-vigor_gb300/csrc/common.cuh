// Shared device/host helpers for the fairsim-vigor_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "../../include/fairsim_gb300.h"

namespace fsim {

// ---- status handling -------------------------------------------------------
void set_error(const char* fmt, ...);
const char* last_error();
// every device allocation of the library goes through here (fsim_debug_fail_alloc hook)
cudaError_t dev_alloc(void** p, size_t bytes);
template <class T>
cudaError_t dev_alloc(T** p, size_t bytes) {
  return dev_alloc(reinterpret_cast<void**>(p), bytes);
}
cudaError_t dev_alloc_async(void** p, size_t bytes, cudaStream_t st);
template <class T>
cudaError_t dev_alloc_async(T** p, size_t bytes, cudaStream_t st) {
  return dev_alloc_async(reinterpret_cast<void**>(p), bytes, st);
}

#define FSIM_CUDA(call)                                                                \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      ::fsim::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      return (e_ == cudaErrorMemoryAllocation) ? FSIM_EOOM : FSIM_ECUDA;               \
    }                                                                                  \
  } while (0)

#define FSIM_CHECK_LAUNCH()                                                            \
  do {                                                                                 \
    cudaError_t e_ = cudaGetLastError();                                               \
    if (e_ != cudaSuccess) {                                                           \
      ::fsim::set_error("%s:%d launch: %s", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return FSIM_ECUDA;                                                               \
    }                                                                                  \
  } while (0)

#define FSIM_REQUIRE(cond, code, ...)   \
  do {                                  \
    if (!(cond)) {                      \
      ::fsim::set_error(__VA_ARGS__);   \
      return (code);                    \
    }                                   \
  } while (0)

// ---- complex helpers (interleaved re,im as float2) ------------------------------
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 cconjf(float2 a) { return make_float2(a.x, -a.y); }

// Frequency coordinate conventions of the reference (S/OtfProvider.java:345-346):
// x index -> x < w/2 ? x : x - w ; y index -> y < h/2 ? -y : h - y (y flipped)
__host__ __device__ __forceinline__ int freq_x(int x, int w) { return x < w / 2 ? x : x - w; }
__host__ __device__ __forceinline__ int freq_y(int y, int h) { return y < h / 2 ? -y : h - y; }

inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace fsim
