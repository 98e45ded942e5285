// Process-wide library context (one device, one default stream).
#pragma once

#include "common.cuh"

namespace fsim {

constexpr int RED_SLOTS = 4096;  // doubles of reduction output space in the context

struct Ctx {
  bool ready = false;
  int device = -1;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  double* red = nullptr;       // device reduction outputs
  double* red_host = nullptr;  // pinned mirror
  int* status = nullptr;       // device status word: bits set by kernels whose bounded waits expired
};

Ctx& ctx();
int ensure_init();

}  // namespace fsim

// Device vector handle (replaces the reference's accel vector struct,
// accel/cuda_common.h:77-113): device data only, no JVM references.
struct fsim_vec {
  float* d = nullptr;  // n floats (real) or 2n floats (complex)
  int w = 0, h = 0;
  int cplx = 0;
  size_t n = 0;  // elements
  size_t floats() const { return cplx ? 2 * n : n; }
};
