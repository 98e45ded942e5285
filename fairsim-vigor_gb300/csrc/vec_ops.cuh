// Internal entry points shared between the vector API and the SIM-level host code.
#pragma once

#include "common.cuh"
#include "runtime.cuh"

namespace fsim {
int vec_add(fsim_vec* y, const fsim_vec* x);
// 2D C2C FFT of a w x h complex array in place on `stream` (inverse scaled by 1/(w*h)).
int fft2d_device(float2* data, int w, int h, bool inverse, cudaStream_t stream, int batch = 1);
bool fft2d_supported(int w, int h);
// mode 0: sum of squares, 1: sum, 2: sum conj(x)*y (float products), 3: sum x*conj(y) (double products)
int reduce_device(int mode, const float* x, const float* y, size_t nf, int cplx, cudaStream_t st, double* a, double* b);
int norm2_device(const float2* v, size_t n, double* out, cudaStream_t st);
// norm2 left on the device (scratch: RED_SLOTS doubles; *result points into it)
int norm2_device_async(const float2* v, size_t n, double* scratch, const double** result, cudaStream_t st);
int times_real_device(float2* y, const float* x, size_t n, cudaStream_t st);
int times_cplx_device(float2* y, const float2* x, size_t n, bool conj, cudaStream_t st);  // y = (conj)x .* y
int raw_to_cplx_device(float2* y, const void* raw, int input_u16, const float* damp, size_t n, size_t frames,
                       cudaStream_t st);
}  // namespace fsim
