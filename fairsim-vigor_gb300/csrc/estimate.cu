// Parameter estimation on the device: Correlation.commonRegion / locatePeak / fitPeak /
// getPeak and SimAlgorithm.estimateParameters (S/Correlation.java:43-288,
// S/SimAlgorithm.java:37-159; the live refit of LM/ReconstructionRunner.java:642-746).
//
// The 10x10 sub-pixel grid of fitPeak is evaluated in two passes instead of 100 shifted
// vector copies (corr_grid.cuh): row sums per image row, then the column sums, in a fixed
// order (deterministic).
#include <cmath>
#include <vector>

#include "common.cuh"
#include "corr_grid.cuh"
#include "estimate.cuh"
#include "filters.cuh"
#include "otf.cuh"
#include "runtime.cuh"
#include "sim_host.h"
#include "vec_ops.cuh"

namespace fsim {

// ---- commonRegion as a gather (Correlation.java:227-288) --------------------------------
// Cplx.Float.abs: (float)sqrt((double)re*re + (double)im*im)
__device__ __forceinline__ float cabs_java(float2 v) {
  return (float)__dsqrt_rn(__dadd_rn(__dmul_rn((double)v.x, (double)v.x), __dmul_rn((double)v.y, (double)v.y)));
}
// Cplx.Float.div(a, b) = mult(a, reciproc(b)), reciproc = (re/s, -im/s), s = re^2 + im^2
__device__ __forceinline__ float2 cdiv_java(float2 a, float2 b) {
  const float s = __fadd_rn(__fmul_rn(b.x, b.x), __fmul_rn(b.y, b.y));
  const float rr = __fdiv_rn(b.x, s), ri = __fdiv_rn(-b.y, s);
  return make_float2(__fsub_rn(__fmul_rn(a.x, rr), __fmul_rn(a.y, ri)), __fadd_rn(__fmul_rn(a.x, ri), __fmul_rn(a.y, rr)));
}

__global__ void k_common_region(float2* __restrict__ b0, float2* __restrict__ b1, int w, int h,
                                const OtfTable* __restrict__ t, double kx, double ky, double dist, double wl, int divide,
                                int bn0, int bn1) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  const double xh = freq_x(x, w), yh = freq_y(y, h);
  const size_t i = (size_t)y * w + x;
  float2 v0 = b0[i], v1 = b1[i];
  if (t->measured) {
    // weights of bands bn0 / bn1 at 0 and at +-k (writeOtfVector), complex
    const float2 z = make_float2(0.f, 0.f);
    float2 w0, w1, t0, t1;
    if (!otf_at_c(*t, bn0, xh, yh, 0, 0, false, &w0)) w0 = z;
    if (!otf_at_c(*t, bn1, xh, yh, 0, 0, false, &w1)) w1 = z;
    if (!otf_at_c(*t, bn0, xh, yh, kx, ky, false, &t0)) t0 = z;
    if (!otf_at_c(*t, bn1, xh, yh, -kx, -ky, false, &t1)) t1 = z;
    if (cabs_java(w0) < wl || cabs_java(t0) < wl)
      v0 = z;
    else if (divide)
      v0 = cdiv_java(v0, w0);
    if (cabs_java(w1) < wl || cabs_java(t1) < wl)
      v1 = z;
    else if (divide)
      v1 = cdiv_java(v1, w1);
  } else {
    float w0 = 0.f, w1 = 0.f, t0 = 0.f, t1 = 0.f;
    if (!otf_at(*t, xh, yh, 0, 0, false, &w0)) w0 = 0.f;
    w1 = w0;  // single-band OTF: weight1 == weight0
    if (!otf_at(*t, xh, yh, kx, ky, false, &t0)) t0 = 0.f;
    if (!otf_at(*t, xh, yh, -kx, -ky, false, &t1)) t1 = 0.f;
    // |OTF| of (val, 0) computed as (float)sqrt((double)val*val) == |val|
    if (fabsf(w0) < wl || fabsf(t0) < wl) {
      v0 = make_float2(0.f, 0.f);
    } else if (divide) {
      float r = __fdiv_rn(w0, __fmul_rn(w0, w0));  // Cplx.Float.reciproc, real part
      v0 = make_float2(__fmul_rn(v0.x, r), __fmul_rn(v0.y, r));
    }
    if (fabsf(w1) < wl || fabsf(t1) < wl) {
      v1 = make_float2(0.f, 0.f);
    } else if (divide) {
      float r = __fdiv_rn(w1, __fmul_rn(w1, w1));
      v1 = make_float2(__fmul_rn(v1.x, r), __fmul_rn(v1.y, r));
    }
  }
  const double mx = __dsqrt_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)));  // unfused, as Java
  auto cut = [&](int xx, int yy) {
    long long a = (xx < w / 2) ? (long long)xx * xx : (long long)(xx - w) * (xx - w);
    long long b = (yy < h / 2) ? (long long)yy * yy : (long long)(yy - h) * (yy - h);
    double ratio = sqrt((double)(a + b)) / mx;
    return (ratio < dist) || (ratio > (1 - dist));
  };
  if (cut(x, y)) v0 = make_float2(0.f, 0.f);
  // band1 is zeroed at ((x-(int)kx+w)%w, (y+(int)ky+h)%h) for every cut (x,y)
  const int ikx = (int)kx, iky = (int)ky;
  const int xs = ((x + ikx) % w + w) % w, ys = ((y - iky) % h + h) % h;
  if (cut(xs, ys)) v1 = make_float2(0.f, 0.f);
  b0[i] = v0;
  b1[i] = v1;
}

// ---- locatePeak: argmax |v| outside kMin, first in y-major scan order --------------------
__global__ void k_peak_partial(const float2* __restrict__ v, int w, int h, double kmin, float* pmag, int* pidx) {
  float best = -1.f;
  int bi = 0x7fffffff;
  const int n = w * h;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int x = i % w, y = i / w;
    long long a = (x < w / 2) ? (long long)x * x : (long long)(x - w) * (x - w);
    long long b = (y < h / 2) ? (long long)y * y : (long long)(y - h) * (y - h);
    double rad = sqrt((double)(a + b));
    if (rad > kmin) {
      float2 z = v[i];
      float m = (float)sqrt((double)z.x * z.x + (double)z.y * z.y);  // Cplx.Float.abs()
      if (m > best || (m == best && i < bi)) {
        best = m;
        bi = i;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    float m2 = __shfl_down_sync(0xffffffffu, best, o);
    int i2 = __shfl_down_sync(0xffffffffu, bi, o);
    if (m2 > best || (m2 == best && i2 < bi)) {
      best = m2;
      bi = i2;
    }
  }
  __shared__ float sm[32];
  __shared__ int si[32];
  if (threadIdx.x % 32 == 0) {
    sm[threadIdx.x / 32] = best;
    si[threadIdx.x / 32] = bi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x / 32); k++)
      if (sm[k] > best || (sm[k] == best && si[k] < bi)) {
        best = sm[k];
        bi = si[k];
      }
    pmag[blockIdx.x] = best;
    pidx[blockIdx.x] = bi;
  }
}

// ---- host side ------------------------------------------------------------------------------
int common_region_device(float2* b0, float2* b1, int w, int h, const OtfTable* t, double kx, double ky, double dist,
                         double wl, bool divide, cudaStream_t st, int bn0, int bn1) {
  dim3 g(div_up(w, 128), h);
  k_common_region<<<g, 128, 0, st>>>(b0, b1, w, h, t, kx, ky, dist, wl, divide ? 1 : 0, bn0, bn1);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int locate_peak_device(const float2* v, int w, int h, double kmin, EstScratch& s, cudaStream_t st, double out4[4]) {
  const int blocks = 128;
  k_peak_partial<<<blocks, 256, 0, st>>>(v, w, h, kmin, s.pmag, s.pidx);
  FSIM_CHECK_LAUNCH();
  std::vector<float> m(blocks);
  std::vector<int> idx(blocks);
  FSIM_CUDA(cudaMemcpyAsync(m.data(), s.pmag, sizeof(float) * blocks, cudaMemcpyDeviceToHost, st));
  FSIM_CUDA(cudaMemcpyAsync(idx.data(), s.pidx, sizeof(int) * blocks, cudaMemcpyDeviceToHost, st));
  FSIM_CUDA(cudaStreamSynchronize(st));
  float best = -1.f;
  int bi = 0x7fffffff;
  for (int b = 0; b < blocks; b++)
    if (m[b] > best || (m[b] == best && idx[b] < bi)) {
      best = m[b];
      bi = idx[b];
    }
  double xPos = -0., yPos = -1, phase = 0;
  double max = -1;
  if (bi != 0x7fffffff && best >= 0) {
    xPos = bi % w;
    yPos = bi / w;
    max = best;
    float2 z;
    FSIM_CUDA(cudaMemcpyAsync(&z, v + bi, sizeof(float2), cudaMemcpyDeviceToHost, st));
    FSIM_CUDA(cudaStreamSynchronize(st));
    phase = (double)(float)std::atan2((double)z.y, (double)z.x);  // Cplx.Float.phase()
  }
  if (xPos > w / 2) xPos = xPos - w;
  if (yPos > h / 2)
    yPos = h - yPos;
  else
    yPos *= -1;
  out4[0] = xPos;
  out4[1] = yPos;
  out4[2] = max;
  out4[3] = phase;
  return FSIM_OK;
}

int EstScratch::alloc(int N, cudaStream_t st) {
  if (n == N && b0) return FSIM_OK;
  free(st);
  const size_t img = (size_t)N * N * sizeof(float2);
  // all or nothing: a partial set would pass the reuse test above next time
  cudaError_t e = fsim::dev_alloc_async(&b0, img, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&b1, img, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&tx, sizeof(float2) * 10 * N, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&ty, sizeof(float2) * 10 * N, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&Q, sizeof(double2) * 10 * N, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&corr, sizeof(double2) * 100, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&kbuf, sizeof(double) * 20, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&pmag, sizeof(float) * 256, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&pidx, sizeof(int) * 256, st);
  if (e != cudaSuccess) {
    free(st);
    set_error("estimation scratch for %d x %d: %s", N, N, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? FSIM_EOOM : FSIM_ECUDA;
  }
  n = N;
  return FSIM_OK;
}
void EstScratch::free(cudaStream_t st) {
  void* ps[] = {b0, b1, tx, ty, Q, corr, kbuf, pmag, pidx};
  for (void* p : ps)
    if (p) cudaFreeAsync(p, st);
  b0 = b1 = nullptr;
  tx = ty = nullptr;
  Q = corr = nullptr;
  kbuf = nullptr;
  pmag = nullptr;
  pidx = nullptr;
  n = 0;
}

// Evaluates corr(xi, yi) for kx grid kxs[nx] and ky grid kys[ny] (before the fourierShift
// sign flip of ky) on real-space b0/b1 already prepared; out[yi*nx + xi].
int corr_grid_device(const float2* b0, const float2* b1, int N, const double* kxs, int nx, const double* kys, int ny,
                     double scal, EstScratch& s, cudaStream_t st, std::vector<std::complex<double>>& out) {
  FSIM_REQUIRE(nx >= 1 && nx <= CORR_MAX_K && ny >= 1 && ny <= CORR_MAX_K, FSIM_EINVAL,
               "correlation grid: %d x %d beyond %d x %d", nx, ny, CORR_MAX_K, CORR_MAX_K);
  double k[2 * CORR_MAX_K] = {0};
  for (int i = 0; i < nx; i++) k[i] = kxs[i];
  for (int i = 0; i < ny; i++) k[CORR_MAX_K + i] = -kys[i];
  FSIM_CUDA(cudaMemcpyAsync(s.kbuf, k, sizeof(k), cudaMemcpyHostToDevice, st));
  launch_corr_grid(b0, b1, N, s.kbuf, nx, ny, scal, s.tx, s.ty, s.Q, s.corr, st);
  FSIM_CHECK_LAUNCH();
  std::vector<double2> h(nx * ny);
  FSIM_CUDA(cudaMemcpyAsync(h.data(), s.corr, sizeof(double2) * nx * ny, cudaMemcpyDeviceToHost, st));
  FSIM_CUDA(cudaStreamSynchronize(st));
  out.resize(nx * ny);
  for (int i = 0; i < nx * ny; i++) out[i] = std::complex<double>(h[i].x, h[i].y);
  return FSIM_OK;
}

// norm2 of a device vector in FP64 (float squares), synchronous
int norm2_device(const float2* v, size_t n, double* out, cudaStream_t st);

// Correlation.fitPeak (Correlation.java:43-136) on device spectra band0/band1 (w x w).
int fit_peak_device(const float2* band0, const float2* band1, int N, const OtfTable* t, double kx, double ky, double wl,
                    double search, EstScratch& s, cudaStream_t st, double out4[4], double* grid_out, int bn0, int bn1) {
  double resPhase = 0, resMag = 0;
  const size_t img = (size_t)N * N * sizeof(float2);
  for (int iter = 0; iter < 3; iter++) {
    FSIM_CUDA(cudaMemcpyAsync(s.b0, band0, img, cudaMemcpyDeviceToDevice, st));
    FSIM_CUDA(cudaMemcpyAsync(s.b1, band1, img, cudaMemcpyDeviceToDevice, st));
    int rc = common_region_device(s.b0, s.b1, N, N, t, kx, ky, 0.15, wl, true, st, bn0, bn1);
    if (rc) return rc;
    rc = fft2d_device(s.b0, N, N, true, st);
    if (rc) return rc;
    rc = fft2d_device(s.b1, N, N, true, st);
    if (rc) return rc;
    double n2 = 0;
    rc = norm2_device(s.b0, (size_t)N * N, &n2, st);
    if (rc) return rc;
    const double scal = 1. / n2;
    double kxs[10], kys[10];
    for (int i = 0; i < 10; i++) {
      kxs[i] = kx + ((i - 4.5) / 4.5) * search;
      kys[i] = ky + ((i - 4.5) / 4.5) * search;
    }
    std::vector<std::complex<double>> corr;
    rc = corr_grid_device(s.b0, s.b1, N, kxs, 10, kys, 10, scal, s, st, corr);
    if (rc) return rc;
    double max = 0, newKx = 0, newKy = 0;
    for (int yi = 0; yi < 10; yi++)
      for (int xi = 0; xi < 10; xi++) {
        std::complex<double> c = corr[yi * 10 + xi];
        double hv = std::hypot(c.real(), c.imag());
        if (grid_out) {
          grid_out[(iter * 100 + yi * 10 + xi) * 2] = c.real();
          grid_out[(iter * 100 + yi * 10 + xi) * 2 + 1] = c.imag();
        }
        if (hv > max) {
          max = hv;
          newKx = kxs[xi];
          newKy = kys[yi];
          resPhase = std::atan2(c.imag(), c.real());
          resMag = hv;
        }
      }
    kx = newKx;
    ky = newKy;
    search /= 5;
  }
  out4[0] = kx;
  out4[1] = ky;
  out4[2] = resPhase;
  out4[3] = resMag;
  return FSIM_OK;
}

// Correlation.getPeak (Correlation.java:183-209)
int get_peak_device(const float2* band0, const float2* band1, int N, const OtfTable* t, double kx, double ky, double wl,
                    EstScratch& s, cudaStream_t st, std::complex<double>* out, int bn0, int bn1) {
  const size_t img = (size_t)N * N * sizeof(float2);
  FSIM_CUDA(cudaMemcpyAsync(s.b0, band0, img, cudaMemcpyDeviceToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(s.b1, band1, img, cudaMemcpyDeviceToDevice, st));
  int rc = common_region_device(s.b0, s.b1, N, N, t, kx, ky, 0.15, wl, true, st, bn0, bn1);
  if (rc) return rc;
  if ((rc = fft2d_device(s.b0, N, N, true, st))) return rc;
  if ((rc = fft2d_device(s.b1, N, N, true, st))) return rc;
  double n2 = 0;
  if ((rc = norm2_device(s.b0, (size_t)N * N, &n2, st))) return rc;
  std::vector<std::complex<double>> c;
  rc = corr_grid_device(s.b0, s.b1, N, &kx, 1, &ky, 1, 1. / n2, s, st, c);
  if (rc) return rc;
  *out = c[0];
  return FSIM_OK;
}

}  // namespace fsim
