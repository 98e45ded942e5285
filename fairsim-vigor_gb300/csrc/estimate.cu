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

// OTF weights from float-float table positions (otf_at_fast: the reference's double-precision
// lookup within 1e-8 of a boundary). The ratio cut |r|/|k| < dist or > 1 - dist is monotonic
// in the integer r^2, so it is decided by the thresholds r2_lo / r2_hi that the host finds with
// the reference's double expression (mx == 0 keeps the expression itself). Weight limits
// compare floats with wlf, the smallest float >= wl ((double)f < wl exactly when f < wlf).
struct CrParams {  // commonRegion's shift and its ratio-cut thresholds
  double kx, ky;
  FShift kf;
  long long r2_lo, r2_hi;
  int mx_zero;
};
// The thresholds of the ratio cut for |k| = mx: ratio = sqrt((double)r^2) / mx is
// non-decreasing in the integer r^2, so "ratio < dist" holds below r2_lo and
// "ratio > 1 - dist" above r2_hi (bisection; sqrt and division are correctly rounded on the
// host and the device alike, so both find the same integers).
// The search starts at the estimate (dist * mx)^2 and steps until the predicate flips, a few
// evaluations (the device runs it on one thread, where a bisection's chain of FP64 square
// roots and divisions took tens of microseconds).
__host__ __device__ inline void cr_thresholds(double mx, double dist, long long r2max, long long* r2_lo,
                                              long long* r2_hi) {
  auto below = [&](long long m) { return sqrt((double)m) / mx < dist; };       // the inner cut
  auto above = [&](long long m) { return sqrt((double)m) / mx > (1 - dist); };  // the outer cut
  auto clampr = [&](double v) { return v < 0 ? 0LL : (v > (double)r2max ? r2max : (long long)v); };
  long long e = clampr(dist * mx * (dist * mx));  // first r2 with !below
  while (e <= r2max && below(e)) e++;
  while (e > 0 && !below(e - 1)) e--;
  *r2_lo = e;
  e = clampr((1 - dist) * mx * ((1 - dist) * mx));  // last r2 with !above
  while (e >= 0 && above(e)) e--;
  while (e < r2max && !above(e + 1)) e++;
  *r2_hi = e;
}

__device__ __forceinline__ void common_region_px(float2* __restrict__ b0, float2* __restrict__ b1, int w, int h,
                                                 const OtfTable* __restrict__ t, const CrParams& cp, double dist,
                                                 float wlf, int divide, int bn0, int bn1, int x, int y) {
  const double kx = cp.kx, ky = cp.ky;
  const FShift kf = cp.kf;
  const long long r2_lo = cp.r2_lo, r2_hi = cp.r2_hi;
  const int mx_zero = cp.mx_zero;
  const int xh = freq_x(x, w), yh = freq_y(y, h);
  const size_t i = (size_t)y * w + x;
  float2 v0 = b0[i], v1 = b1[i];
  const FShift k0{0.f, 0.f, 0.f, 0.f};
  const float2 z = make_float2(0.f, 0.f);
  if (t->measured) {
    // weights of bands bn0 / bn1 at 0 and at +-k (writeOtfVector), complex
    float2 w0, w1, t0, t1;
    if (!otf_at_fast(*t, bn0, xh, yh, k0, 0, 0, false, &w0)) w0 = z;
    if (!otf_at_fast(*t, bn1, xh, yh, k0, 0, 0, false, &w1)) w1 = z;
    if (!otf_at_fast(*t, bn0, xh, yh, kf, kx, ky, false, &t0)) t0 = z;
    if (!otf_at_fast(*t, bn1, xh, yh, fshift_neg(kf), -kx, -ky, false, &t1)) t1 = z;
    if (cabs_java(w0) < wlf || cabs_java(t0) < wlf)
      v0 = z;
    else if (divide)
      v0 = cdiv_java(v0, w0);
    if (cabs_java(w1) < wlf || cabs_java(t1) < wlf)
      v1 = z;
    else if (divide)
      v1 = cdiv_java(v1, w1);
  } else {
    float2 c;
    const float w0 = otf_at_fast(*t, 0, xh, yh, k0, 0, 0, false, &c) ? c.x : 0.f;
    const float w1 = w0;  // single-band OTF: weight1 == weight0
    const float t0 = otf_at_fast(*t, 0, xh, yh, kf, kx, ky, false, &c) ? c.x : 0.f;
    const float t1 = otf_at_fast(*t, 0, xh, yh, fshift_neg(kf), -kx, -ky, false, &c) ? c.x : 0.f;
    // |OTF| of (val, 0) computed as (float)sqrt((double)val*val) == |val|
    if (fabsf(w0) < wlf || fabsf(t0) < wlf) {
      v0 = z;
    } else if (divide) {
      float r = __fdiv_rn(w0, __fmul_rn(w0, w0));  // Cplx.Float.reciproc, real part
      v0 = make_float2(__fmul_rn(v0.x, r), __fmul_rn(v0.y, r));
    }
    if (fabsf(w1) < wlf || fabsf(t1) < wlf) {
      v1 = z;
    } else if (divide) {
      float r = __fdiv_rn(w1, __fmul_rn(w1, w1));
      v1 = make_float2(__fmul_rn(v1.x, r), __fmul_rn(v1.y, r));
    }
  }
  auto cut = [&](int xx, int yy) {
    long long a = (xx < w / 2) ? (long long)xx * xx : (long long)(xx - w) * (xx - w);
    long long b = (yy < h / 2) ? (long long)yy * yy : (long long)(yy - h) * (yy - h);
    if (mx_zero) {  // ratio = sqrt(r^2) / 0: the reference's expression (NaN at the origin)
      const double ratio = sqrt((double)(a + b)) / 0.0;
      return (ratio < dist) || (ratio > (1 - dist));
    }
    return (a + b < r2_lo) || (a + b > r2_hi);
  };
  if (cut(x, y)) v0 = z;
  // band1 is zeroed at ((x-(int)kx+w)%w, (y+(int)ky+h)%h) for every cut (x,y)
  const int ikx = (int)kx, iky = (int)ky;
  const int xs = ((x + ikx) % w + w) % w, ys = ((y - iky) % h + h) % h;
  if (cut(xs, ys)) v1 = z;
  b0[i] = v0;
  b1[i] = v1;
}
__global__ void k_common_region(float2* __restrict__ b0, float2* __restrict__ b1, int w, int h,
                                const OtfTable* __restrict__ t, CrParams cp, double dist, float wlf, int divide,
                                int bn0, int bn1) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  common_region_px(b0, b1, w, h, t, cp, dist, wlf, divide, bn0, bn1, x, y);
}

// ---- locatePeak: argmax |v| outside kMin, first in y-major scan order --------------------
// The radius test sqrt((double)r^2) > kmin holds exactly for r^2 > r2_lim (the host finds the
// threshold with the same double expression). The magnitude Cplx.Float.abs() is evaluated in
// double only where a float estimate (within 4e-7 of it) can reach the running maximum, so
// the argmax, ties to the first index included, is the reference's.
__global__ void k_peak_partial(const float2* __restrict__ v, int w, int h, long long r2_lim, float* pmag, int* pidx) {
  float best = -1.f;
  int bi = 0x7fffffff;
  const int n = w * h;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int x = i % w, y = i / w;
    long long a = (x < w / 2) ? (long long)x * x : (long long)(x - w) * (x - w);
    long long b = (y < h / 2) ? (long long)y * y : (long long)(y - h) * (y - h);
    if (a + b > r2_lim) {
      const float2 z = v[i];
      const float est = sqrtf(z.x * z.x + z.y * z.y);
      if (est >= best * (1.f - 1e-6f)) {
        const float m = (float)sqrt((double)z.x * z.x + (double)z.y * z.y);  // Cplx.Float.abs()
        if (m > best || (m == best && i < bi)) {
          best = m;
          bi = i;
        }
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
static float weight_limit_float(double wl) {  // the smallest float >= wl
  float wlf = (float)wl;
  if ((double)wlf < wl) wlf = std::nextafter(wlf, INFINITY);
  return wlf;
}

int common_region_device(float2* b0, float2* b1, int w, int h, const OtfTable* t, double kx, double ky, double dist,
                         double wl, bool divide, cudaStream_t st, int bn0, int bn1) {
  CrParams cp{};
  cp.kx = kx;
  cp.ky = ky;
  cp.kf = fshift_host(kx, ky);
  const double mx = std::sqrt(kx * kx + ky * ky);  // unfused, as Java (host code)
  cp.mx_zero = mx > 0 ? 0 : 1;
  if (mx > 0) cr_thresholds(mx, dist, (long long)(w / 2) * (w / 2) + (long long)(h / 2) * (h / 2), &cp.r2_lo, &cp.r2_hi);
  dim3 g(div_up(w, 128), h);
  k_common_region<<<g, 128, 0, st>>>(b0, b1, w, h, t, cp, dist, weight_limit_float(wl), divide ? 1 : 0, bn0, bn1);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int locate_peak_device(const float2* v, int w, int h, double kmin, EstScratch& s, cudaStream_t st, double out4[4]) {
  const int blocks = EST_PEAK_BLOCKS;
  // the last r^2 with sqrt((double)r^2) <= kmin (sqrt is monotonic): the radius test
  // rad > kmin is r^2 > r2_lim
  const long long r2max = (long long)(w / 2) * (w / 2) + (long long)(h / 2) * (h / 2);
  long long lo = -1, hi = r2max;
  while (lo < hi) {
    const long long m = hi - (hi - lo) / 2;
    if (std::sqrt((double)m) > kmin) hi = m - 1;
    else lo = m;
  }
  k_peak_partial<<<blocks, 256, 0, st>>>(v, w, h, lo, s.pmag, s.pidx);
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

// ---- fitPeak on the device ------------------------------------------------------------------
// The three iterations of Correlation.fitPeak run without host round trips: single-thread
// kernels form each iteration's grid shifts and commonRegion parameters from the state the
// previous iteration's scan left, and the scan (yi outer, xi inner, strict >, Math.hypot and
// atan2 in double) writes the next centre; the host reads the state once at the end.
struct FitState {
  double kx, ky, search, res_phase, res_mag;
  double kxs[CORR_MAX_K], kys[CORR_MAX_K];
  double kv[2 * CORR_MAX_K];  // ramp shifts: x at [0, 10), the negated y shifts at [10, 20)
  CrParams cp;
  double grid[3 * 100 * 2];
};
__global__ void k_fit_init(FitState* f, double kx, double ky, double search) {
  f->kx = kx;
  f->ky = ky;
  f->search = search;
  f->res_phase = 0;
  f->res_mag = 0;
}
// k + ((i - 4.5) / 4.5) * search (rounded as the host does), and the commonRegion parameters
__global__ void k_fit_setup(FitState* f, double dist, int w, int h) {
  const double kx = f->kx, ky = f->ky, search = f->search;
  for (int i = 0; i < CORR_MAX_K; i++) {
    const double d = __dmul_rn(__ddiv_rn((double)i - 4.5, 4.5), search);
    f->kxs[i] = __dadd_rn(kx, d);
    f->kys[i] = __dadd_rn(ky, d);
    f->kv[i] = f->kxs[i];
    f->kv[CORR_MAX_K + i] = -f->kys[i];
  }
  CrParams cp{};
  cp.kx = kx;
  cp.ky = ky;
  cp.kf = fshift_host(kx, ky);
  const double mx = __dsqrt_rn(__dadd_rn(__dmul_rn(kx, kx), __dmul_rn(ky, ky)));
  cp.mx_zero = mx > 0 ? 0 : 1;
  if (mx > 0) cr_thresholds(mx, dist, (long long)(w / 2) * (w / 2) + (long long)(h / 2) * (h / 2), &cp.r2_lo, &cp.r2_hi);
  f->cp = cp;
}
__global__ void k_common_region_fit(float2* __restrict__ b0, float2* __restrict__ b1, int w, int h,
                                    const OtfTable* __restrict__ t, const FitState* __restrict__ f, double dist,
                                    float wlf, int bn0, int bn1) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  common_region_px(b0, b1, w, h, t, f->cp, dist, wlf, 1, bn0, bn1, x, y);
}
// 100 threads form the magnitudes, one thread compares them in the reference's order
__global__ void __launch_bounds__(128) k_fit_scan(FitState* f, const double2* __restrict__ corr, int iter,
                                                  int keep_grid) {
  __shared__ double hv[100];
  const int i = threadIdx.x;
  if (i < 100) {
    const double2 c = corr[i];
    hv[i] = hypot(c.x, c.y);
    if (keep_grid) {
      f->grid[(iter * 100 + i) * 2] = c.x;
      f->grid[(iter * 100 + i) * 2 + 1] = c.y;
    }
  }
  __syncthreads();
  if (i != 0) return;
  double mx = 0, nkx = 0, nky = 0;
  int best = -1;
  for (int k = 0; k < 100; k++)  // yi outer, xi inner
    if (hv[k] > mx) {
      mx = hv[k];
      best = k;
    }
  if (best >= 0) {
    nkx = f->kxs[best % 10];
    nky = f->kys[best / 10];
    f->res_phase = atan2(corr[best].y, corr[best].x);
    f->res_mag = mx;
  }
  f->kx = nkx;
  f->ky = nky;
  f->search = f->search / 5;
}

int EstScratch::alloc(int N, cudaStream_t st) {
  if (n == N && b0) return FSIM_OK;
  free(st);
  const size_t img = (size_t)N * N * sizeof(float2);
  // all or nothing: a partial set would pass the reuse test above next time
  // b0 and b1 back to back: fitPeak transforms both in one batched call
  cudaError_t e = fsim::dev_alloc_async(&b0, 2 * img, st);
  if (e == cudaSuccess) b1 = b0 + (size_t)N * N;
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&tx, sizeof(float2) * 10 * N, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&ty, sizeof(float2) * 10 * N, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&Q, sizeof(double2) * 10 * N, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&corr, sizeof(double2) * 100, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&kbuf, sizeof(double) * 20, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&pmag, sizeof(float) * EST_PEAK_BLOCKS, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&pidx, sizeof(int) * EST_PEAK_BLOCKS, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&red, sizeof(double) * RED_SLOTS, st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&fit, sizeof(FitState), st);
  if (e == cudaSuccess) e = fsim::dev_alloc_async(&results, sizeof(double) * 8 * FSIM_MAX_DIRS, st);
  if (e != cudaSuccess) {
    free(st);
    set_error("estimation scratch for %d x %d: %s", N, N, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? FSIM_EOOM : FSIM_ECUDA;
  }
  n = N;
  return FSIM_OK;
}
void EstScratch::free(cudaStream_t st) {
  void* ps[] = {b0, tx, ty, Q, corr, kbuf, pmag, pidx, red, fit, results};  // b1 lies inside b0's allocation
  for (void* p : ps)
    if (p) cudaFreeAsync(p, st);
  b0 = b1 = nullptr;
  tx = ty = nullptr;
  Q = corr = nullptr;
  kbuf = nullptr;
  pmag = nullptr;
  pidx = nullptr;
  red = nullptr;
  fit = nullptr;
  results = nullptr;
  n = 0;
}

// Evaluates corr(xi, yi) for kx grid kxs[nx] and ky grid kys[ny] (before the fourierShift
// sign flip of ky) on real-space b0/b1 already prepared; out[yi*nx + xi].
int corr_grid_device(const float2* b0, const float2* b1, int N, const double* kxs, int nx, const double* kys, int ny,
                     double scal, EstScratch& s, cudaStream_t st, std::vector<std::complex<double>>& out,
                     const double* n2) {
  FSIM_REQUIRE(nx >= 1 && nx <= CORR_MAX_K && ny >= 1 && ny <= CORR_MAX_K, FSIM_EINVAL,
               "correlation grid: %d x %d beyond %d x %d", nx, ny, CORR_MAX_K, CORR_MAX_K);
  double k[2 * CORR_MAX_K] = {0};
  for (int i = 0; i < nx; i++) k[i] = kxs[i];
  for (int i = 0; i < ny; i++) k[CORR_MAX_K + i] = -kys[i];
  FSIM_CUDA(cudaMemcpyAsync(s.kbuf, k, sizeof(k), cudaMemcpyHostToDevice, st));
  launch_corr_grid(b0, b1, N, s.kbuf, nx, ny, scal, n2, s.tx, s.ty, s.Q, s.corr, st);
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
  const size_t img = (size_t)N * N * sizeof(float2);
  FitState* f = s.fit;
  const float wlf = weight_limit_float(wl);
  k_fit_init<<<1, 1, 0, st>>>(f, kx, ky, search);
  for (int iter = 0; iter < 3; iter++) {
    k_fit_setup<<<1, 1, 0, st>>>(f, 0.15, N, N);
    FSIM_CUDA(cudaMemcpyAsync(s.b0, band0, img, cudaMemcpyDeviceToDevice, st));
    FSIM_CUDA(cudaMemcpyAsync(s.b1, band1, img, cudaMemcpyDeviceToDevice, st));
    k_common_region_fit<<<dim3(div_up(N, 128), N), 128, 0, st>>>(s.b0, s.b1, N, N, t, f, 0.15, wlf, bn0, bn1);
    FSIM_CHECK_LAUNCH();
    int rc = fft2d_device(s.b0, N, N, true, st, 2);  // b0 and b1 (adjacent)
    if (rc) return rc;
    // the normaliser 1 / b0.norm2() stays on the device
    const double* n2 = nullptr;
    rc = norm2_device_async(s.b0, (size_t)N * N, s.red, &n2, st);
    if (rc) return rc;
    launch_corr_grid(s.b0, s.b1, N, f->kv, 10, 10, 0., n2, s.tx, s.ty, s.Q, s.corr, st);
    k_fit_scan<<<1, 128, 0, st>>>(f, s.corr, iter, grid_out ? 1 : 0);
    FSIM_CHECK_LAUNCH();
  }
  FitState h;
  FSIM_CUDA(cudaMemcpyAsync(&h, f, sizeof(FitState), cudaMemcpyDeviceToHost, st));
  FSIM_CUDA(cudaStreamSynchronize(st));
  if (grid_out)
    for (int i = 0; i < 3 * 100 * 2; i++) grid_out[i] = h.grid[i];
  out4[0] = h.kx;
  out4[1] = h.ky;
  out4[2] = h.res_phase;
  out4[3] = h.res_mag;
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
  if ((rc = fft2d_device(s.b0, N, N, true, st, 2))) return rc;  // b0 and b1 (adjacent)
  const double* n2 = nullptr;
  if ((rc = norm2_device_async(s.b0, (size_t)N * N, s.red, &n2, st))) return rc;
  std::vector<std::complex<double>> c;
  rc = corr_grid_device(s.b0, s.b1, N, &kx, 1, &ky, 1, 0., s, st, c, n2);
  if (rc) return rc;
  *out = c[0];
  return FSIM_OK;
}

// ---- the parameter fit's steps chained on the device ------------------------------------------
// locatePeak's final reduction: the partial maxima in a fixed tree order (the comparison, the
// larger magnitude and then the smaller index, is a total order, so any order gives the
// reference's first maximum), the position converted as Correlation.locatePeak does
// (Correlation.java:159-164) and stored as fitPeak's start (-x, -y), search width 2.5.
__global__ void __launch_bounds__(EST_PEAK_BLOCKS) k_peak_final(const float* __restrict__ pmag,
                                                                const int* __restrict__ pidx, int w, int h,
                                                                FitState* f) {
  __shared__ float sm[EST_PEAK_BLOCKS];
  __shared__ int si[EST_PEAK_BLOCKS];
  const int i = threadIdx.x;
  sm[i] = pmag[i];
  si[i] = pidx[i];
  __syncthreads();
  for (int o = EST_PEAK_BLOCKS / 2; o > 0; o >>= 1) {
    if (i < o && (sm[i + o] > sm[i] || (sm[i + o] == sm[i] && si[i + o] < si[i]))) {
      sm[i] = sm[i + o];
      si[i] = si[i + o];
    }
    __syncthreads();
  }
  if (i != 0) return;
  double xPos = -0., yPos = -1;
  if (si[0] != 0x7fffffff && sm[0] >= 0) {
    xPos = si[0] % w;
    yPos = si[0] / w;
  }
  if (xPos > w / 2) xPos = xPos - w;
  if (yPos > h / 2) yPos = h - yPos;
  else yPos *= -1;
  f->kx = -xPos;
  f->ky = -yPos;
  f->search = 2.5;
  f->res_phase = 0;
  f->res_mag = 0;
}
__global__ void k_fit_store(const FitState* __restrict__ f, double* res) {
  res[0] = f->kx;
  res[1] = f->ky;
  res[2] = f->res_phase;
  res[3] = f->res_mag;
}
// getPeak at the fitted shift times a power of two (exact, as the host's divisions)
__global__ void k_gp_init(FitState* f, const double* __restrict__ res, double scale) {
  f->kx = res[0] * scale;
  f->ky = res[1] * scale;
  f->search = 0;  // the grid's first point is the shift itself
}
__global__ void k_gp_store(const double2* __restrict__ corr, double* out2) {
  out2[0] = corr[0].x;
  out2[1] = corr[0].y;
}

int locate_peak_to_fit(const float2* v, int w, int h, double kmin, EstScratch& s, cudaStream_t st) {
  const long long r2max = (long long)(w / 2) * (w / 2) + (long long)(h / 2) * (h / 2);
  long long lo = -1, hi = r2max;  // the last r^2 with sqrt((double)r^2) <= kmin
  while (lo < hi) {
    const long long m = hi - (hi - lo) / 2;
    if (std::sqrt((double)m) > kmin) hi = m - 1;
    else lo = m;
  }
  k_peak_partial<<<EST_PEAK_BLOCKS, 256, 0, st>>>(v, w, h, lo, s.pmag, s.pidx);
  k_peak_final<<<1, EST_PEAK_BLOCKS, 0, st>>>(s.pmag, s.pidx, w, h, s.fit);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int fit_peak_iterate(const float2* band0, const float2* band1, int N, const OtfTable* t, double wl, EstScratch& s,
                     cudaStream_t st, double* res, int bn0, int bn1) {
  const size_t img = (size_t)N * N * sizeof(float2);
  FitState* f = s.fit;
  const float wlf = weight_limit_float(wl);
  for (int iter = 0; iter < 3; iter++) {
    k_fit_setup<<<1, 1, 0, st>>>(f, 0.15, N, N);
    FSIM_CUDA(cudaMemcpyAsync(s.b0, band0, img, cudaMemcpyDeviceToDevice, st));
    FSIM_CUDA(cudaMemcpyAsync(s.b1, band1, img, cudaMemcpyDeviceToDevice, st));
    k_common_region_fit<<<dim3(div_up(N, 128), N), 128, 0, st>>>(s.b0, s.b1, N, N, t, f, 0.15, wlf, bn0, bn1);
    FSIM_CHECK_LAUNCH();
    int rc = fft2d_device(s.b0, N, N, true, st, 2);  // b0 and b1 (adjacent)
    if (rc) return rc;
    const double* n2 = nullptr;
    rc = norm2_device_async(s.b0, (size_t)N * N, s.red, &n2, st);
    if (rc) return rc;
    launch_corr_grid(s.b0, s.b1, N, f->kv, 10, 10, 0., n2, s.tx, s.ty, s.Q, s.corr, st);
    k_fit_scan<<<1, 128, 0, st>>>(f, s.corr, iter, 0);
    FSIM_CHECK_LAUNCH();
  }
  if (res) k_fit_store<<<1, 1, 0, st>>>(f, res);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int get_peak_at_fit(const float2* band0, const float2* band1, int N, const OtfTable* t, double wl, EstScratch& s,
                    cudaStream_t st, const double* res, double scale, double* out2, int bn0, int bn1) {
  const size_t img = (size_t)N * N * sizeof(float2);
  FitState* f = s.fit;
  k_gp_init<<<1, 1, 0, st>>>(f, res, scale);
  k_fit_setup<<<1, 1, 0, st>>>(f, 0.15, N, N);
  FSIM_CUDA(cudaMemcpyAsync(s.b0, band0, img, cudaMemcpyDeviceToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(s.b1, band1, img, cudaMemcpyDeviceToDevice, st));
  k_common_region_fit<<<dim3(div_up(N, 128), N), 128, 0, st>>>(s.b0, s.b1, N, N, t, f, 0.15,
                                                                weight_limit_float(wl), bn0, bn1);
  FSIM_CHECK_LAUNCH();
  int rc = fft2d_device(s.b0, N, N, true, st, 2);
  if (rc) return rc;
  const double* n2 = nullptr;
  if ((rc = norm2_device_async(s.b0, (size_t)N * N, s.red, &n2, st))) return rc;
  launch_corr_grid(s.b0, s.b1, N, f->kv, 1, 1, 0., n2, s.tx, s.ty, s.Q, s.corr, st);
  k_gp_store<<<1, 1, 0, st>>>(s.corr, out2);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

}  // namespace fsim
