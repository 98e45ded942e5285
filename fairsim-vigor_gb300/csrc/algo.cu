// SIM-level entry points built from the vector kernels: the op-by-op reconstruction
// (SimAlgorithm.runReconstruction, S/SimAlgorithm.java:268-582, run on device vectors the
// way the reference's Java runs it on an accel vector factory) and the parameter fit
// (S/SimAlgorithm.java:37-159, LM/ReconstructionRunner.java:642-746).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "estimate.cuh"
#include "filters.cuh"
#include "otf.cuh"
#include "runtime.cuh"
#include "sim_host.h"
#include "vec_ops.cuh"

namespace fsim {

// SimUtils.fadeBorderCos applied to a vector of ones (S/SimUtils.java:162-185;
// LM/ReconstructionRunner.java:781-783): float storage, double factors.
std::vector<float> fade_vector(int w, int h, int px) {
  std::vector<float> d((size_t)w * h, 1.0f);
  if (px <= 0) return d;
  const double fac = 1. / px * M_PI / 2.;
  auto at = [&](int x, int y) -> float& { return d[(size_t)x + (size_t)w * y]; };
  for (int y = 0; y < px; y++)
    for (int x = 0; x < w; x++) at(x, y) = (float)(at(x, y) * std::pow(std::sin(y * fac), 2));
  for (int y = h - px; y < h; y++)
    for (int x = 0; x < w; x++) at(x, y) = (float)(at(x, y) * std::pow(std::sin((h - y - 1) * fac), 2));
  for (int y = 0; y < h; y++)
    for (int x = 0; x < px; x++) at(x, y) = (float)(at(x, y) * std::pow(std::sin(x * fac), 2));
  for (int y = 0; y < h; y++)
    for (int x = w - px; x < w; x++) at(x, y) = (float)(at(x, y) * std::pow(std::sin((w - x - 1) * fac), 2));
  return d;
}

// A device OTF table owned by one caller.
struct DevOtf {
  OtfTable* d = nullptr;
  int set(const fsim_sim_param* p, cudaStream_t st) {
    OtfTable h;
    build_otf_table(p, &h);
    if (!d) FSIM_CUDA(fsim::dev_alloc_async(&d, sizeof(OtfTable), st));
    FSIM_CUDA(cudaMemcpyAsync(d, &h, sizeof(OtfTable), cudaMemcpyHostToDevice, st));
    FSIM_CUDA(cudaStreamSynchronize(st));  // h is on this stack frame
    return FSIM_OK;
  }
  void release(cudaStream_t st) {
    if (d) cudaFreeAsync(d, st);
    d = nullptr;
  }
};

// RAII bundle of stream-ordered device allocations
struct DevBufs {
  cudaStream_t st;
  std::vector<void*> ptrs;
  explicit DevBufs(cudaStream_t s) : st(s) {}
  template <class T>
  int get(T** p, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = fsim::dev_alloc_async(&q, bytes, st);
    if (e != cudaSuccess) {
      set_error("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
      return FSIM_EOOM;
    }
    ptrs.push_back(q);
    *p = (T*)q;
    return FSIM_OK;
  }
  ~DevBufs() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
};

#define TRY(x)            \
  do {                    \
    int rc_ = (x);        \
    if (rc_) return rc_;  \
  } while (0)

int estimate_core(fsim_sim_param* p, const float2* const* spec, int fit_band, double fit_exclude, bool live,
                  double* peaks_out, cudaStream_t st) {
  TRY(validate_param(p));
  if (!live && fit_band != 1 && fit_band != 2) {
    set_error("Fitband neither 1 nor 2");
    return FSIM_EINVAL;
  }
  const int N = p->w, nP = p->nr_phases, nB = p->nr_bands, nC = 2 * nB - 1;
  const size_t n = (size_t)N * N;
  DevBufs bufs(st);
  float2 *sep, *c0, *c1;
  float* att;
  TRY(bufs.get(&sep, sizeof(float2) * n * nC));
  TRY(bufs.get(&c0, sizeof(float2) * n));
  TRY(bufs.get(&c1, sizeof(float2) * n));
  TRY(bufs.get(&att, sizeof(float) * n));
  DevOtf otf;
  TRY(otf.set(p, st));
  EstScratch s;
  TRY(s.alloc(N, st));
  OtfTable ht;
  build_otf_table(p, &ht);
  const double vec_cpm = ht.vec_cpm;
  // otfAtt = writeAttenuationVector(.99, 0.15*cutoff, 0, 0) (SimAlgorithm.java:65-66)
  TRY(att_device(att, N, N, vec_cpm, .99, 0.15 * ht.cutoff, 0, 0, st));
  int rc = FSIM_OK;
  for (int a = 0; a < p->nr_dirs && rc == FSIM_OK; a++) {
    auto coef = separation_coeffs(p, a, true);  // phaOff 0, fac null
    SepArgs sa{};
    sa.n_in = nP;
    sa.n_out = nC;
    for (int i = 0; i < nP; i++) sa.in[i] = spec[a * nP + i];
    for (int b = 0; b < nC; b++) sa.out[b] = sep + b * n;
    for (int b = 0; b < nC; b++)
      for (int q = 0; q < nP; q++) sa.coef[b * nP + q] = make_float2(coef[b * nP + q].real(), coef[b * nP + q].imag());
    TRY(separate_device(sa, n, st));
    const int lb = 1, hb = (nB == 3) ? 3 : 1;
    const int target = live ? hb : ((fit_band == 1) ? lb : hb);
    // coarse correlation of band0 with the target band (SimAlgorithm.java:85-106)
    FSIM_CUDA(cudaMemcpyAsync(c0, sep, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st));
    FSIM_CUDA(cudaMemcpyAsync(c1, sep + target * n, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st));
    TRY(times_real_device(c0, att, n, st));
    TRY(times_real_device(c1, att, n, st));
    TRY(fft2d_device(c0, N, N, true, st));
    TRY(fft2d_device(c1, N, N, true, st));
    TRY(times_cplx_device(c1, c0, n, true, st));
    TRY(fft2d_device(c1, N, N, false, st));
    const double minDist = fit_exclude * ht.cutoff / vec_cpm;
    // locatePeak -> fitPeak -> getPeak on the device (no host round trips); the results of
    // direction a: fit (kx, ky, phase, magnitude) at r[0..3], p1 at r[4..5], p2 at r[6..7]
    double* r = s.results + 8 * a;
    TRY(locate_peak_to_fit(c1, N, N, minDist, s, st));
    const int fb = live ? hb : ((fit_band == 1) ? lb : hb);
    TRY(fit_peak_iterate(sep, sep + fb * n, N, otf.d, 0.05, s, st, r, 0, live ? 1 : fit_band));
    if (live) {
      const int nBand = nB - 1;  // fit / nBand (nBand 1 or 2: exact)
      TRY(get_peak_at_fit(sep, sep + lb * n, N, otf.d, 0.05, s, st, r, 1.0 / nBand, r + 4));
    } else if (lb != hb) {
      // the host doubles the fit for fit band 1: p1 at fit' / 2, p2 at fit'
      const double f2 = (fit_band == 1) ? 2.0 : 1.0;
      TRY(get_peak_at_fit(sep, sep + lb * n, N, otf.d, 0.05, s, st, r, f2 / 2, r + 4));
      TRY(get_peak_at_fit(sep, sep + hb * n, N, otf.d, 0.05, s, st, r, f2, r + 6, 0, 2));
    } else {
      TRY(get_peak_at_fit(sep, sep + 1 * n, N, otf.d, 0.05, s, st, r, 1.0, r + 4));
    }
  }
  // one read of every direction's results
  double res[8 * FSIM_MAX_DIRS];
  FSIM_CUDA(cudaMemcpyAsync(res, s.results, sizeof(double) * 8 * p->nr_dirs, cudaMemcpyDeviceToHost, st));
  FSIM_CUDA(cudaStreamSynchronize(st));
  for (int a = 0; a < p->nr_dirs; a++) {
    const double* r = res + 8 * a;
    double fit[4] = {r[0], r[1], r[2], r[3]};
    const std::complex<double> p1(r[4], r[5]), p2(r[6], r[7]);
    const int lb = 1, hb = (nB == 3) ? 3 : 1;
    if (live) {
      p->px[a] = -fit[0] / (nB - 1);
      p->py[a] = -fit[1] / (nB - 1);
      p->pha_off[a] = std::atan2(p1.imag(), p1.real());
      p->modulation[a][1] = std::hypot(p1.real(), p1.imag());
    } else if (lb != hb) {
      if (fit_band == 1) {
        fit[0] *= 2;
        fit[1] *= 2;
      }
      p->px[a] = -fit[0] / (nB - 1);
      p->py[a] = -fit[1] / (nB - 1);
      p->pha_off[a] = std::atan2(p1.imag(), p1.real());
      p->modulation[a][1] = std::hypot(p1.real(), p1.imag());
      p->modulation[a][2] = std::hypot(p2.real(), p2.imag());
    } else {
      p->px[a] = -fit[0] / (nB - 1);
      p->py[a] = -fit[1] / (nB - 1);
      p->pha_off[a] = std::atan2(p1.imag(), p1.real());
      p->modulation[a][1] = std::hypot(p1.real(), p1.imag());
    }
    if (peaks_out)
      for (int i = 0; i < 4; i++) peaks_out[4 * a + i] = fit[i];
  }
  s.free(st);
  otf.release(st);
  FSIM_CUDA(cudaStreamSynchronize(st));
  return rc;
}

// raw frames on the device -> spectra (damp, forward FFT), as the GUI / live code prepares them
static int raw_to_spectra(const fsim_sim_param* p, const void* raw, int input_u16, int fade_px, float2* spec,
                          DevBufs& bufs, cudaStream_t st) {
  const int N = p->w, frames = p->nr_dirs * p->nr_phases;
  const size_t n = (size_t)N * N;
  float* damp = nullptr;
  if (fade_px > 0) {
    std::vector<float> h = fade_vector(N, N, fade_px);
    TRY(bufs.get(&damp, sizeof(float) * n));
    FSIM_CUDA(cudaMemcpyAsync(damp, h.data(), sizeof(float) * n, cudaMemcpyHostToDevice, st));
    FSIM_CUDA(cudaStreamSynchronize(st));
  }
  TRY(raw_to_cplx_device(spec, raw, input_u16, damp, n, frames, st));
  return fft2d_device(spec, N, N, false, st, frames);
}

// ---- the op-by-op reconstruction -------------------------------------------------------------
__global__ void k_max_partial(const float* __restrict__ v, size_t n, float* part) {
  float m = 0.f;  // clipAndScale starts its max at 0 (S/SimUtils.java:247-253)
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    m = fmaxf(m, v[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  __shared__ float s[32];
  if (threadIdx.x % 32 == 0) s[threadIdx.x / 32] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x / 32); k++) m = fmaxf(m, s[k]);
    part[blockIdx.x] = m;
  }
}
__global__ void k_clip_scale(float* __restrict__ v, size_t n, const float* __restrict__ part, int nparts, int scale) {
  float f = 1.f;
  if (scale) {
    float m = 0.f;
    for (int k = 0; k < nparts; k++) m = fmaxf(m, part[k]);
    f = __fdiv_rn(255.f, m);
  }
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float x = v[i];
    if (scale) x = __fmul_rn(x, f);
    if (x < 0) x = 0;
    v[i] = x;
  }
}
__global__ void k_real_part(float* __restrict__ out, const float2* __restrict__ in, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) out[i] = in[i].x;
}
__global__ void k_paste(float2* __restrict__ out, int wo, const float2* __restrict__ in, int wi) {
  // pasteFreq(in, 0, 0) for wo == 2*wi as a gather
  int xo = blockIdx.x * blockDim.x + threadIdx.x, yo = blockIdx.y;
  if (xo >= wo) return;
  int xs = xo < wi / 2 ? xo : (xo >= wo - (wi - wi / 2) ? xo - wo / 2 : -1);
  int ys = yo < wi / 2 ? yo : (yo >= wo - (wi - wi / 2) ? yo - wo / 2 : -1);
  out[(size_t)yo * wo + xo] = (xs >= 0 && ys >= 0) ? in[(size_t)ys * wi + xs] : make_float2(0.f, 0.f);
}
__global__ void k_shift_ramp(float2* __restrict__ v, int N, double kx, double ky) {
  // v *= exp(i 2 pi (kx x + ky y)/N), phase reduced modulo one turn in double per axis
  __shared__ float2 tx[32], ty[8];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  if (tid < 40) {
    const bool isx = tid < 32;
    const int c = isx ? x0 + tid : y0 + tid - 32;
    double f = (isx ? kx : ky) * (double)c / (double)N;
    f -= floor(f);
    double s, co;
    sincospi(2.0 * f, &s, &co);
    if (isx)
      tx[tid] = make_float2((float)co, (float)s);
    else
      ty[tid - 32] = make_float2((float)co, (float)s);
  }
  __syncthreads();
  int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  if (x < N && y < N) {
    size_t i = (size_t)y * N + x;
    v[i] = cmul(v[i], cmul(tx[threadIdx.x], ty[threadIdx.y]));
  }
}

__global__ void k_mask(float2* __restrict__ v, int w, int h, double vec_cpm, double cutoff, double kx, double ky) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  double rad = __dmul_rn(d_hypot_java(__dsub_rn((double)freq_x(x, w), kx), __dsub_rn((double)freq_y(y, h), ky)), vec_cpm);
  if (rad > cutoff) v[(size_t)y * w + x] = make_float2(0.f, 0.f);
}
__global__ void k_accum(float2* __restrict__ y, const float2* __restrict__ x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float2 a = y[i], b = x[i];
    y[i] = make_float2(a.x + b.x, a.y + b.y);
  }
}

static int grid1(size_t n) { return (int)std::min<size_t>((n + 255) / 256, (size_t)ctx().num_sms * 8); }

// Vec.scal(float): v *= a (real factor)
__global__ void k_scal_band0(float2* __restrict__ v, size_t n, float a) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float2 x = v[i];
    v[i] = make_float2(__fmul_rn(x.x, a), __fmul_rn(x.y, a));
  }
}

// ---- Richardson-Lucy (RLDeconvolution.deconvolve, S/RLDeconvolution.java:45-103) -------------
// next = d .* reciproc(next): AbstractVectorCplx.reciproc (s = re^2 + im^2; re/s, -im/s,
// L/AbstractVectorCplx.java:208-216), then times(d) (y = x .* y with x = d)
__global__ void k_rl_div(float2* __restrict__ next, const float2* __restrict__ d, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float2 v = next[i], x = d[i];
    const float s = __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y));
    const float rr = __fdiv_rn(v.x, s), ri = __fdiv_rn(-v.y, s);
    next[i] = make_float2(__fsub_rn(__fmul_rn(x.x, rr), __fmul_rn(x.y, ri)),
                          __fadd_rn(__fmul_rn(x.y, rr), __fmul_rn(x.x, ri)));
  }
}
// next = deconv .* next (times(deconvImg)), then deconvImg.copy(nextImg): both hold u_{j+1}
__global__ void k_rl_update(float2* __restrict__ next, float2* __restrict__ deconv, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float2 v = next[i], x = deconv[i];
    const float2 r = make_float2(__fsub_rn(__fmul_rn(x.x, v.x), __fmul_rn(x.y, v.y)),
                                 __fadd_rn(__fmul_rn(x.y, v.x), __fmul_rn(x.x, v.y)));
    next[i] = r;
    deconv[i] = r;
  }
}

// u_{j+1} = u_j x [(d / (u_j * psf)) * psf], the convolutions as products with `otf` in
// frequency space, u_0 = d (the observed image); in_freq: img holds a spectrum
int rl_deconvolve_device(float2* img, const float2* otf, int w, int h, int steps, bool in_freq, cudaStream_t st) {
  FSIM_REQUIRE(fft2d_supported(w, h), FSIM_EINVAL, "RL deconvolution: unsupported size %d x %d", w, h);
  FSIM_REQUIRE(steps >= 0, FSIM_EINVAL, "RL deconvolution: negative step count %d", steps);
  const size_t n = (size_t)w * h;
  DevBufs bufs(st);
  float2 *deconv, *next;
  TRY(bufs.get(&deconv, sizeof(float2) * n));
  TRY(bufs.get(&next, sizeof(float2) * n));
  if (in_freq) TRY(fft2d_device(img, w, h, true, st));
  FSIM_CUDA(cudaMemcpyAsync(deconv, img, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(next, img, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st));
  for (int i = 0; i < steps; i++) {
    TRY(fft2d_device(next, w, h, false, st));  // u_j * psf
    TRY(times_cplx_device(next, otf, n, false, st));
    TRY(fft2d_device(next, w, h, true, st));
    k_rl_div<<<grid1(n), 256, 0, st>>>(next, img, n);  // d / (u_j * psf)
    FSIM_CHECK_LAUNCH();
    TRY(fft2d_device(next, w, h, false, st));  // ... * psf
    TRY(times_cplx_device(next, otf, n, false, st));
    TRY(fft2d_device(next, w, h, true, st));
    k_rl_update<<<grid1(n), 256, 0, st>>>(next, deconv, n);  // u_j x [...]
    FSIM_CHECK_LAUNCH();
  }
  FSIM_CUDA(cudaMemcpyAsync(img, deconv, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st));
  if (in_freq) TRY(fft2d_device(img, w, h, false, st));
  return FSIM_OK;
}

// Correlation.autoCorrelation (S/Correlation.java:294-325)
int auto_correlation_device(const float2* band, int n, double kx, double ky, double* re, double* im, cudaStream_t st) {
  const int N = 2 * n;
  FSIM_REQUIRE(fft2d_supported(N, N), FSIM_EINVAL, "autoCorrelation: unsupported size %d", n);
  const size_t n2 = (size_t)N * N;
  DevBufs bufs(st);
  float2 *a, *b;
  TRY(bufs.get(&a, sizeof(float2) * n2));
  TRY(bufs.get(&b, sizeof(float2) * n2));
  const dim3 pg(div_up(N, 256), N), sg(div_up(N, 32), div_up(N, 8));
  k_paste<<<pg, 256, 0, st>>>(a, N, band, n);
  k_paste<<<pg, 256, 0, st>>>(b, N, band, n);
  FSIM_CHECK_LAUNCH();
  TRY(fft2d_device(b, N, N, true, st));  // timesShiftVector(kx, -ky) between the transforms
  k_shift_ramp<<<sg, dim3(32, 8), 0, st>>>(b, N, kx, -ky);
  FSIM_CHECK_LAUNCH();
  TRY(fft2d_device(b, N, N, false, st));
  double sr = 0, si = 0, n2a = 0;
  TRY(reduce_device(3, reinterpret_cast<const float*>(a), reinterpret_cast<const float*>(b), 2 * n2, 1, st, &sr, &si));
  TRY(norm2_device(a, n2, &n2a, st));
  *re = sr / n2a;
  *im = si / n2a;
  return FSIM_OK;
}

int run_reconstruction_device(const fsim_sim_param* p, const float2* const* spec, float* out, bool otf_before_shift,
                              int clip_scale, cudaStream_t st) {
  TRY(validate_param(p));
  const int N = p->w, W = 2 * N, nP = p->nr_phases, nB = p->nr_bands, nC = 2 * nB - 1;
  const size_t n = (size_t)N * N, n2 = (size_t)W * W;
  DevBufs bufs(st);
  float2 *sep, *shifted, *full, *apo;
  float *denom, *part;
  TRY(bufs.get(&sep, sizeof(float2) * n * nC));
  TRY(bufs.get(&shifted, sizeof(float2) * n2 * nC));
  TRY(bufs.get(&full, sizeof(float2) * n2));
  TRY(bufs.get(&apo, sizeof(float2) * n2));
  TRY(bufs.get(&denom, sizeof(float) * n2));
  TRY(bufs.get(&part, sizeof(float) * 1024));
  DevOtf otf;
  TRY(otf.set(p, st));
  OtfTable ht;
  build_otf_table(p, &ht);
  // SimParam.useWienerFilter / useRLonInput / useRLonOutput (S/SimParam.java:287-304)
  const int fs = p->filter_style;
  const bool use_wiener = fs == FSIM_FILTER_WIENER || fs == FSIM_FILTER_RL_IN;
  const bool rl_in = fs == FSIM_FILTER_RL_IN || fs == FSIM_FILTER_RL_BOTH;
  const bool rl_out = fs == FSIM_FILTER_RL_OUT || fs == FSIM_FILTER_RL_BOTH;
  // RL on the input deconvolves the first nrBand*2-1 input images and separates those
  // (S/SimAlgorithm.java:331-354): with more phases than components the reference throws
  FSIM_REQUIRE(!rl_in || nP == nC, FSIM_EINVAL, "#input images != phases per band");
  float2 *in_otf = nullptr, *rl_tmp = nullptr;
  if (rl_in) {
    TRY(bufs.get(&in_otf, sizeof(float2) * n));
    TRY(bufs.get(&rl_tmp, sizeof(float2) * n * nC));
    TRY(otf_vector_device(in_otf, N, N, otf.d, 0, 0, 0, false, true, st));  // writeOtfVector(band 0)
  }
  // WienerFilter(param) + getDenominator(wiener) (SimAlgorithm.java:298, 509)
  TRY(wiener_denominator_device(denom, p, p->wiener, otf.d, true, st));
  FSIM_CUDA(cudaMemsetAsync(full, 0, sizeof(float2) * n2, st));
  const dim3 pg(div_up(W, 256), W), sg(div_up(W, 32), div_up(W, 8));
  for (int a = 0; a < p->nr_dirs; a++) {
    auto coef = separation_coeffs(p, a, false);
    SepArgs sa{};
    sa.n_in = nP;
    sa.n_out = nC;
    for (int i = 0; i < nP; i++) sa.in[i] = spec[a * nP + i];
    if (rl_in) {
      for (int i = 0; i < nC; i++) {
        float2* t = rl_tmp + (size_t)i * n;
        FSIM_CUDA(cudaMemcpyAsync(t, spec[a * nP + i], sizeof(float2) * n, cudaMemcpyDeviceToDevice, st));
        TRY(rl_deconvolve_device(t, in_otf, N, N, p->rl_iterations, true, st));
        sa.in[i] = t;
      }
    }
    for (int b = 0; b < nC; b++) sa.out[b] = sep + b * n;
    for (int b = 0; b < nC; b++)
      for (int q = 0; q < nP; q++) sa.coef[b * nP + q] = make_float2(coef[b * nP + q].real(), coef[b * nP + q].imag());
    TRY(separate_device(sa, n, st));
    if (otf_before_shift && use_wiener)
      for (int i = 0; i < nC; i++) TRY(otf_vector_device(sep + i * n, N, N, otf.d, (i + 1) / 2, 0, 0, p->use_attenuation, false, st));
    for (int i = 0; i < nC; i++) k_paste<<<pg, 256, 0, st>>>(shifted + i * n2, W, sep + i * n, N);
    FSIM_CHECK_LAUNCH();
    for (int b = 1; b < nB; b++) {
      for (int sgn = 0; sgn < 2; sgn++) {
        const int comp = sgn == 0 ? 2 * b : 2 * b - 1;
        const double kx = (sgn == 0 ? 1 : -1) * band_px(p, a, b), ky = (sgn == 0 ? 1 : -1) * band_py(p, a, b);
        float2* v = shifted + comp * n2;
        // SimUtils.fourierShift: ifft, times exp(i 2pi (kx x - ky y)/N), fft (S/SimUtils.java:43-50)
        TRY(fft2d_device(v, W, W, true, st));
        k_shift_ramp<<<sg, dim3(32, 8), 0, st>>>(v, W, kx, -ky);
        FSIM_CHECK_LAUNCH();
        TRY(fft2d_device(v, W, W, false, st));
      }
    }
    if (!use_wiener) {
      // RL styles: no OTF on the shifted bands; band 0 scaled by 1.f/nrDir for RL on the output
      if (rl_out) {
        k_scal_band0<<<grid1(n2), 256, 0, st>>>(shifted, n2, 1.f / (float)p->nr_dirs);
        FSIM_CHECK_LAUNCH();
      }
    } else if (!otf_before_shift) {
      TRY(otf_vector_device(shifted, W, W, otf.d, 0, 0, 0, p->use_attenuation, false, st));
      for (int b = 1; b < nB; b++) {
        TRY(otf_vector_device(shifted + 2 * b * n2, W, W, otf.d, b, band_px(p, a, b), band_py(p, a, b), p->use_attenuation,
                              false, st));
        TRY(otf_vector_device(shifted + (2 * b - 1) * n2, W, W, otf.d, b, -band_px(p, a, b), -band_py(p, a, b),
                              p->use_attenuation, false, st));
      }
    } else {
      // the reference passes (angIdx, component) as the mask centre (S/SimAlgorithm.java:407-409)
      for (int i = 0; i < nC; i++)
        k_mask<<<dim3(div_up(W, 128), W), 128, 0, st>>>(shifted + i * n2, W, W, ht.vec_cpm, ht.cutoff, (double)a, (double)i);
      FSIM_CHECK_LAUNCH();
    }
    for (int i = 0; i < nC; i++) k_accum<<<grid1(n2), 256, 0, st>>>(full, shifted + i * n2, n2);
    FSIM_CHECK_LAUNCH();
  }
  if (use_wiener) {
    // Wiener denominator, then apodization (bend apo_bend, cutoff apo_cutoff) as a complex vector
    TRY(times_real_device(full, denom, n2, st));
    TRY(apo_device(reinterpret_cast<float*>(apo), 1, W, W, ht.vec_cpm, ht.cutoff * p->apo_cutoff, p->apo_bend, st));
    TRY(times_cplx_device(full, apo, n2, false, st));
  } else {
    // RL on the output with the effective SIM OTF: band 0 (1/nrDir per direction) and every
    // other band at +-k of every direction (S/SimAlgorithm.java:591-611, 630-631); `apo`
    // holds the sum, shifted[0] / shifted[1] the OTF vectors
    float2 *osim = apo, *opos = shifted, *oneg = shifted + n2;
    FSIM_CUDA(cudaMemsetAsync(osim, 0, sizeof(float2) * n2, st));
    for (int a = 0; a < p->nr_dirs; a++)
      for (int b = 0; b < nB; b++) {
        const double kx = band_px(p, a, b), ky = band_py(p, a, b);
        TRY(otf_vector_device(opos, W, W, otf.d, b, kx, ky, false, true, st));
        if (b == 0) {
          k_scal_band0<<<grid1(n2), 256, 0, st>>>(opos, n2, 1.f / (float)p->nr_dirs);
          k_accum<<<grid1(n2), 256, 0, st>>>(osim, opos, n2);
        } else {
          TRY(otf_vector_device(oneg, W, W, otf.d, b, -kx, -ky, false, true, st));
          k_accum<<<grid1(n2), 256, 0, st>>>(osim, opos, n2);
          k_accum<<<grid1(n2), 256, 0, st>>>(osim, oneg, n2);
        }
        FSIM_CHECK_LAUNCH();
      }
    TRY(rl_deconvolve_device(full, osim, W, W, p->rl_iterations, true, st));
  }
  // SimUtils.spatial: inverse FFT, real part, clipAndScale
  TRY(fft2d_device(full, W, W, true, st));
  k_real_part<<<grid1(n2), 256, 0, st>>>(out, full, n2);
  FSIM_CHECK_LAUNCH();
  if (clip_scale == 1 || clip_scale == 2) {
    k_max_partial<<<256, 256, 0, st>>>(out, n2, part);
    k_clip_scale<<<grid1(n2), 256, 0, st>>>(out, n2, part, 256, clip_scale == 2);
    FSIM_CHECK_LAUNCH();
  }
  otf.release(st);
  return FSIM_OK;
}

}  // namespace fsim

using namespace fsim;

#define NEED_INIT()          \
  do {                       \
    int rc_ = ensure_init(); \
    if (rc_) return rc_;     \
  } while (0)

static int spectra_ptrs(const fsim_sim_param* p, fsim_vec* const* in, std::vector<const float2*>& out) {
  const int k = p->nr_dirs * p->nr_phases;
  out.resize(k);
  for (int i = 0; i < k; i++) {
    FSIM_REQUIRE(in && in[i] && in[i]->cplx && in[i]->w == p->w && in[i]->h == p->w, FSIM_EINVAL,
                 "input spectrum %d: complex %d x %d vector required", i, p->w, p->w);
    out[i] = reinterpret_cast<const float2*>(in[i]->d);
  }
  return FSIM_OK;
}

extern "C" {

int fsim_common_region(fsim_vec* b0, fsim_vec* b1, const fsim_sim_param* p, double kx, double ky, double dist,
                       double weight_limit, int divide) {
  NEED_INIT();
  FSIM_REQUIRE(b0 && b1 && b0->cplx && b1->cplx && b0->n == b1->n && b0->w == p->w, FSIM_EINVAL,
               "commonRegion: complex w x w vectors required");
  TRY(validate_param(p));
  cudaStream_t st = ctx().stream;
  DevOtf otf;
  TRY(otf.set(p, st));
  int rc = common_region_device(reinterpret_cast<float2*>(b0->d), reinterpret_cast<float2*>(b1->d), b0->w, b0->h,
                                otf.d, kx, ky, dist, weight_limit, divide != 0, st);
  otf.release(st);
  return rc;
}

int fsim_locate_peak(const fsim_vec* v, double k_min, double out4[4]) {
  NEED_INIT();
  FSIM_REQUIRE(v && v->cplx, FSIM_EINVAL, "locatePeak: complex vector required");
  EstScratch s;
  TRY(s.alloc(8, ctx().stream));
  int rc = locate_peak_device(reinterpret_cast<const float2*>(v->d), v->w, v->h, k_min, s, ctx().stream, out4);
  s.free(ctx().stream);
  return rc;
}

int fsim_fit_peak(const fsim_vec* band0, const fsim_vec* band1, const fsim_sim_param* p, double kx, double ky,
                  double weight_limit, double search, double out4[4], double* grid_out) {
  NEED_INIT();
  FSIM_REQUIRE(band0 && band1 && band0->cplx && band1->cplx && band0->w == band0->h && band0->n == band1->n,
               FSIM_EINVAL, "fitPeak: square complex vectors of equal size required");
  TRY(validate_param(p));
  cudaStream_t st = ctx().stream;
  DevOtf otf;
  TRY(otf.set(p, st));
  EstScratch s;
  TRY(s.alloc(band0->w, st));
  int rc = fit_peak_device(reinterpret_cast<const float2*>(band0->d), reinterpret_cast<const float2*>(band1->d),
                           band0->w, otf.d, kx, ky, weight_limit, search, s, st, out4, grid_out);
  s.free(st);
  otf.release(st);
  return rc;
}

int fsim_get_peak(const fsim_vec* band0, const fsim_vec* band1, const fsim_sim_param* p, double kx, double ky,
                  double weight_limit, double out2[2]) {
  NEED_INIT();
  FSIM_REQUIRE(band0 && band1 && band0->cplx && band1->cplx && band0->w == band0->h && band0->n == band1->n,
               FSIM_EINVAL, "getPeak: square complex vectors of equal size required");
  TRY(validate_param(p));
  cudaStream_t st = ctx().stream;
  DevOtf otf;
  TRY(otf.set(p, st));
  EstScratch s;
  TRY(s.alloc(band0->w, st));
  std::complex<double> r;
  int rc = get_peak_device(reinterpret_cast<const float2*>(band0->d), reinterpret_cast<const float2*>(band1->d),
                           band0->w, otf.d, kx, ky, weight_limit, s, st, &r);
  s.free(st);
  otf.release(st);
  out2[0] = r.real();
  out2[1] = r.imag();
  return rc;
}

int fsim_estimate_parameters(fsim_sim_param* p, fsim_vec* const* in_fft, int fit_band, double fit_exclude,
                             double* peaks_out) {
  NEED_INIT();
  TRY(validate_param(p));
  std::vector<const float2*> sp;
  TRY(spectra_ptrs(p, in_fft, sp));
  return estimate_core(p, sp.data(), fit_band, fit_exclude, false, peaks_out, ctx().stream);
}

int fsim_estimate_raw(fsim_sim_param* p, const void* raw_device, int input_type, int fade_px, int fit_band,
                      double fit_exclude, double* peaks_out) {
  NEED_INIT();
  TRY(validate_param(p));
  FSIM_REQUIRE(raw_device, FSIM_EINVAL, "null raw pointer");
  cudaStream_t st = ctx().stream;
  const int frames = p->nr_dirs * p->nr_phases;
  const size_t n = (size_t)p->w * p->w;
  DevBufs bufs(st);
  float2* spec;
  TRY(bufs.get(&spec, sizeof(float2) * n * frames));
  TRY(raw_to_spectra(p, raw_device, input_type == FSIM_INPUT_U16, fade_px, spec, bufs, st));
  std::vector<const float2*> ptrs(frames);
  for (int i = 0; i < frames; i++) ptrs[i] = spec + i * n;
  return estimate_core(p, ptrs.data(), fit_band, fit_exclude, false, peaks_out, st);
}

int fsim_live_refit(fsim_sim_param* p, const uint16_t* raw_device, double* peaks_out) {
  NEED_INIT();
  TRY(validate_param(p));
  FSIM_REQUIRE(raw_device, FSIM_EINVAL, "null raw pointer");
  cudaStream_t st = ctx().stream;
  const int frames = p->nr_dirs * p->nr_phases;
  const size_t n = (size_t)p->w * p->w;
  DevBufs bufs(st);
  float2* spec;
  TRY(bufs.get(&spec, sizeof(float2) * n * frames));
  TRY(raw_to_spectra(p, raw_device, 1, 10, spec, bufs, st));
  std::vector<const float2*> ptrs(frames);
  for (int i = 0; i < frames; i++) ptrs[i] = spec + i * n;
  return estimate_core(p, ptrs.data(), 1, .8, true, peaks_out, st);
}

int fsim_rl_deconvolve(fsim_vec* img, const fsim_vec* otf, int steps, int input_in_freq_space) {
  NEED_INIT();
  FSIM_REQUIRE(img && otf && img->d && otf->d && img->cplx && otf->cplx, FSIM_EINVAL,
               "RL deconvolution: complex image and OTF vectors required");
  FSIM_REQUIRE(img->w == otf->w && img->h == otf->h, FSIM_EINVAL, "RL deconvolution: size mismatch %dx%d / %dx%d",
               img->w, img->h, otf->w, otf->h);
  return rl_deconvolve_device(reinterpret_cast<float2*>(img->d), reinterpret_cast<const float2*>(otf->d), img->w,
                              img->h, steps, input_in_freq_space != 0, ctx().stream);
}

int fsim_auto_correlation(const fsim_vec* band, double kx, double ky, double* re, double* im) {
  NEED_INIT();
  FSIM_REQUIRE(band && band->d && band->cplx && re && im, FSIM_EINVAL, "autoCorrelation: null argument");
  FSIM_REQUIRE(band->w == band->h, FSIM_EINVAL, "Vector len mismatch %d %d", band->w, band->h);  // checkSquare
  return auto_correlation_device(reinterpret_cast<const float2*>(band->d), band->w, kx, ky, re, im, ctx().stream);
}

int fsim_run_reconstruction(const fsim_sim_param* p, fsim_vec* const* in_fft, fsim_vec* out_real, int otf_before_shift,
                            int clip_scale) {
  NEED_INIT();
  TRY(validate_param(p));
  FSIM_REQUIRE(out_real && !out_real->cplx && out_real->w == 2 * p->w && out_real->h == 2 * p->w, FSIM_EINVAL,
               "runReconstruction: output must be a real 2w x 2w vector");
  std::vector<const float2*> sp;
  TRY(spectra_ptrs(p, in_fft, sp));
  return run_reconstruction_device(p, sp.data(), out_real->d, otf_before_shift != 0, clip_scale, ctx().stream);
}

}  // extern "C"
