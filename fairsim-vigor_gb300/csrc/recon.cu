// Fused, batched 2D SIM reconstruction: SimAlgorithm.runReconstruction
// (S/SimAlgorithm.java:268-582; Wiener filter style, OTF applied after a Fourier shift on
// the 2w x 2w grid) in three passes over HBM instead of ~40 vector ops.
//
// The reference's per-component chain, with W = 2N,
//   sep_c = sum_p M[c][p] FFT_N(raw_p);  V_c = FFT_W(ramp_c * iFFT_W(paste(sep_c)));
//   T = sum_{a,c} conj(OTF(r - k_c)) V_c;  out = Re iFFT_W(T * wiener * apo)
// is separable along x and y except for the OTF/Wiener/apo multiplications, which act
// where both axes are in frequency space. The passes are therefore:
//   A  (rows,    per dataset x angle x raw row): band mix of the raw rows in real space
//      (FFT is linear, so mixing before the transform is the same separation), FFT_N along
//      x, paste, and for shifted components the x half of the shift
//      (iFFT_W, ramp_x, FFT_W) -> only the columns inside each component's OTF support
//      window are written (the OTF zeroes everything else);
//   B  (columns, per dataset x 4-column quad): FFT_N along y, paste, y half of the shift,
//      times the exact conj(OTF) mask, accumulate all components, times wiener*apo,
//      iFFT_W along y;
//   C  (rows,    per output row): iFFT_W along x, real part, 1/W^2.
// Shift phases use exact per-axis ramp tables; OTF masks and the Wiener*apo filter are
// resident per plan, built with the reference's double-precision radius and floor-indexed
// OTF lookup.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fft_line.cuh"
#include "filters.cuh"
#include "otf.cuh"
#include "recon.cuh"
#include "runtime.cuh"
#include "sim_host.h"

namespace fsim {

std::vector<float> fade_vector(int w, int h, int px);

// ---- per-size launch configuration -------------------------------------------------------
template <int N>
struct Cfg {
  static constexpr int W = 2 * N;
  static constexpr int EW = (N % 3 == 0) ? 24 : 16;  // elements per thread in W-length lines
  static constexpr int T = W / EW;                    // threads per line
  static constexpr int CB = (N >= 2048) ? 2 : 4;      // interleaved columns in pass B
  static constexpr int GC = (T >= 128) ? 1 : (128 / T);  // rows per block in pass C
};

// ---- pass A ------------------------------------------------------------------------------
// Copies a job descriptor into shared memory once per block (the passes read its fields
// after global stores, which would otherwise force reloads).
__device__ __forceinline__ void load_job(JobDesc* dst, const JobDesc* src, int tid, int nthreads) {
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int i = tid; i < (int)(sizeof(JobDesc) / sizeof(int)); i += nthreads) d[i] = s[i];
}

template <int N>
__global__ void __launch_bounds__(Cfg<N>::T, (Cfg<N>::T <= 64 ? 8 : 4)) k_pass_a(const JobDesc* __restrict__ jobs) {
  using P = Cfg<N>;
  constexpr int W = P::W, T = P::T, EN = N / T, EW = W / T;
  const int y = blockIdx.x, a = blockIdx.y, t = threadIdx.x;
  __shared__ JobDesc J;
  __shared__ float2 s[smem_line_elems(W, 1)];
  __shared__ float2 twN[stw_len(N, EN)], twW[stw_len(W, EW)];
  __shared__ float2 coef[SEP_MAX_OUT * FSIM_MAX_PHASES];
  extern __shared__ float rows[];  // nP raw rows of this image row, damped
  load_job(&J, jobs + blockIdx.z, t, T);
  stage_stage_twiddles<N, EN>(twN, t, T);
  stage_stage_twiddles<W, EW>(twW, t, T);
  __syncthreads();
  if (a >= J.nA) return;  // uniform per block
  const int nP = J.nP, nC = J.nC;
  for (int i = t; i < nC * nP; i += T) coef[i] = J.coef[a * nC * nP + i];
  const size_t frame = (size_t)N * N, row = (size_t)y * N;
  for (int p = 0; p < nP; p++) {
    const size_t base = (size_t)(a * nP + p) * frame + row;
#pragma unroll
    for (int i = 0; i < EN; i++) {
      const int x = t + i * T;
      float v = J.input_u16 ? (float)((const uint16_t*)J.raw)[base + x] : ((const float*)J.raw)[base + x];
      if (J.bgr != 0.f) {
        v = v - J.bgr;
        if (v < 0) v = 0;
      }
      if (J.damp) v = v * J.damp[row + x];
      rows[p * N + x] = v;
    }
  }
  __syncthreads();
  for (int c = 0; c < nC; c++) {
    // band mix of the raw rows in real space
#pragma unroll
    for (int i = 0; i < EN; i++) {
      const int x = t + i * T;
      float2 z = make_float2(0.f, 0.f);
      for (int p = 0; p < nP; p++) {
        const float2 m = coef[c * nP + p];
        const float v = rows[p * N + x];
        z.x += m.x * v;
        z.y += m.y * v;
      }
      s[sidx(x)] = z;
    }
    __syncthreads();
    line_fft_st<N, T, 1, false>(s, t, twN);
    // paste along x: m < N/2 stays, m >= N/2 moves to m + N; the middle becomes zero
    float2 v[EN];
#pragma unroll
    for (int i = 0; i < EN; i++) v[i] = s[sidx(t + i * T)];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < EN; i++) {
      const int m = t + i * T;
      s[sidx(m < N / 2 ? m : m + N)] = v[i];
      s[sidx(N / 2 + m)] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (c > 0) {
      line_fft_st<W, T, 1, true>(s, t, twW);
      const float2* rx = J.ramps + (size_t)(a * nC + c) * 2 * W;
#pragma unroll
      for (int i = 0; i < EW; i++) {
        const int k = t + i * T;
        s[sidx(k)] = cmul(s[sidx(k)], __ldg(&rx[k]));
      }
      __syncthreads();
      line_fft_st<W, T, 1, false>(s, t, twW);
    }
    // keep the OTF-support window: columns Xs .. Xs+nWin-1 (mod W), quad layout
    const int Xs = J.win[2 * (a * nC + c)];
    float2* I = J.I + (size_t)(a * nC + c) * J.nWin * N;
    for (int xl = t; xl < J.nWin; xl += T) {
      int X = Xs + xl;
      if (X >= W) X -= W;
      I[((size_t)(xl >> 2) * N + y) * 4 + (xl & 3)] = s[sidx(X)];
    }
    __syncthreads();
  }
}

// ---- pass B ------------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(Cfg<N>::CB* Cfg<N>::T, (Cfg<N>::CB * Cfg<N>::T <= 256 ? 2 : 1)) k_pass_b(const JobDesc* __restrict__ jobs) {
  using P = Cfg<N>;
  constexpr int W = P::W, T = P::T, CB = P::CB, EN = N / T, EW = W / T;
  const int q = blockIdx.x;  // column group: X = q*CB + lane
  const int lt = threadIdx.x, lane = lt % CB, t = lt / CB;
  __shared__ JobDesc J;
  __shared__ float2 twN[stw_len(N, EN)], twW[stw_len(W, EW)];
  extern __shared__ float2 sm[];
  float2* acc = sm;
  float2* wk = sm + smem_line_elems(W, CB);
  load_job(&J, jobs + blockIdx.y, lt, CB * T);
  stage_stage_twiddles<N, EN>(twN, lt, CB * T);
  stage_stage_twiddles<W, EW>(twW, lt, CB * T);
  __syncthreads();
  const int nC = J.nC, nWin = J.nWin;
#pragma unroll
  for (int i = 0; i < EW; i++) acc[sidx((t + i * T) * CB + lane)] = make_float2(0.f, 0.f);
  // components: band 0 of all angles shares the unshifted mask and is summed before its
  // FFT; every shifted component is transformed on its own.
  for (int a = -1; a < J.nA; a++) {
    for (int c = (a < 0 ? 0 : 1); c < (a < 0 ? 1 : nC); c++) {
      const int aw = a < 0 ? 0 : a;
      int xl = q * CB - J.win[2 * (aw * nC + c)];
      if (xl < 0) xl += W;
      if (xl >= nWin) continue;  // uniform: the whole group is outside this window
      const int qi = xl / 4, sub = xl & 3;
      // load the window column(s), summing band 0 over angles
#pragma unroll
      for (int i = 0; i < EN; i++) {
        const int k = t + i * T;
        float2 v = make_float2(0.f, 0.f);
        const int a0 = a < 0 ? 0 : a, a1 = a < 0 ? J.nA : a + 1;
        for (int aa = a0; aa < a1; aa++) {
          const float2* I = J.I + (size_t)(aa * nC + c) * nWin * N;
          const float2 u = I[((size_t)qi * N + k) * 4 + sub + lane];
          v.x += u.x;
          v.y += u.y;
        }
        wk[sidx(k * CB + lane)] = v;
      }
      __syncthreads();
      line_fft_st<N, T, CB, false>(wk, lt, twN);
      float2 v[EN];
#pragma unroll
      for (int i = 0; i < EN; i++) v[i] = wk[sidx((t + i * T) * CB + lane)];
      __syncthreads();
#pragma unroll
      for (int i = 0; i < EN; i++) {
        const int m = t + i * T;
        wk[sidx((m < N / 2 ? m : m + N) * CB + lane)] = v[i];
        wk[sidx((N / 2 + m) * CB + lane)] = make_float2(0.f, 0.f);
      }
      __syncthreads();
      if (c > 0) {
        line_fft_st<W, T, CB, true>(wk, lt, twW);
        const float2* ry = J.ramps + (size_t)(a * nC + c) * 2 * W + W;
#pragma unroll
        for (int i = 0; i < EW; i++) {
          const int k = t + i * T;
          wk[sidx(k * CB + lane)] = cmul(wk[sidx(k * CB + lane)], __ldg(&ry[k]));
        }
        __syncthreads();
        line_fft_st<W, T, CB, false>(wk, lt, twW);
      }
      // times conj(OTF) inside the window rows, accumulate
      const int Ys = J.win[2 * (aw * nC + c) + 1];
      const float* mk = J.masks + (size_t)(aw * nC + c) * nWin * nWin;
      for (int yl = t; yl < nWin; yl += T) {
        int Y = Ys + yl;
        if (Y >= W) Y -= W;
        const float m = __ldg(&mk[((size_t)qi * nWin + yl) * 4 + sub + lane]);
        const float2 u = wk[sidx(Y * CB + lane)];
        float2& o = acc[sidx(Y * CB + lane)];
        o.x += m * u.x;
        o.y += m * u.y;
      }
      __syncthreads();
    }
  }
  // Wiener denominator x apodization, then the inverse transform along y
  const int X0 = q * CB;
  const float* wa = J.wa + (size_t)(X0 / 4) * W * 4 + (X0 & 3);
#pragma unroll
  for (int i = 0; i < EW; i++) {
    const int k = t + i * T;
    const float f = __ldg(&wa[(size_t)k * 4 + lane]);
    float2& o = acc[sidx(k * CB + lane)];
    o.x *= f;
    o.y *= f;
  }
  __syncthreads();
  line_fft_st<W, T, CB, true>(acc, lt, twW);
#pragma unroll
  for (int i = 0; i < EW; i++) {
    const int k = t + i * T;
    J.O[(size_t)k * W + X0 + lane] = acc[sidx(k * CB + lane)];
  }
}

// ---- pass C ------------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(Cfg<N>::GC* Cfg<N>::T) k_pass_c(const JobDesc* __restrict__ jobs) {
  using P = Cfg<N>;
  constexpr int W = P::W, T = P::T, G = P::GC, EW = W / T;
  const JobDesc& J = jobs[blockIdx.y];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int Y = blockIdx.x * G + g;
  __shared__ float2 sm[G * smem_line_elems(W, 1)];
  __shared__ float2 tw[stw_len(W, EW)];
  stage_stage_twiddles<W, EW>(tw, threadIdx.x, G * T);
  float2* s = sm + g * smem_line_elems(W, 1);
  const float2* row = J.O + (size_t)Y * W;
#pragma unroll
  for (int i = 0; i < EW; i++) s[sidx(t + i * T)] = row[t + i * T];
  __syncthreads();
  line_fft_st<W, T, 1, true>(s, t, tw);
  const float scale = 1.f / ((float)W * (float)W);
  float* out = J.out + (size_t)Y * W;
#pragma unroll
  for (int i = 0; i < EW; i++) out[t + i * T] = s[sidx(t + i * T)].x * scale;
}

// ---- plan build kernels -------------------------------------------------------------------------
// conj(OTF(r - k)) mask of one component over its window, quad layout [xl/4][yl][xl%4]
__global__ void k_build_mask(float* __restrict__ mask, int W, int nWin, int Xs, int Ys, double kx, double ky,
                             const OtfTable* __restrict__ t, int att) {
  const int xl = blockIdx.x * blockDim.x + threadIdx.x, yl = blockIdx.y;
  if (xl >= nWin) return;
  int X = (Xs + xl) % W, Y = (Ys + yl) % W;
  float v = 0.f;
  if (!otf_at(*t, (double)freq_x(X, W), (double)freq_y(Y, W), kx, ky, att != 0, &v)) v = 0.f;
  mask[((size_t)(xl >> 2) * nWin + yl) * 4 + (xl & 3)] = v;
}

// 1/(sum |OTF|^2 + w^2) * apo, quad layout [X/4][Y][X%4]
__global__ void k_build_wa(float* __restrict__ wa, int W, const OtfTable* __restrict__ t, ShiftSet shifts, int use_att,
                           float wp, double apo_cut_abs, double bend) {
  const int X = blockIdx.x * blockDim.x + threadIdx.x, Y = blockIdx.y;
  if (X >= W) return;
  const double xh = freq_x(X, W), yh = freq_y(Y, W);
  const double cpm = t->vec_cpm;
  float acc = 0.f;
  for (int d = 0; d < shifts.n_dirs; d++)
    for (int b = 0; b < shifts.n_bands; b++) {
      const double kx = shifts.px[d] * b, ky = shifts.py[d] * b;
      double r1 = __dmul_rn(d_hypot_java(__dsub_rn(xh, kx), __dsub_rn(yh, ky)), cpm);
      double r2 = __dmul_rn(d_hypot_java(__dadd_rn(xh, kx), __dadd_rn(yh, ky)), cpm);
      float o1 = otf_val(*t, r1, false), o2 = otf_val(*t, r2, false);
      float v1 = __fmul_rn(o1, o1), v2 = __fmul_rn(o2, o2);
      if (use_att) {
        v1 = __fmul_rn(v1, att_val(*t, r1));
        v2 = __fmul_rn(v2, att_val(*t, r2));
      }
      acc = __fadd_rn(__fadd_rn(acc, v1), v2);
    }
  const float den = __fdiv_rn(1.f, __fadd_rn(acc, wp));
  double rad = d_hypot_java(xh, yh);
  double frac = __dmul_rn(rad, cpm) / apo_cut_abs;
  const float apo = (float)pow(ideal_otf_dev(frac), bend);
  wa[((size_t)(X >> 2) * W + Y) * 4 + (X & 3)] = __fmul_rn(den, apo);
}

// ---- plan --------------------------------------------------------------------------------------
static int floor4(int v) { return (v >= 0) ? (v / 4) * 4 : -(((-v) + 3) / 4) * 4; }

int plan_window(const fsim_sim_param* p, double R, int* nwin) {
  const int W = 2 * p->w;
  int n = ((2 * (int)std::ceil(R) + 3 + 3) / 4) * 4 + 4;
  if (n >= W) n = W;
  *nwin = n;
  return FSIM_OK;
}

static void comp_shift(const fsim_sim_param* p, int a, int c, double* kx, double* ky) {
  if (c == 0) {
    *kx = 0;
    *ky = 0;
    return;
  }
  const int b = (c + 1) / 2;
  const double s = (c % 2 == 0) ? 1.0 : -1.0;  // pos = 2b, neg = 2b-1 (SimAlgorithm.java:385-391)
  *kx = s * band_px(p, a, b);
  *ky = s * band_py(p, a, b);
}

int Plan::build(cudaStream_t st) {
  const int N = prm.w, W = 2 * N, nA = prm.nr_dirs, nP = prm.nr_phases, nC = 2 * prm.nr_bands - 1;
  OtfTable ht;
  build_otf_table(&prm, &ht);
  const double R = ht.cutoff / ht.vec_cpm;  // OTF support radius in frequency pixels
  plan_window(&prm, R, &nwin);
  // host-side tables
  std::vector<float2> coef((size_t)nA * nC * nP);
  for (int a = 0; a < nA; a++) {
    auto m = separation_coeffs(&prm, a, false);
    for (int c = 0; c < nC; c++)
      for (int q = 0; q < nP; q++) coef[(a * nC + c) * nP + q] = make_float2(m[c * nP + q].real(), m[c * nP + q].imag());
  }
  std::vector<float2> ramps((size_t)nA * nC * 2 * W);
  std::vector<int> win((size_t)nA * nC * 2);
  for (int a = 0; a < nA; a++)
    for (int c = 0; c < nC; c++) {
      double kx, ky;
      comp_shift(&prm, a, c, &kx, &ky);
      float2* rx = &ramps[(size_t)(a * nC + c) * 2 * W];
      float2* ry = rx + W;
      for (int n = 0; n < W; n++) {
        // x: exp(+2 pi i kx n/W)/W ; y: exp(-2 pi i ky n/W)/W  (fourierShift(kx, -ky))
        double fx = kx * n / W, fy = -ky * n / W;
        fx -= std::floor(fx);
        fy -= std::floor(fy);
        rx[n] = make_float2((float)(std::cos(2 * M_PI * fx) / W), (float)(std::sin(2 * M_PI * fx) / W));
        ry[n] = make_float2((float)(std::cos(2 * M_PI * fy) / W), (float)(std::sin(2 * M_PI * fy) / W));
      }
      int xs, ys;
      if (nwin >= W) {
        xs = 0;
        ys = 0;
      } else {
        int xlo = (int)std::floor(kx - R) - 1;
        int ylo = (int)std::floor(-ky - R) - 1;  // index-space row of display y: Y = -yh mod W
        xs = ((floor4(xlo) % W) + W) % W;
        ys = ((ylo % W) + W) % W;
      }
      win[2 * (a * nC + c)] = xs;
      win[2 * (a * nC + c) + 1] = ys;
    }
  // device layout: one allocation
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t off_coef = 0, off_ramp = off_coef + al(coef.size() * sizeof(float2));
  size_t off_win = off_ramp + al(ramps.size() * sizeof(float2));
  size_t off_otf = off_win + al(win.size() * sizeof(int));
  size_t off_damp = off_otf + al(sizeof(OtfTable));
  size_t off_mask = off_damp + al((size_t)N * N * sizeof(float));
  size_t off_wa = off_mask + al((size_t)nA * nC * nwin * nwin * sizeof(float));
  size_t total = off_wa + al((size_t)W * W * sizeof(float));
  if (total > dev_bytes) {
    if (dev) cudaFree(dev);
    dev = nullptr;
    FSIM_CUDA(cudaMalloc(&dev, total));
    dev_bytes = total;
  }
  char* b = (char*)dev;
  d_coef = (float2*)(b + off_coef);
  d_ramps = (float2*)(b + off_ramp);
  d_win = (int*)(b + off_win);
  d_otf = (OtfTable*)(b + off_otf);
  d_damp = fade_px > 0 ? (float*)(b + off_damp) : nullptr;
  d_masks = (float*)(b + off_mask);
  d_wa = (float*)(b + off_wa);
  // uploads are synchronous (pageable sources on this stack frame)
  FSIM_CUDA(cudaMemcpyAsync(d_coef, coef.data(), coef.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_ramps, ramps.data(), ramps.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_win, win.data(), win.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_otf, &ht, sizeof(OtfTable), cudaMemcpyHostToDevice, st));
  if (d_damp) {
    std::vector<float> dv = fade_vector(N, N, fade_px);
    FSIM_CUDA(cudaMemcpyAsync(d_damp, dv.data(), dv.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    FSIM_CUDA(cudaStreamSynchronize(st));
  }
  FSIM_CUDA(cudaStreamSynchronize(st));
  // masks (exact double-precision OTF lookups), Wiener x apo
  for (int a = 0; a < nA; a++)
    for (int c = 0; c < nC; c++) {
      double kx, ky;
      comp_shift(&prm, a, c, &kx, &ky);
      dim3 g(div_up(nwin, 128), nwin);
      k_build_mask<<<g, 128, 0, st>>>(d_masks + (size_t)(a * nC + c) * nwin * nwin, W, nwin, win[2 * (a * nC + c)],
                                      win[2 * (a * nC + c) + 1], kx, ky, d_otf, prm.use_attenuation);
    }
  {
    dim3 g(div_up(W, 128), W);
    k_build_wa<<<g, 128, 0, st>>>(d_wa, W, d_otf, shift_set(&prm), prm.use_attenuation, (float)(prm.wiener * prm.wiener),
                                  ht.cutoff * prm.apo_cutoff, prm.apo_bend);
  }
  FSIM_CHECK_LAUNCH();
  FSIM_CUDA(cudaStreamSynchronize(st));
  filter_bytes = total;
  return FSIM_OK;
}

size_t Plan::workspace_bytes() const {
  const int N = prm.w, W = 2 * N, nC = 2 * prm.nr_bands - 1;
  size_t I = (size_t)prm.nr_dirs * nC * nwin * N * sizeof(float2);
  size_t O = (size_t)W * W * sizeof(float2);
  return ((I + 255) & ~(size_t)255) + ((O + 255) & ~(size_t)255);
}

void Plan::fill_job(JobDesc& j, const void* raw, float* out, float* wf, char* ws) const {
  const int N = prm.w, nC = 2 * prm.nr_bands - 1;
  j.raw = raw;
  j.out = out;
  j.widefield = wf;
  j.input_u16 = input_type == FSIM_INPUT_U16;
  j.nA = prm.nr_dirs;
  j.nP = prm.nr_phases;
  j.nC = nC;
  j.nWin = nwin;
  j.bgr = (float)bgr;
  j.damp = d_damp;
  j.coef = d_coef;
  j.ramps = d_ramps;
  j.win = d_win;
  j.masks = d_masks;
  j.wa = d_wa;
  size_t I = (size_t)prm.nr_dirs * nC * nwin * N * sizeof(float2);
  j.I = (float2*)ws;
  j.O = (float2*)(ws + ((I + 255) & ~(size_t)255));
}

// ---- launch --------------------------------------------------------------------------------------
template <int N>
static int launch_offline(const JobDesc* d_jobs, int njobs, int maxA, int maxP, cudaStream_t st) {
  cudaEvent_t* ev = profile_events();
  using P = Cfg<N>;
  constexpr int W = P::W;
  static bool attr = false;
  const size_t smem_b = sizeof(float2) * (2 * smem_line_elems(W, P::CB));
  if (!attr) {
    FSIM_CUDA(cudaFuncSetAttribute(k_pass_b<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b));
    FSIM_CUDA(cudaFuncSetAttribute(k_pass_a<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(sizeof(float) * FSIM_MAX_PHASES * N)));
    attr = true;
  }
  if (ev) cudaEventRecord(ev[0], st);
  k_pass_a<N><<<dim3(N, maxA, njobs), P::T, sizeof(float) * maxP * N, st>>>(d_jobs);
  if (ev) cudaEventRecord(ev[1], st);
  k_pass_b<N><<<dim3(W / P::CB, njobs), P::CB * P::T, smem_b, st>>>(d_jobs);
  if (ev) cudaEventRecord(ev[2], st);
  k_pass_c<N><<<dim3(W / P::GC, njobs), P::GC * P::T, 0, st>>>(d_jobs);
  if (ev) {
    cudaEventRecord(ev[3], st);
    profile_mark(3);
  }
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

#define FSIM_RECON_SIZES(X) X(64) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) X(2048)

bool offline_size_supported(int n) {
  switch (n) {
#define CASE(v) case v:
    FSIM_RECON_SIZES(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}

int launch_offline_size(int n, const JobDesc* d_jobs, int njobs, int maxA, int maxP, cudaStream_t st) {
  switch (n) {
#define CASE(v) \
  case v:       \
    return launch_offline<v>(d_jobs, njobs, maxA, maxP, st);
    FSIM_RECON_SIZES(CASE)
#undef CASE
  }
  set_error("fused reconstruction: unsupported image size %d", n);
  return FSIM_EINVAL;
}

}  // namespace fsim
