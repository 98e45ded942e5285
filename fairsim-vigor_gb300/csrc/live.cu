// Fused live reconstruction: the per-stack work of ReconstructionThread.run
// (LM/ReconstructionRunner.java:434-542) with the filters of setupFilters (:773-813):
// u16 frames x border damping, FFT_N, band separation, times conj(OTF) (band 0,
// attenuated), the *fast* shift of SimUtils.pasteAndFourierShift (S/SimUtils.java:65-91:
// fractional shift on the N grid, then pasteFreq at the integer offset), sum, times
// Wiener denominator and apodization (bend 1, cutoff 2), iFFT_W, real part; plus the
// widefield mean of the damped frames.
//
// The fractional shift FFT_N(ramp * iFFT_N(.)) is separable, but the OTF product sits
// between the forward transforms and the shift, so four passes are used:
//   LA rows    (per dataset x raw row):     damp, widefield, band mix, FFT_N along x
//   LB columns (per dataset x 4 columns):   FFT_N along y, x conj(OTF), y half of the shift
//   LC rows    (per dataset x output row):  x half of the shift, paste at the integer
//                                           offsets, sum, x Wiener*apo, iFFT_W along x
//   LD columns (per dataset x 8 columns):   iFFT_W along y, real part, 1/W^2
#include <cmath>
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
int plan_window(const fsim_sim_param* p, double R, int* nwin);

template <int N>
struct LCfg {
  static constexpr int W = 2 * N;
  static constexpr int EN = (N % 3 == 0) ? 12 : 16;
  static constexpr int TN = N / EN;                            // threads per N-line
  static constexpr int GA = TN >= 128 ? 1 : 128 / TN;          // rows per block, pass LA
  static constexpr int CBL = 4;                                // columns per block, pass LB
  static constexpr int EW = (N % 3 == 0) ? 24 : 16;
  static constexpr int TW = W / EW;                            // threads per W-line
  static constexpr int CD = (N >= 2048) ? 2 : (N >= 1024 ? 4 : 8);  // columns per block, pass LD
};

// Register budget of about 80 per thread for the column and shift passes (they otherwise keep
// 120-130 and run at 16 warps per SM).
__host__ __device__ constexpr int live_min_blocks(int threads) {
  return 65536 / (threads * 80) > 0 ? 65536 / (threads * 80) : 1;
}

// pasteFreq's source index for output index o (as in vec_ops.cu)
__device__ __forceinline__ int paste_source(int o, int off, int ni, int no) {
  int p1 = ((o - off) % no + no) % no;
  int p2 = ((o - off - no / 2) % no + no) % no;
  int best = -1;
  if (p1 < ni / 2) best = p1;
  if (p2 >= ni / 2 && p2 < ni && p2 > best) best = p2;
  return best;
}

// ---- LA -----------------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(LCfg<N>::GA* LCfg<N>::TN) k_live_a(const JobDesc* __restrict__ jobs) {
  using P = LCfg<N>;
  constexpr int T = P::TN, G = P::GA, E = P::EN;
  const JobDesc& J = jobs[blockIdx.y];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int y = blockIdx.x * G + g;
  __shared__ float2 sm[G * smem_line_elems(N, 1)];
  const float2* tw = g_stw + stw_offset(N, E);  // stage twiddles through L1
  float2* s = sm + g * smem_line_elems(N, 1);
  const size_t frame = (size_t)N * N, row = (size_t)y * N;
  const float* rawf = (const float*)J.raw;
  const uint16_t* rawu = (const uint16_t*)J.raw;
  const int nA = J.nA, nP = J.nP, nC = J.nC;
  // setFrom16bitPixels + times(dampBorder) of the row of frame f at this thread's elements
  // t + i*T; frames outer and elements inner, so that a row's E loads are in flight at once
  auto px_row = [&](int f, float (&v)[E]) {
    const size_t at = (size_t)f * frame + row + t;
    if (J.input_u16) {
#pragma unroll
      for (int i = 0; i < E; i++) v[i] = (float)__ldg(&rawu[at + i * T]);
    } else {
#pragma unroll
      for (int i = 0; i < E; i++) v[i] = __ldg(&rawf[at + i * T]);
    }
    if (J.damp) {
#pragma unroll
      for (int i = 0; i < E; i++) v[i] = __fmul_rn(v[i], __ldg(&J.damp[row + t + i * T]));
    }
  };
  if (J.widefield) {
    const float sc = 1.f / (float)(nA * nP);
    float wf[E];
#pragma unroll
    for (int i = 0; i < E; i++) wf[i] = 0.f;
#pragma unroll 1
    for (int f = 0; f < nA * nP; f++) {
      float v[E];
      px_row(f, v);
#pragma unroll
      for (int i = 0; i < E; i++) wf[i] = __fadd_rn(wf[i], v[i]);
    }
#pragma unroll
    for (int i = 0; i < E; i++) J.widefield[row + t + i * T] = __fmul_rn(wf[i], sc);
  }
  for (int a = 0; a < nA; a++)
    for (int c = 0; c < nC; c++) {
      const float2* coef = J.coef + (a * nC + c) * nP;
      float2 xv[E];  // element t + i*T of the line, in registers through the transform
#pragma unroll
      for (int i = 0; i < E; i++) xv[i] = make_float2(0.f, 0.f);
#pragma unroll 1
      for (int p = 0; p < nP; p++) {
        float v[E];
        px_row(a * nP + p, v);
        const float2 m = coef[p];
#pragma unroll
        for (int i = 0; i < E; i++) {
          xv[i].x += m.x * v[i];
          xv[i].y += m.y * v[i];
        }
      }
      line_fft_reg<N, T, 1, false>(xv, s, 0, t, tw);
      float2* X = J.I + (size_t)(a * nC + c) * frame + row;
#pragma unroll
      for (int i = 0; i < E; i++) X[t + i * T] = xv[i];
    }
}

// ---- LB -----------------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(LCfg<N>::CBL* LCfg<N>::TN, live_min_blocks(LCfg<N>::CBL* LCfg<N>::TN))
    k_live_b(const JobDesc* __restrict__ jobs) {
  using P = LCfg<N>;
  constexpr int T = P::TN, C = P::CBL, E = P::EN;
  const JobDesc& J = jobs[blockIdx.y];
  const int lt = threadIdx.x, lane = lt % C, t = lt / C;
  const int x = blockIdx.x * C + lane;
  __shared__ float2 s[smem_line_elems(N, C)];
  const float2* tw = g_stw + stw_offset(N, E);  // stage twiddles through L1
  const size_t frame = (size_t)N * N;
  for (int a = 0; a < J.nA; a++)
    for (int c = 0; c < J.nC; c++) {
      float2* X = J.I + (size_t)(a * J.nC + c) * frame;
      float2 v[E];  // element t + i*T of this lane's column, in registers through the transforms
#pragma unroll
      for (int i = 0; i < E; i++) v[i] = X[(size_t)(t + i * T) * N + x];
      line_fft_reg<N, T, C, false>(v, s, lane, t, tw);
      // times conj(OTF): the OTF vector is real (estimate), conj(OTF)*v = (v.re*o, v.im*o)
#pragma unroll
      for (int i = 0; i < E; i++) {
        const float o = __ldg(&J.masks[(size_t)(t + i * T) * N + x]);
        v[i] = make_float2(__fmul_rn(v[i].x, o), __fmul_rn(v[i].y, o));
      }
      if (c > 0) {
        line_fft_reg<N, T, C, true>(v, s, lane, t, tw);
        const float2* ry = J.ramps + (size_t)(a * J.nC + c) * 2 * N + N;
#pragma unroll
        for (int i = 0; i < E; i++) v[i] = cmul(v[i], __ldg(&ry[t + i * T]));
        line_fft_reg<N, T, C, false>(v, s, lane, t, tw);
      }
#pragma unroll
      for (int i = 0; i < E; i++) X[(size_t)(t + i * T) * N + x] = v[i];
    }
}

// ---- LC -----------------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(LCfg<N>::TW, live_min_blocks(LCfg<N>::TW)) k_live_c(const JobDesc* __restrict__ jobs) {
  using P = LCfg<N>;
  constexpr int W = P::W, TW = P::TW, EW = P::EW, EN = N / TW;
  const JobDesc& J = jobs[blockIdx.y];
  const int Y = blockIdx.x, t = threadIdx.x;
  // Stage twiddles are read through L1 (g_stw), as in the offline passes: per-block copies in
  // shared memory held the pass to 16 warps per SM. Row values outside the transforms (the
  // paste read-out, the sum) use the unpadded index: a half-warp's 16 consecutive float2 then
  // fall into distinct bank pairs from any starting element.
  __shared__ float2 acc[smem_line_elems(W, 1)];
  __shared__ float2 s[smem_line_elems(N, 1)];
  const float2* twN = g_stw + stw_offset(N, EN);
  const float2* twW = g_stw + stw_offset(W, EW);
#pragma unroll
  for (int i = 0; i < EW; i++) acc[t + i * TW] = make_float2(0.f, 0.f);
  const size_t frame = (size_t)N * N;
  for (int a = 0; a < J.nA; a++)
    for (int c = 0; c < J.nC; c++) {
      const int xInt = J.win[2 * (a * J.nC + c)], yInt = J.win[2 * (a * J.nC + c) + 1];
      const int ys = paste_source(Y, yInt, N, W);
      if (ys < 0) continue;  // uniform per block
      const float2* X = J.I + (size_t)(a * J.nC + c) * frame + (size_t)ys * N;
      float2 v[EN];  // element t + i*TW of the row, in registers through the transforms
#pragma unroll
      for (int i = 0; i < EN; i++) v[i] = X[t + i * TW];
      __syncthreads();  // the previous paste has read s
      if (c > 0) {
        line_fft_reg<N, TW, 1, true>(v, s, 0, t, twN);
        const float2* rx = J.ramps + (size_t)(a * J.nC + c) * 2 * N;
#pragma unroll
        for (int i = 0; i < EN; i++) v[i] = cmul(v[i], __ldg(&rx[t + i * TW]));
        line_fft_reg<N, TW, 1, false>(v, s, 0, t, twN);
      }
#pragma unroll
      for (int i = 0; i < EN; i++) s[t + i * TW] = v[i];
      __syncthreads();
      // pasteFreq at (xInt, yInt) and fullResult.add
#pragma unroll
      for (int i = 0; i < EW; i++) {
        const int Xo = t + i * TW;
        const int xs = paste_source(Xo, xInt, N, W);
        if (xs >= 0) {
          float2& o = acc[Xo];
          const float2 v = s[xs];
          o = make_float2(__fadd_rn(o.x, v.x), __fadd_rn(o.y, v.y));
        }
      }
      __syncthreads();
    }
  const float* wa = J.wa + (size_t)Y * W;
  float2 u[EW];
#pragma unroll
  for (int i = 0; i < EW; i++) {
    const int k = t + i * TW;
    const float f = __ldg(&wa[k]);
    const float2 o = acc[k];
    u[i] = make_float2(o.x * f, o.y * f);
  }
  __syncthreads();  // acc is read: it becomes the transform's scratch
  line_fft_reg<W, TW, 1, true>(u, acc, 0, t, twW);
  float2* O = J.O + (size_t)Y * W;
#pragma unroll
  for (int i = 0; i < EW; i++) O[t + i * TW] = u[i];
}

// ---- LD -----------------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(LCfg<N>::CD* LCfg<N>::TW) k_live_d(const JobDesc* __restrict__ jobs) {
  using P = LCfg<N>;
  constexpr int W = P::W, TW = P::TW, EW = P::EW, C = P::CD;
  const JobDesc& J = jobs[blockIdx.y];
  const int lt = threadIdx.x, lane = lt % C, t = lt / C;
  const int X = blockIdx.x * C + lane;
  extern __shared__ float2 s[];
  const float2* tw = g_stw + stw_offset(W, EW);  // stage twiddles through L1
  float2 v[EW];  // element t + i*TW of the column, in registers through the transform
#pragma unroll
  for (int i = 0; i < EW; i++) v[i] = J.O[(size_t)(t + i * TW) * W + X];
  line_fft_reg<W, TW, C, true>(v, s, lane, t, tw);
  const float scale = 1.f / ((float)W * (float)W);
#pragma unroll
  for (int i = 0; i < EW; i++) J.out[(size_t)(t + i * TW) * W + X] = v[i].x * scale;
}

// ---- plan tables ----------------------------------------------------------------------------
__global__ void k_live_otf(float* __restrict__ v, int N, const OtfTable* __restrict__ t, int att) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= N) return;
  float2 o = make_float2(0.f, 0.f);
  if (!otf_at_fast(*t, 0, freq_x(x, N), freq_y(y, N), FShift{0.f, 0.f, 0.f, 0.f}, 0, 0, att != 0, &o)) o.x = 0.f;
  v[(size_t)y * N + x] = o.x;
}
// getDenominator x writeApoVector (the apodization from its octant table, W/2 + 1 per row)
__global__ void k_live_wa(float* __restrict__ wa, int W, const OtfTable* __restrict__ t, ShiftSet shifts, FShiftSet fsh,
                          int use_att, float wp, const float* __restrict__ apo) {
  const int X = blockIdx.x * blockDim.x + threadIdx.x, Y = blockIdx.y;
  if (X >= W) return;
  const int xh = freq_x(X, W), yh = freq_y(Y, W);
  float acc = 0.f;
  for (int d = 0; d < shifts.n_dirs; d++)
    for (int b = 0; b < shifts.n_bands; b++) {
      const double kx = shifts.px[d] * b, ky = shifts.py[d] * b;
      const FShift k = fsh.k[d][b];
      const float v1 = wiener_term(*t, 0, xh, yh, k, kx, ky, use_att != 0);
      const float v2 = wiener_term(*t, 0, xh, yh, fshift_neg(k), -kx, -ky, use_att != 0);
      acc = __fadd_rn(__fadd_rn(acc, v1), v2);
    }
  const float den = __fdiv_rn(1.f, __fadd_rn(acc, wp));
  const int ax = abs(xh), ay = abs(yh);
  wa[(size_t)Y * W + X] = __fmul_rn(den, __ldg(apo + (size_t)max(ax, ay) * (W / 2 + 1) + min(ax, ay)));
}

int Plan::build_live(cudaStream_t st) {
  const int N = prm.w, W = 2 * N, nA = prm.nr_dirs, nP = prm.nr_phases, nC = 2 * prm.nr_bands - 1;
  OtfTable ht;
  build_otf_table(&prm, &ht);
  nwin = 0;
  std::vector<float2> coef((size_t)nA * nC * nP);
  for (int a = 0; a < nA; a++) {
    auto m = separation_coeffs(&prm, a, false);
    for (int c = 0; c < nC; c++)
      for (int q = 0; q < nP; q++) coef[(a * nC + c) * nP + q] = make_float2(m[c * nP + q].real(), m[c * nP + q].imag());
  }
  std::vector<float2> ramps((size_t)nA * nC * 2 * N);
  std::vector<int> off((size_t)nA * nC * 2, 0);
  for (int a = 0; a < nA; a++)
    for (int c = 1; c < nC; c++) {
      const int b = (c + 1) / 2;
      const double sg = (c % 2 == 0) ? 1.0 : -1.0;  // pos = 2b, neg = 2b-1
      const double kx = sg * band_px(&prm, a, b), ky = sg * band_py(&prm, a, b);
      // SimUtils.pasteAndFourierShift, fast mode (S/SimUtils.java:77-86)
      const double xFrac = kx - std::floor(kx), yFrac = -ky - std::floor(-ky);
      off[2 * (a * nC + c)] = (int)std::floor(kx);
      off[2 * (a * nC + c) + 1] = (int)std::floor(-ky);
      float2* rx = &ramps[(size_t)(a * nC + c) * 2 * N];
      float2* ry = rx + N;
      for (int n = 0; n < N; n++) {
        double fx = xFrac * n / N, fy = yFrac * n / N;
        fx -= std::floor(fx);
        fy -= std::floor(fy);
        rx[n] = make_float2((float)(std::cos(2 * M_PI * fx) / N), (float)(std::sin(2 * M_PI * fx) / N));
        ry[n] = make_float2((float)(std::cos(2 * M_PI * fy) / N), (float)(std::sin(2 * M_PI * fy) / N));
      }
    }
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t o_coef = 0, o_ramp = o_coef + al(coef.size() * sizeof(float2));
  size_t o_off = o_ramp + al(ramps.size() * sizeof(float2));
  size_t o_otf = o_off + al(off.size() * sizeof(int));
  size_t o_damp = o_otf + al(sizeof(OtfTable));
  size_t o_mask = o_damp + al((size_t)N * N * sizeof(float));
  size_t o_wa = o_mask + al((size_t)N * N * sizeof(float));
  size_t o_apo = o_wa + al((size_t)W * W * sizeof(float));
  size_t total = o_apo + al((size_t)(N + 1) * (N + 1) * sizeof(float));
  if (total > dev_bytes) {
    if (dev) cudaFree(dev);
    dev = nullptr;
    FSIM_CUDA(fsim::dev_alloc(&dev, total));
    dev_bytes = total;
  }
  char* b = (char*)dev;
  d_coef = (float2*)(b + o_coef);
  d_ramps = (float2*)(b + o_ramp);
  d_win = (int*)(b + o_off);
  d_otf = (OtfTable*)(b + o_otf);
  d_damp = fade_px > 0 ? (float*)(b + o_damp) : nullptr;
  d_masks = (float*)(b + o_mask);
  d_wa = (float*)(b + o_wa);
  FSIM_CUDA(cudaMemcpyAsync(d_coef, coef.data(), coef.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_ramps, ramps.data(), ramps.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_win, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_otf, &ht, sizeof(OtfTable), cudaMemcpyHostToDevice, st));
  std::vector<float> dv;
  if (d_damp) {
    dv = fade_vector(N, N, fade_px);
    FSIM_CUDA(cudaMemcpyAsync(d_damp, dv.data(), dv.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  }
  FSIM_CUDA(cudaStreamSynchronize(st));
  k_live_otf<<<dim3(div_up(N, 128), N), 128, 0, st>>>(d_masks, N, d_otf, prm.use_attenuation);
  // setupFilters: getDenominator(wienParam) and writeApoVector(apo, 1, 2)
  {
    float* d_apo = (float*)(b + o_apo);
    int rc = apo_octant_device(d_apo, N, ht.vec_cpm, ht.cutoff * 2.0, 1.0, st);
    if (rc) return rc;
    const ShiftSet sh = shift_set(&prm);
    k_live_wa<<<dim3(div_up(W, 128), W), 128, 0, st>>>(d_wa, W, d_otf, sh, fshift_set(sh), prm.use_attenuation,
                                                       (float)(prm.wiener * prm.wiener), d_apo);
  }
  FSIM_CHECK_LAUNCH();
  FSIM_CUDA(cudaStreamSynchronize(st));
  filter_bytes = total;
  return FSIM_OK;
}

size_t Plan::workspace_bytes_live() const {
  const int N = prm.w, W = 2 * N, nC = 2 * prm.nr_bands - 1;
  size_t I = (size_t)prm.nr_dirs * nC * N * N * sizeof(float2);
  size_t O = (size_t)W * W * sizeof(float2);
  return ((I + 255) & ~(size_t)255) + ((O + 255) & ~(size_t)255);
}

void Plan::fill_job_live(JobDesc& j, const void* raw, float* out, float* wf, char* ws) const {
  const int N = prm.w, nC = 2 * prm.nr_bands - 1;
  j.raw = raw;
  j.out = out;
  j.widefield = wf;
  j.input_u16 = input_type == FSIM_INPUT_U16;
  j.nA = prm.nr_dirs;
  j.nP = prm.nr_phases;
  j.nC = nC;
  j.status = ctx().status;
  j.nWin = 0;
  j.bgr = 0.f;
  j.damp = d_damp;
  j.coef = d_coef;
  j.ramps = d_ramps;
  j.win = d_win;
  j.masks = d_masks;
  j.wa = d_wa;
  j.nyq = nullptr;
  j.D = nullptr;
  j.G = nullptr;
  j.Tw = nullptr;
  j.Dy = nullptr;
  j.On = nullptr;
  j.clip_max = nullptr;
  j.clip = 0;
  j.cmask = 0;
  j.fwf = nullptr;
  j.wff = nullptr;
  j.Wf = nullptr;
  size_t I = (size_t)prm.nr_dirs * nC * N * N * sizeof(float2);
  j.I = (float2*)ws;
  j.O = (float2*)(ws + ((I + 255) & ~(size_t)255));
}

template <int N>
static int launch_live(const JobDesc* d_jobs, int njobs, int maxA, cudaStream_t st) {
  using P = LCfg<N>;
  constexpr int W = P::W;
  (void)maxA;
  const size_t smem_d = sizeof(float2) * smem_line_elems(W, P::CD);
  static bool attr = false;
  if (!attr) {
    FSIM_CUDA(cudaFuncSetAttribute(k_live_d<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_d));
    attr = true;
  }
  cudaEvent_t* ev = profile_events();
  if (ev) cudaEventRecord(ev[0], st);
  k_live_a<N><<<dim3(N / P::GA, njobs), P::GA * P::TN, 0, st>>>(d_jobs);
  if (ev) cudaEventRecord(ev[1], st);
  k_live_b<N><<<dim3(N / P::CBL, njobs), P::CBL * P::TN, 0, st>>>(d_jobs);
  if (ev) cudaEventRecord(ev[2], st);
  k_live_c<N><<<dim3(W, njobs), P::TW, 0, st>>>(d_jobs);
  if (ev) cudaEventRecord(ev[3], st);
  k_live_d<N><<<dim3(W / P::CD, njobs), P::CD * P::TW, smem_d, st>>>(d_jobs);
  if (ev) {
    cudaEventRecord(ev[4], st);
    profile_mark(4);
  }
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

#define FSIM_LIVE_SIZES(X) X(64) X(128) X(256) X(384) X(512) X(768) X(1024) X(2048)

bool live_size_supported(int n) {
  switch (n) {
#define CASE(v) case v:
    FSIM_LIVE_SIZES(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}

int launch_live_size(int n, const JobDesc* d_jobs, int njobs, int maxA, cudaStream_t st) {
  switch (n) {
#define CASE(v) \
  case v:       \
    return launch_live<v>(d_jobs, njobs, maxA, st);
    FSIM_LIVE_SIZES(CASE)
#undef CASE
  }
  set_error("live reconstruction: unsupported image size %d", n);
  return FSIM_EINVAL;
}

}  // namespace fsim
