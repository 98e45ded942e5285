// Kernels of the fused offline reconstruction (templates instantiated per size in
// recon_inst_*.cu). See recon.cu for the algorithm and the pass structure.
//
// Every 1D operation here is done with N-length line FFTs. The reference's shift of a
// pasted N-point spectrum Z on the W = 2N grid, FFT_W(r * iFFT_W(paste(Z))), is evaluated
// through its exact even/odd split: with u = iFFT_W(paste(Z)),
//   u[2n]   = z[n] / 2                       (z = iFFT_N(Z), the line in real space)
//   u[2n+1] = iFFT_N(Z * s)[n] / W,  s(m) = exp(+i pi m~/N), m~ the pasted signed frequency
// so that, with E = FFT_N(r[2n] u[2n]) and O = FFT_N(r[2n+1] u[2n+1]),
//   FFT_W(r * u)[X] = E[X mod N] + exp(-2 pi i X/W) O[X mod N].
// The per-component ramps r (even and odd samples, 1/2 and 1/W folded in) are resident
// tables; s and exp(-2 pi i X/W) come from the W-point twiddle table. The final inverse
// FFT_W along y is folded the same way into two N-point inverse FFTs (even/odd rows).
#pragma once

#include "bulk.cuh"
#include "common.cuh"
#include "fft_line.cuh"
#include "filters.cuh"
#include "otf.cuh"
#include "recon.cuh"

// Register budgets (registers per thread) of passes A, B1 and B2 at 8 elements per thread.
#ifndef FSIM_PA_REGS
#define FSIM_PA_REGS 64
#endif
#ifndef FSIM_B1_REGS
#define FSIM_B1_REGS 64
#endif
#ifndef FSIM_B2_REGS
#define FSIM_B2_REGS 64
#endif

namespace fsim {

// ---- launch configuration (variants picked per size by the autotuner) --------------------
// ENV: elements per thread of the N-length lines (radix plan and threads per line follow);
// CBV: interleaved columns per block in pass B.
template <int N, int ENV = 0, int CBV = 0>
struct Cfg {
  static constexpr int W = 2 * N;
  static constexpr int EN = ENV ? ENV : ((N % 3 == 0) ? 12 : 8);
  static constexpr int T = N / EN;  // threads per line
  static constexpr int CB = CBV ? CBV : 4;  // passes B1, B2: interleaved columns per block
  static constexpr int GC = (T >= 128) ? 1 : (128 / T);  // pass C: rows per block
};

// Copies a job descriptor into shared memory once per block (the passes read its fields
// after global stores, which would otherwise force reloads).
__device__ __forceinline__ void load_job(JobDesc* dst, const JobDesc* src, int tid, int nthreads) {
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int i = tid; i < (int)(sizeof(JobDesc) / sizeof(int)); i += nthreads) d[i] = s[i];
}

// exp(+i pi m~ / N) for the pasted signed frequency m~ of index m (m < N/2: m, else m - N)
template <int N>
__device__ __forceinline__ float2 half_shift(const float2* twW, int m) {
  const int ms = m < N / 2 ? m : m - N;
  return cconjf(twW[ms < 0 ? ms + 2 * N : ms]);
}
// source index in an N-point spectrum of output index X of pasteFreq onto 2N (or -1)
template <int N>
__device__ __forceinline__ int paste_src(int X) {
  return X < N / 2 ? X : (X >= 3 * N / 2 ? X - N : -1);
}

// ---- pass A: rows ----------------------------------------------------------------------------
// Register budgets (registers per thread; the compiler otherwise keeps 90-230 registers per
// thread in the longer radix plans, which caps occupancy at a few warps per scheduler):
// 64 per thread at up to 8 elements per thread (32 warps per SM), 96 at 12 elements.
template <int T, int EN>
__host__ __device__ constexpr int pass_a_min_blocks() {
  return EN <= 8 ? (65536 / (T * FSIM_PA_REGS) > 0 ? 65536 / (T * FSIM_PA_REGS) : 1)
                 : (EN == 12 ? (65536 / (T * 96) > 0 ? 65536 / (T * 96) : 1) : 1);
}
// The column passes: 64 registers per thread at 8 elements, 80 at 12.
template <int THREADS, int EN, int REGS8 = 64>
__host__ __device__ constexpr int col_min_blocks() {
  return EN <= 8 ? (65536 / (THREADS * REGS8) > 0 ? 65536 / (THREADS * REGS8) : 1)
                 : (EN == 12 ? (65536 / (THREADS * 80) > 0 ? 65536 / (THREADS * 80) : 1) : 1);
}
// Raw pixels fo + row + t + i*T (frame offset fo, row start row) with the background clip
// and the border damping applied: all EN loads of the row are issued before any is used.
template <int EN, int T, bool DAMP = true>
__device__ __forceinline__ void raw_row(const JobDesc& J, size_t fo, size_t row, int t, float (&v)[EN]) {
  if (J.input_u16) {
    const uint16_t* r = (const uint16_t*)J.raw + fo + row + t;
#pragma unroll
    for (int i = 0; i < EN; i++) v[i] = (float)__ldg(r + i * T);
  } else {
    const float* r = (const float*)J.raw + fo + row + t;
#pragma unroll
    for (int i = 0; i < EN; i++) v[i] = __ldg(r + i * T);
  }
  if (J.bgr != 0.f) {
#pragma unroll
    for (int i = 0; i < EN; i++) {
      v[i] = v[i] - J.bgr;
      if (v[i] < 0) v[i] = 0;
    }
  }
  if (DAMP && J.damp) {
    const float* d = J.damp + row + t;
#pragma unroll
    for (int i = 0; i < EN; i++) v[i] = v[i] * __ldg(d + i * T);
  }
}
// The border damping of a mixed row: the mix of damped rows is the damped mix (the damping
// is one real factor per pixel), so the factors are read once per row, not once per frame.
template <int EN, int T>
__device__ __forceinline__ void damp_row(const JobDesc& J, size_t row, int t, float2 (&z)[EN]) {
  if (J.damp) {
    const float* d = J.damp + row + t;
#pragma unroll
    for (int i = 0; i < EN; i++) {
      const float f = __ldg(d + i * T);
      z[i].x *= f;
      z[i].y *= f;
    }
  }
}

// Rows per pass-A block: the rows of a block share the job descriptor and the separation
// coefficients, and write their windows together, so that each quad of the quad layout
// (4 columns x RB rows) is one contiguous run of RB * 32 bytes instead of one 32-byte piece
// per row and quad (global store wavefronts 1.21 M -> 0.55 M per 16 datasets of 512^2 3x3 at
// four rows). Up to 128 threads per block: the rows meet at the block's barriers (the
// transforms' exchanges included), and at 256 threads those waits cost more than the store
// wavefronts save (pass A 0.568 ms per 64 datasets at two rows of 64 threads, 0.572 at one,
// 0.599 at four; 0.582 at four with one named barrier per row, which also holds the block to
// four per SM). The row buffers are RS float2 apart, RS = 4 (mod 16) for RB >= 4 and
// 8 (mod 16) for RB = 2, so that a half-warp of the read-out (RB >= 4: four rows x four
// columns; RB = 2: two rows x two quads) reads 16 distinct bank pairs.
__host__ __device__ constexpr int pass_a_row_stride(int N, int RB) {
  const int s = smem_line_elems(N, 1), m = RB >= 4 ? 4 : 8;
  return s + ((m - s % 16) % 16 + 16) % 16;
}
__host__ __device__ constexpr int pass_a_rows(int N, int T) {
  int rb = 1;
  while (2 * rb * T <= 128 && N % (2 * rb) == 0 && 2 * (2 * rb) * pass_a_row_stride(N, 2 * rb) * 8 <= 44 * 1024)
    rb *= 2;
  return rb;
}
template <int N, int ENV>
struct PassA {
  static constexpr int T = Cfg<N, ENV>::T;
  static constexpr int RB = pass_a_rows(N, T);
  static constexpr int RS = pass_a_row_stride(N, RB);
  static constexpr int NT = RB * T;  // threads per block
  static_assert(RS >= smem_line_elems(N, 1) && (RB == 1 || RS % 16 == (RB >= 4 ? 4 : 8)),
                "row buffers: a transform's scratch, read-out half-warps on distinct bank pairs");
};

template <int N, int ENV>
__global__ void __launch_bounds__(PassA<N, ENV>::NT, pass_a_min_blocks<PassA<N, ENV>::NT, Cfg<N, ENV>::EN>())
    k_pass_a(const JobDesc* __restrict__ jobs) {
  using P = Cfg<N, ENV>;
  using PA = PassA<N, ENV>;
  constexpr int W = P::W, T = P::T, EN = P::EN, RB = PA::RB, RS = PA::RS, NT = PA::NT;
  const int tid = threadIdx.x, g = tid / T, t = tid % T;
  const int y0 = blockIdx.x * RB, y = y0 + g, a = blockIdx.y;
  __shared__ JobDesc J;
  __shared__ float2 sbz[RB * RS], sbh[RB * RS];
  __shared__ float2 coef[FSIM_MAX_DIRS * FSIM_MAX_PHASES];
  float2* bz = sbz + g * RS;  // this row group's buffers
  float2* bh = sbh + g * RS;
  const float2* twN = g_stw + stw_offset(N, EN);  // stage table, read through L1
  const float2* twW = g_tw + tw_offset(W);
  const JobDesc* jg = jobs + blockIdx.z;
  load_job(&J, jg, tid, NT);
  // the counts and the separation coefficients straight from the descriptor in global
  // memory, so that one barrier covers both shared-memory copies
  const int nA = jg->nA, nP = jg->nP, nC = jg->nC, nPair = (nC - 1) / 2;
  if (a > nA || (a < nA && nPair == 0)) return;  // uniform per block; one band: band 0 only
  if (a == nA) {
    for (int i = tid; i < nA * nP; i += NT) coef[i] = jg->coef[((i / nP) * nC) * nP + i % nP];
  } else {
    for (int i = tid; i < nC * nP; i += NT) coef[i] = jg->coef[a * nC * nP + i];
  }
  __syncthreads();
  const size_t frame = (size_t)N * N, row = (size_t)y * N;
  // Window read-out of the block's RB rows: element idx = (quad q, row r, column j) with
  // (r, j) fastest, stored at ((q * N + y0) * 4 + 4 r + j) of the quad layout.
  auto window_pos = [&](int idx, int& q, int& r, int& xl) {
    q = idx / (4 * RB);
    const int rem = idx - q * 4 * RB;
    r = rem >> 2;
    xl = 4 * q + (rem & 3);
    return ((size_t)q * N + y0) * 4 + rem;
  };
  if (a == nA) {
    // Band 0 is summed over the angles before the column pass, and its band separation
    // and row FFT are linear: one row group per row mixes the band-0 rows of every angle and
    // transforms the sum once into slot 0 (band 0 has no shift: one window for all angles).
    const int nF = nA * nP;
    float2 x[EN];
#pragma unroll
    for (int i = 0; i < EN; i++) x[i] = make_float2(0.f, 0.f);
#pragma unroll 3
    for (int f = 0; f < nF; f++) {
      float v[EN];
      raw_row<EN, T, false>(J, f * frame, row, t, v);
      const float2 c = coef[f];
#pragma unroll
      for (int i = 0; i < EN; i++) {
        x[i].x += c.x * v[i];
        x[i].y += c.y * v[i];
      }
    }
    damp_row<EN, T>(J, row, t, x);
    line_fft_reg<N, T, 1, false>(x, bh, 0, t, twN);
#pragma unroll
    for (int i = 0; i < EN; i++) bh[t + i * T] = x[i];
    __syncthreads();  // the read-out reads every row group's buffer
    const int Xs = J.win[0];
    for (int idx = tid; idx < J.nWin * RB; idx += NT) {
      int q, r, xl;
      const size_t o = window_pos(idx, q, r, xl);
      int X = Xs + xl;
      if (X >= W) X -= W;
      const int m = paste_src<N>(X);
      J.I[o] = m >= 0 ? sbh[r * RS + m] : make_float2(0.f, 0.f);
    }
    if (y0 == 0 && tid == 0) *J.clip_max = 0.f;  // CLIPSCALE.BOTH: pass C takes the maximum from 0
    return;
  }
  // band separation in real space of component cm for this thread's elements t + i*T: the
  // phases outer, so that every element's load of a phase row is in flight at once (pass A
  // 0.61 ms per 64 datasets of 512^2 3x3, 0.94 ms with the elements outer and one load in
  // flight; 0.63 ms with three phase rows per round, which spills)
  auto mix = [&](int cm, float2 (&z)[EN]) {
#pragma unroll
    for (int i = 0; i < EN; i++) z[i] = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int p = 0; p < nP; p++) {
      float v[EN];
      raw_row<EN, T, false>(J, (size_t)(a * nP + p) * frame, row, t, v);
      const float2 m = coef[cm * nP + p];
#pragma unroll
      for (int i = 0; i < EN; i++) {
        z[i].x += m.x * v[i];
        z[i].y += m.y * v[i];
      }
    }
    damp_row<EN, T>(J, row, t, z);
  };
  // Row values outside the transforms (the stashed mixed row, transform outputs, window
  // read-out) use the unpadded index: 16 consecutive float2 of a half-warp then fall into
  // distinct bank pairs from any starting element, where the padded layout of the transforms'
  // exchanges splits a run that crosses a 16-element boundary (2-way conflicts on the window
  // read-out).
  // Components: band 0, then per band b the pair neg = 2b-1, pos = 2b. The separation
  // coefficients of a pair are complex conjugates, so z_pos = conj(z_neg): the pos
  // component's row transform follows from the neg one's (below). A line stays in
  // registers from one transform to the next (x[i] = element t + i*T), bz and bh serve as
  // scratch.
  // the band pairs of this block's angle (band 0 of every angle is the blockIdx.y == nA block's)
  float2 x[EN];
  // pair (neg, pos): only the neg component is transformed and stored. With
  // z_pos = conj(z_neg) and opposite shifts (ro_pos = conj(ro_neg), re_pos = conj(re_neg)):
  //   E_pos[m] = conj(E_neg[-m]),
  //   O_pos[m] = conj(O_neg[-m]) + d * Q[m],  d = -2i conj(Z_neg[N/2]),
  // where the d term is the pasted Nyquist bin, whose half-sample phase s(N/2) = -i is
  // not conjugate-symmetric, and Q = FFT_N((-1)^n ro_pos[n]) is a plan table. So the pos
  // row spectrum is conj(F_neg[-X]) + exp(-2 pi i X/W) Q[X mod N] d: the column pass
  // forms it from the neg windows (mirror images of the pos windows) and d, kept here.
  for (int b = 1; b <= nPair; b++) {
    const int cn = 2 * b - 1;
    mix(cn, x);
    if (b > 1) __syncthreads();  // the previous pair's read-out of every row group's buffers is done
    // the mixed row waits in bz (each thread its own elements) for the even-sample product
    // below, instead of in 16 registers across the three transforms of the odd samples
#pragma unroll
    for (int i = 0; i < EN; i++) bz[t + i * T] = x[i];
    line_fft_reg<N, T, 1, false>(x, bh, 0, t, twN);  // Z = FFT_N(z)
    if (t == (N / 2) % T) {
      const float2 zn = x[(N / 2) / T];
      J.D[(size_t)(a * nPair + (b - 1)) * N + y] = make_float2(-2.f * zn.y, -2.f * zn.x);
    }
    const float2* re = J.ramps + (size_t)(a * nC + cn) * 2 * W;
    const float2* ro = re + N;
    // odd samples of the upsampled line, iFFT_N(Z * s), times the odd-sample ramp, FFT: O
#pragma unroll
    for (int i = 0; i < EN; i++) x[i] = cmul(x[i], half_shift<N>(twW, t + i * T));
    line_fft_reg<N, T, 1, true>(x, bh, 0, t, twN);
#pragma unroll
    for (int i = 0; i < EN; i++) x[i] = cmul(x[i], __ldg(ro + t + i * T));
    line_fft_reg<N, T, 1, false>(x, bh, 0, t, twN);
#pragma unroll
    for (int i = 0; i < EN; i++) bh[t + i * T] = x[i];
    // even samples times the even-sample ramp, FFT: E
#pragma unroll
    for (int i = 0; i < EN; i++) x[i] = cmul(bz[t + i * T], __ldg(re + t + i * T));
    __syncthreads();  // every thread has its elements back before the transform reuses bz
    line_fft_reg<N, T, 1, false>(x, bz, 0, t, twN);
#pragma unroll
    for (int i = 0; i < EN; i++) bz[t + i * T] = x[i];
    __syncthreads();  // the read-out reads every row group's buffers
    // neg window of the shifted spectrum: E[X mod N] + exp(-2 pi i X/W) O[X mod N]
    const int Xs = J.win[2 * (a * nC + cn)];
    float2* I = J.I + (size_t)(1 + a * nPair + (b - 1)) * J.nWin * N;  // slot of (a, b)
    for (int idx = tid; idx < J.nWin * RB; idx += NT) {
      int q, r, xl;
      const size_t o = window_pos(idx, q, r, xl);
      int X = Xs + xl;
      if (X >= W) X -= W;
      const int m = X < N ? X : X - N;
      I[o] = cadd(sbz[r * RS + m], cmul(twW[X], sbh[r * RS + m]));
    }
  }
}

// ---- pass G: the pos components' Nyquist columns ----------------------------------------------
// The pos row spectrum of a pair differs from the mirrored neg one by exp(-2 pi i X/W) Qx[X]
// times d(y) (pass A). Along y that column d is transformed once per angle and pair with the
// pos component's y shift; pass B adds it scaled by exp(-2 pi i X/W) Qx[X mod N].
template <int N, int ENV>
__global__ void __launch_bounds__(Cfg<N, ENV>::T) k_pass_g(const JobDesc* __restrict__ jobs) {
  using P = Cfg<N, ENV>;
  constexpr int W = P::W, T = P::T, EN = P::EN;
  const int t = threadIdx.x, ab = blockIdx.x;
  __shared__ JobDesc J;
  __shared__ float2 bz[smem_line_elems(N, 1)], bh[smem_line_elems(N, 1)];
  const float2* twN = g_stw + stw_offset(N, EN);
  const float2* twW = g_tw + tw_offset(W);
  load_job(&J, jobs + blockIdx.y, t, T);
  __syncthreads();
  const int nC = J.nC, nPair = (nC - 1) / 2;
  if (ab >= J.nA * nPair) return;  // uniform per block
  const int a = ab / nPair, cp = 2 * (1 + ab % nPair);
  const float2* d = J.D + (size_t)ab * N;
#pragma unroll
  for (int i = 0; i < EN; i++) {
    const int k = t + i * T;
    const float2 v = d[k];
    bz[sidx(k)] = v;
    bh[sidx(k)] = v;
  }
  __syncthreads();
  line_fft_st<N, T, 1, false>(bh, t, twN);
#pragma unroll
  for (int i = 0; i < EN; i++) {
    const int m = t + i * T;
    bh[sidx(m)] = cmul(bh[sidx(m)], half_shift<N>(twW, m));
  }
  __syncthreads();
  line_fft_st<N, T, 1, true>(bh, t, twN);
  const float2* re = J.ramps + (size_t)(a * nC + cp) * 2 * W + W;  // y ramps
  const float2* ro = re + N;
#pragma unroll
  for (int i = 0; i < EN; i++) {
    const int m = t + i * T;
    bz[sidx(m)] = cmul(bz[sidx(m)], __ldg(re + m));
    bh[sidx(m)] = cmul(bh[sidx(m)], __ldg(ro + m));
  }
  __syncthreads();
  line_fft_st<N, T, 1, false>(bz, t, twN);
  line_fft_st<N, T, 1, false>(bh, t, twN);
  const int Ys = J.win[2 * (a * nC + cp) + 1];
  for (int yl = t; yl < J.nWin; yl += T) {
    int Y = Ys + yl;
    if (Y >= W) Y -= W;
    const int m = Y < N ? Y : Y - N;
    J.G[(size_t)ab * J.nWin + yl] = cadd(bz[sidx(m)], cmul(twW[Y], bh[sidx(m)]));
  }
}

// ---- pass B1: column transforms of band 0 and of the neg components ----------------------------
// One block per CB window columns of one component: band 0 (the windows of all angles summed:
// they share one unshifted mask) is transformed along y and pasted; each pair's neg
// component gets the full y shift (even/odd split). The results over the component's
// row window go to Tw in quad layout; for neg columns also d' = -2i conj(Z[N/2]).
template <int N, int ENV, int CBV>
__global__ void __launch_bounds__(Cfg<N, ENV, CBV>::CB* Cfg<N, ENV, CBV>::T,
                                  col_min_blocks<Cfg<N, ENV, CBV>::CB * Cfg<N, ENV, CBV>::T, Cfg<N, ENV, CBV>::EN,
                                                 FSIM_B1_REGS>())
    k_pass_b1(const JobDesc* __restrict__ jobs) {
  using P = Cfg<N, ENV, CBV>;
  constexpr int W = P::W, T = P::T, CB = P::CB, EN = P::EN;
  const int lt = threadIdx.x, lane = lt % CB, t = lt / CB;
  __shared__ JobDesc J;
  extern __shared__ float2 sm[];
  float2* bz = sm;                           // N x CB
  float2* bh = bz + smem_line_elems(N, CB);  // N x CB
  const float2* twN = g_stw + stw_offset(N, EN);
  const float2* twW = g_tw + tw_offset(W);
  load_job(&J, jobs + blockIdx.z, lt, CB * T);
  __syncthreads();
  const int nC = J.nC, nWin = J.nWin, nPair = (nC - 1) / 2;
  const int comp = blockIdx.y;  // 0: band 0; 1 + a*nPair + (b-1): neg of (a, b)
  if (comp > J.nA * nPair || (int)blockIdx.x * CB >= nWin) return;  // uniform per block
  const int xl = blockIdx.x * CB + lane;  // nWin is a multiple of 4: every lane is inside
  const size_t quad = ((size_t)(xl >> 2) * N) * 4 + (xl & 3);
  float2* out = J.Tw + (size_t)comp * nWin * nWin + ((size_t)(xl >> 2) * nWin) * 4 + (xl & 3);
  float2 x[EN];  // element t + i*T of this lane's column, in registers through the transforms
  if (comp == 0) {  // band 0: summed over the angles and row-transformed in pass A (slot 0)
#pragma unroll
    for (int i = 0; i < EN; i++) x[i] = J.I[quad + (size_t)(t + i * T) * 4];
    line_fft_reg<N, T, CB, false>(x, bh, lane, t, twN);
#pragma unroll
    for (int i = 0; i < EN; i++) bh[sidx_t<true>((t + i * T) * CB + lane)] = x[i];
    __syncthreads();
    const int Ys = J.win[1];
    for (int yl = t; yl < nWin; yl += T) {
      int Y = Ys + yl;
      if (Y >= W) Y -= W;
      const int m = paste_src<N>(Y);
      out[(size_t)yl * 4] = m >= 0 ? bh[sidx_t<true>(m * CB + lane)] : make_float2(0.f, 0.f);
    }
    return;
  }
  const int a = (comp - 1) / nPair, b = 1 + (comp - 1) % nPair, cn = 2 * b - 1;
  const float2* I = J.I + (size_t)comp * nWin * N + quad;  // slot 1 + a*nPair + (b-1)
#pragma unroll
  for (int i = 0; i < EN; i++) x[i] = I[(size_t)(t + i * T) * 4];
  line_fft_reg<N, T, CB, false>(x, bh, lane, t, twN);  // Z along y
  if (t == (N / 2) % T) {
    const float2 z = x[(N / 2) / T];
    J.Dy[(size_t)(comp - 1) * nWin + xl] = make_float2(-2.f * z.y, -2.f * z.x);
  }
  const float2* re = J.ramps + (size_t)(a * nC + cn) * 2 * W + W;  // y ramps
  const float2* ro = re + N;
  // odd samples, iFFT_N(Z * s), times the odd-sample ramp, FFT: O
#pragma unroll
  for (int i = 0; i < EN; i++) x[i] = cmul(x[i], half_shift<N>(twW, t + i * T));
  line_fft_reg<N, T, CB, true>(x, bh, lane, t, twN);
#pragma unroll
  for (int i = 0; i < EN; i++) x[i] = cmul(x[i], __ldg(ro + t + i * T));
  line_fft_reg<N, T, CB, false>(x, bh, lane, t, twN);
#pragma unroll
  for (int i = 0; i < EN; i++) bh[sidx_t<true>((t + i * T) * CB + lane)] = x[i];
  // even samples (the column again, from L2) times the even-sample ramp, FFT: E
#pragma unroll
  for (int i = 0; i < EN; i++) x[i] = cmul(I[(size_t)(t + i * T) * 4], __ldg(re + t + i * T));
  line_fft_reg<N, T, CB, false>(x, bz, lane, t, twN);
#pragma unroll
  for (int i = 0; i < EN; i++) bz[sidx_t<true>((t + i * T) * CB + lane)] = x[i];
  __syncthreads();
  const int Yn = J.win[2 * (a * nC + cn) + 1];
  for (int yl = t; yl < nWin; yl += T) {
    int Y = Yn + yl;
    if (Y >= W) Y -= W;
    const int m = Y < N ? Y : Y - N;
    out[(size_t)yl * 4] = cadd(bz[sidx_t<true>(m * CB + lane)], cmul(twW[Y], bh[sidx_t<true>(m * CB + lane)]));
  }
}

// ---- pass B2: masked Hermitian sum over components, Wiener x apodization, inverse along y ----
// The image is real: out = Re iFFT2(F) = iFFT2(H) with the Hermitian part
// H(X, Y) = (F(X, Y) + conj F(-X, -Y)) / 2, so only the columns X = 0..N of H are formed and
// stored (pass C completes each row by symmetry): half the column-transformed windows,
// masks and Wiener x apodization reads, inverse transforms and writes of a full-width pass.
// CB output columns per block, 2T threads per column: each thread keeps the EN rows
// Y = t + i*2T of its column in registers (twice the threads of a transform, so that twice
// the loads are in flight for the same registers). With the pair identities of pass A (the pos component of a pair at (X, Y) is
// the conjugate of the neg transform at (-X, -Y) plus two rank-one Nyquist terms n1, and
// the neg/pos masks are mirror images: mask_neg(-X,-Y) = mask_pos(X,Y)), a pair adds
//   H += mask_neg(X,Y) (A + conj(n2)/2) + mask_pos(X,Y) (conj(B) + n1/2),
// A = the neg transform at (X, Y), B = the neg transform at (-X, -Y) (stored at the
// mirrored position of the neg window, which is the pos window's mirror image), and
// n1 / n2 the pos component's Nyquist terms at (X, Y) / (-X, -Y):
//   n1(X,Y) = exp(-2 pi i Y/W) d'(-X) Qy[Y mod N] + exp(-2 pi i X/W) Qx[X mod N] G[Y];
// band 0 adds mask_0(X,Y) (T0(X,Y) + conj T0(-X,-Y)) / 2.
// Measured OTFs give complex masks (CM): the masks still depend on |k - shift| only, so the
// mirror relations hold, and a pair adds Re(mask_neg) A + Re(mask_pos) conj(B) +
// (mask_pos n1 + conj(mask_neg n2)) / 2, band 0 (mask_0 T0(X,Y) + conj(mask_0 T0(-X,-Y))) / 2.
// A launch of one kind skips the jobs of the other (uniform per block).
// Loads of pass B2's pair terms: through the read-only path from global memory, or plain
// loads from the shared-memory stage of the bulk-copy variant.
template <bool SM, class V>
__device__ __forceinline__ V b2_ld(const V* p) {
  if constexpr (SM) return *p;
  else return __ldg(p);
}
// Pass B2's accumulation in explicitly rounded operations (fixed FMA forms): the bits do not
// depend on how the compiler contracts the expressions in each kernel that inlines them, so
// the staged and the plain-load variants (chosen per launch) give the same result.
__device__ __forceinline__ float2 b2_cmul(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)), __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float2 b2_cadd(float2 a, float2 b) {
  return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
// Band 0: (T0(X,Y) + conj T0(-X,-Y)) / 2 with one symmetric mask. tv / mk / mkc point at the
// thread's column of the window's column quad (row stride 4), tm at its mirrored column (-X;
// mirror_in false when -X lies outside the window), from global or shared memory (SM).
template <int N, int T2, int EN, bool CM, bool SM>
__device__ __forceinline__ void b2_band0_px(float2 (&acc)[EN], int t, int Ys, int nWin, const float2* tv,
                                            const float2* tm, bool mirror_in, const float* mk, const float2* mkc) {
  constexpr int W = 2 * N;
  auto wrap = [](int v) { return v < 0 ? v + W : (v >= W ? v - W : v); };
#pragma unroll
  for (int i = 0; i < EN; i++) {
    const int Y = t + i * T2;
    const int yl = wrap(Y - Ys), ylm = wrap(wrap(-Y) - Ys);
    if (yl < nWin) {
      const float2 u = b2_ld<SM>(tv + (size_t)yl * 4);
      const float2 um = (mirror_in && ylm < nWin) ? b2_ld<SM>(tm + (size_t)ylm * 4) : make_float2(0.f, 0.f);
      if constexpr (CM) {
        const float2 m = b2_ld<SM>(mkc + (size_t)yl * 4);
        const float2 p = b2_cmul(m, u), q = b2_cmul(m, um);
        acc[i].x = __fmaf_rn(0.5f, __fadd_rn(p.x, q.x), acc[i].x);
        acc[i].y = __fmaf_rn(0.5f, __fsub_rn(p.y, q.y), acc[i].y);
      } else {
        const float f = __fmul_rn(0.5f, b2_ld<SM>(mk + (size_t)yl * 4));
        acc[i].x = __fmaf_rn(f, __fadd_rn(u.x, um.x), acc[i].x);
        acc[i].y = __fmaf_rn(f, __fsub_rn(u.y, um.y), acc[i].y);
      }
    }
  }
}
template <int N, int T2, int EN, bool CM>
__device__ __forceinline__ void b2_band0(const JobDesc& J, float2 (&acc)[EN], int t, int X, int Xm) {
  constexpr int W = 2 * N;
  const int nWin = J.nWin;
  auto wrap = [](int v) { return v < 0 ? v + W : (v >= W ? v - W : v); };
  auto qoff = [&](int xl) { return ((size_t)(xl >> 2) * nWin) * 4 + (xl & 3); };
  const int xl = wrap(X - J.win[0]), xlm = wrap(Xm - J.win[0]);
  if (xl >= nWin) return;
  const bool mirror_in = xlm < nWin;  // (X,Y) in the support puts -X in the window
  b2_band0_px<N, T2, EN, CM, false>(acc, t, J.win[1], nWin, J.Tw + qoff(xl), J.Tw + (mirror_in ? qoff(xlm) : 0),
                                    mirror_in, J.masks + qoff(xl),
                                    reinterpret_cast<const float2*>(J.masks) + qoff(xl));
}
// One component of a band pair. neg (POS false): mask_neg(X,Y) (A + conj(n2)/2), A = the neg
// transform at (X, Y) = tv[yl*4], n2 from G[nWin-1-yl]; pos (POS true): mask_pos(X,Y)
// (conj(B) + n1/2), B = the neg transform at (-X, -Y) = tv[(nWin-1-yl)*4] (the mirrored
// column), n1 from G[yl]. tv / mk / mkc point at the thread's column of a window column quad
// (row stride 4), G at the pair's pos-shift column transform, Qy at its y Nyquist response;
// dd = d' of the neg window column (pos: the mirrored one), cxx = exp(-2 pi i X~/W) Qx[X~ mod N]
// at X~ = -X (neg) or X (pos).
template <int N, int T2, int EN, bool CM, bool POS, bool SM>
__device__ __forceinline__ void b2_pair(float2 (&acc)[EN], int t, int Ys, int nWin, const float2* tv, const float* mk,
                                        const float2* mkc, const float2* G, const float2* Qy, float2 dd, float2 cxx,
                                        const float2* twW) {
  constexpr int W = 2 * N;
  auto wrap = [](int v) { return v < 0 ? v + W : (v >= W ? v - W : v); };
#pragma unroll
  for (int i = 0; i < EN; i++) {
    const int Y = t + i * T2;
    const int yl = wrap(Y - Ys);
    if (yl < nWin) {
      float2 v, n;
      if constexpr (!POS) {
        const int Ym = wrap(-Y);
        v = b2_ld<SM>(tv + (size_t)yl * 4);
        // n2: its pos-window row is nWin-1-yl (the windows are mirror images)
        n = b2_cadd(b2_cmul(twW[Ym], b2_cmul(dd, b2_ld<SM>(Qy + (Ym < N ? Ym : Ym - N)))),
                    b2_cmul(cxx, b2_ld<SM>(G + (nWin - 1 - yl))));
      } else {
        v = b2_ld<SM>(tv + (size_t)(nWin - 1 - yl) * 4);
        n = b2_cadd(b2_cmul(twW[Y], b2_cmul(dd, b2_ld<SM>(Qy + (Y < N ? Y : Y - N)))),
                    b2_cmul(cxx, b2_ld<SM>(G + yl)));
      }
      // neg: A + conj(n2)/2 (times the mask); pos: conj(B) + n1/2
      const float vy = POS ? -v.y : v.y, hy = POS ? 0.5f : -0.5f;
      if constexpr (CM) {
        const float2 m = b2_ld<SM>(mkc + (size_t)yl * 4), q = b2_cmul(m, n);
        acc[i].x = __fadd_rn(acc[i].x, __fmaf_rn(m.x, v.x, __fmul_rn(0.5f, q.x)));
        acc[i].y = __fadd_rn(acc[i].y, __fmaf_rn(m.x, vy, __fmul_rn(hy, q.y)));
      } else {
        const float f = b2_ld<SM>(mk + (size_t)yl * 4);
        acc[i].x = __fmaf_rn(f, __fmaf_rn(0.5f, n.x, v.x), acc[i].x);
        acc[i].y = __fmaf_rn(f, __fmaf_rn(hy, n.y, vy), acc[i].y);
      }
    }
  }
}
// Wiener denominator x apodization, then iFFT_W along y as two N-point inverse FFTs:
//   out[2n] = iFFT_N(A[k] + A[k+N]),  out[2n+1] = iFFT_N((A[k] - A[k+N]) exp(i pi k/N));
// rows k and k + N are acc[i] and acc[i + EN/2] of one thread. The even sequences of the CB
// columns go to bz, the odd ones to bh; threads of the first half then transform the even
// lines and those of the second half the odd ones.
template <int N, int T, int CB, int EN>
__device__ __forceinline__ void b2_finish(const JobDesc& J, float2 (&acc)[EN], float2* bz, float2* bh, int lt, int lane,
                                          int t, int X) {
  constexpr int W = 2 * N, T2 = 2 * T;
  const float2* twN = g_stw + stw_offset(N, EN);
  const float2* twW = g_tw + tw_offset(W);
  {
    const float* wa = J.wa + (size_t)(X >> 2) * W * 4 + (X & 3);
#pragma unroll
    for (int i = 0; i < EN / 2; i++) {
      const int k = t + i * T2;
      const float f0 = __ldg(wa + (size_t)k * 4), f1 = __ldg(wa + (size_t)(k + N) * 4);
      const float2 u0 = make_float2(acc[i].x * f0, acc[i].y * f0);
      const float2 u1 = make_float2(acc[i + EN / 2].x * f1, acc[i + EN / 2].y * f1);
      bz[sidx_t<true>(k * CB + lane)] = cadd(u0, u1);
      bh[sidx_t<true>(k * CB + lane)] = cmul(csub(u0, u1), cconjf(twW[k]));
    }
  }
  __syncthreads();
  const int g = lt / (CB * T), il = lt % CB, it = (lt / CB) % T;
  float2* buf = g ? bh : bz;
  float2 x[EN];  // element it + i*T of line il (even rows for g = 0, odd rows for g = 1)
#pragma unroll
  for (int i = 0; i < EN; i++) x[i] = buf[sidx_t<true>((it + i * T) * CB + il)];
  __syncthreads();  // every thread holds its elements before the transforms reuse the buffers
  line_fft_reg<N, T, CB, true>(x, buf, il, it, twN);
  const int Xo = blockIdx.x * CB + il;
  if (Xo < N) {
#pragma unroll
    for (int i = 0; i < EN; i++) J.O[(size_t)(2 * (it + i * T) + g) * N + Xo] = x[i];
  } else if (Xo == N) {
#pragma unroll
    for (int i = 0; i < EN; i++) J.On[2 * (it + i * T) + g] = x[i];
  }
}

template <int N, int ENV, int CBV, bool CM>
__global__ void __launch_bounds__(2 * Cfg<N, ENV, CBV>::CB* Cfg<N, ENV, CBV>::T,
                                  col_min_blocks<2 * Cfg<N, ENV, CBV>::CB * Cfg<N, ENV, CBV>::T,
                                                 Cfg<N, ENV, CBV>::EN, FSIM_B2_REGS>())
    k_pass_b2(const JobDesc* __restrict__ jobs) {
  using P = Cfg<N, ENV, CBV>;
  constexpr int W = P::W, T = P::T, CB = P::CB, EN = P::EN, T2 = 2 * T;
  static_assert(EN % 2 == 0, "rows k and k + N must share a thread");
  const int lt = threadIdx.x, lane = lt % CB, t = lt / CB;  // t in [0, 2T)
  const int X = blockIdx.x * CB + lane;  // X <= N + CB - 1 < W; only X <= N is stored
  __shared__ JobDesc J;
  extern __shared__ float2 sm[];
  float2* bz = sm;                           // N x CB
  float2* bh = bz + smem_line_elems(N, CB);  // N x CB
  const float2* twW = g_tw + tw_offset(W);
  load_job(&J, jobs + blockIdx.y, lt, CB * T2);
  __syncthreads();
  if ((J.cmask != 0) != CM) return;  // the other launch's job (uniform per block)
  const int nC = J.nC, nWin = J.nWin, nPair = (nC - 1) / 2;
  auto wrap = [](int v) { return v < 0 ? v + W : (v >= W ? v - W : v); };
  const int Xm = wrap(-X);
  const size_t ME = CM ? 2 : 1;  // floats per mask element
  float2 acc[EN];
#pragma unroll
  for (int i = 0; i < EN; i++) acc[i] = make_float2(0.f, 0.f);
  auto qoff = [&](int xl) { return ((size_t)(xl >> 2) * nWin) * 4 + (xl & 3); };
  b2_band0<N, T2, EN, CM>(J, acc, t, X, Xm);
  for (int a = 0; a < J.nA; a++) {
    for (int b = 1; b <= nPair; b++) {
      const int cn = 2 * b - 1, cp = 2 * b, ab = a * nPair + (b - 1);
      const float2* Tc = J.Tw + (size_t)(1 + ab) * nWin * nWin;
      const float2* Qx = J.nyq + (size_t)(ab * 2) * N;
      const float2* Qy = Qx + N;
      const float2* G = J.G + (size_t)ab * nWin;
      const int xn = wrap(X - J.win[2 * (a * nC + cn)]);
      if (xn < nWin) {  // neg at (X, Y), and the pos component's n2 at (-X, -Y)
        const float* mk = J.masks + ((size_t)(a * nC + cn) * nWin * nWin + qoff(xn)) * ME;
        const float2 cxm = cmul(twW[Xm], __ldg(Qx + (Xm < N ? Xm : Xm - N)));
        b2_pair<N, T2, EN, CM, false, false>(acc, t, J.win[2 * (a * nC + cn) + 1], nWin, Tc + qoff(xn), mk,
                                             reinterpret_cast<const float2*>(mk), G, Qy,
                                             J.Dy[(size_t)ab * nWin + xn], cxm, twW);
      }
      const int xp = wrap(X - J.win[2 * (a * nC + cp)]);
      if (xp < nWin) {  // pos at (X, Y) from the neg transform at (-X, -Y)
        const int xm = nWin - 1 - xp;  // window column of -X in the neg window
        const float* mk = J.masks + ((size_t)(a * nC + cp) * nWin * nWin + qoff(xp)) * ME;
        const float2 cx = cmul(twW[X], __ldg(Qx + (X < N ? X : X - N)));
        b2_pair<N, T2, EN, CM, true, false>(acc, t, J.win[2 * (a * nC + cp) + 1], nWin, Tc + qoff(xm), mk,
                                            reinterpret_cast<const float2*>(mk), G, Qy,
                                            J.Dy[(size_t)ab * nWin + xm], cx, twW);
      }
    }
  }
  b2_finish<N, T, CB, EN>(J, acc, bz, bh, lt, lane, t, X);
}

// Pass B2 with bulk-copy staging. The pair components whose window covers a column of this
// block's quad are processed as stages: one thread copies a stage's window column quads of
// the neg transforms, the component's mask quads, the pair's G column and Qy response into a
// ring of `depth` shared-memory slots with cp.async.bulk, `depth` stages ahead, each slot
// tracked by an mbarrier; the block reads the stage from shared memory. A pos component reads
// the mirrored neg column quad, which is aligned with the window's quads; the neg window is
// the mirror image of the aligned pos window, so the block's four columns fall into one or
// two of its quads, adjacent in the quad layout and copied together. Band 0 is the first
// stage (its window column quad, the one or two quads of the mirrored columns, its mask
// quad). The FFT buffers of the epilogue alias the ring. Slot layout (bytes, lw = the launch's
// largest window): pair stages quads [0, 64 lw), masks [64 lw, (64 + 32 ME) lw),
// G [.., + 8 lw), Qy [.., + 8 N); the band-0 stage mirrored quads [0, 64 lw), direct quad
// [64 lw, 96 lw), mask [96 lw, (96 + 16 ME) lw).
constexpr int B2S_MAX_DEPTH = 4;
constexpr int B2S_MAX_STAGES = 1 + 2 * FSIM_MAX_DIRS * (FSIM_MAX_BANDS - 1);
constexpr int B2S_WAIT_LIMIT = 1 << 20;  // polls of about 100 ns: a copy seen incomplete for ~0.1 s
__host__ __device__ constexpr size_t b2s_slot_bytes(int lw, int n, bool cm) {
  // pair stage: quads 64 lw, masks 32 ME lw, G 8 lw, Qy 8 n; band-0 stage: mirrored quads
  // 64 lw, the direct quad 32 lw, its mask 16 ME lw
  return ((((size_t)(64 + 32 * (cm ? 2 : 1) + 8) * lw + (size_t)8 * n) > (size_t)(96 + 16 * (cm ? 2 : 1)) * lw
               ? ((size_t)(64 + 32 * (cm ? 2 : 1) + 8) * lw + (size_t)8 * n)
               : (size_t)(96 + 16 * (cm ? 2 : 1)) * lw) +
          127) /
         128 * 128;
}
template <int N, int ENV, int CBV, bool CM>
__global__ void __launch_bounds__(2 * Cfg<N, ENV, CBV>::CB* Cfg<N, ENV, CBV>::T,
                                  col_min_blocks<2 * Cfg<N, ENV, CBV>::CB * Cfg<N, ENV, CBV>::T,
                                                 Cfg<N, ENV, CBV>::EN, FSIM_B2_REGS>())
    k_pass_b2s(const JobDesc* __restrict__ jobs, int lw, int slot_bytes, int depth) {
  using P = Cfg<N, ENV, CBV>;
  constexpr int W = P::W, T = P::T, CB = P::CB, EN = P::EN, T2 = 2 * T;
  constexpr int ME = CM ? 2 : 1;
  static_assert(EN % 2 == 0, "rows k and k + N must share a thread");
  static_assert(CB == 4, "one block per column quad");
  const int lt = threadIdx.x, lane = lt % CB, t = lt / CB;
  const int X = blockIdx.x * CB + lane;
  __shared__ JobDesc J;
  __shared__ alignas(8) uint64_t full[B2S_MAX_DEPTH];
  // per stage: (a * nPair + b - 1, kind | quads << 2, first Tw quad, first mask quad); kind 0
  // a pair's neg component, 1 its pos component, 2 band 0 (then: -, kind | mirrored quads << 2,
  // the direct quad, the first mirrored quad)
  __shared__ int4 stg[B2S_MAX_STAGES];
  __shared__ int nstg, expired;
  extern __shared__ __align__(128) unsigned char b2s_ring[];
  const float2* twW = g_tw + tw_offset(W);
  load_job(&J, jobs + blockIdx.y, lt, CB * T2);
  __syncthreads();
  if ((J.cmask != 0) != CM) return;
  const int nC = J.nC, nWin = J.nWin, nPair = (nC - 1) / 2;
  auto wrap = [](int v) { return v < 0 ? v + W : (v >= W ? v - W : v); };
  const int Xm = wrap(-X);
  if (lt == 0) {
    const int X0 = blockIdx.x * CB;
    int n = 0;
    {  // band 0: its window is quad-aligned; the mirrored columns fall into one or two quads
      const int xl0 = wrap(X0 - J.win[0]);
      if (xl0 < nWin) {
        int mlo = 1 << 30, mhi = -1;
        for (int l = 0; l < CB; l++) {
          const int xlm = wrap(wrap(-(X0 + l)) - J.win[0]);
          if (xlm < nWin) {
            mlo = min(mlo, xlm >> 2);
            mhi = max(mhi, xlm >> 2);
          }
        }
        if (mhi < 0) stg[n++] = make_int4(-1, 2, xl0 >> 2, 0);
        else if (mhi - mlo <= 1) stg[n++] = make_int4(-1, 2 | ((mhi - mlo + 1) << 2), xl0 >> 2, mlo);
        else if (J.status) atomicOr(J.status, FSIM_STATUS_STAGE_LAYOUT);
      }
    }
    for (int a = 0; a < J.nA; a++)
      for (int b = 1; b <= nPair; b++) {
        const int ab = a * nPair + (b - 1);
        int qlo = 1 << 30, qhi = -1;
        for (int l = 0; l < CB; l++) {
          const int xn = wrap(X0 + l - J.win[2 * (a * nC + 2 * b - 1)]);
          if (xn < nWin) {
            qlo = min(qlo, xn >> 2);
            qhi = max(qhi, xn >> 2);
          }
        }
        // the columns are consecutive inside the window (it is narrower than the grid), so
        // their quads are one or two adjacent ones
        if (qhi >= 0 && qhi - qlo <= 1) stg[n++] = make_int4(ab, (qhi - qlo + 1) << 2, qlo, qlo);
        else if (qhi >= 0 && J.status) atomicOr(J.status, FSIM_STATUS_STAGE_LAYOUT);
        const int xp0 = wrap(X0 - J.win[2 * (a * nC + 2 * b)]);  // the pos window is quad-aligned
        if (xp0 < nWin) stg[n++] = make_int4(ab, 1 | (1 << 2), (nWin - 1 - xp0) >> 2, xp0 >> 2);
      }
    nstg = n;
    expired = 0;
    for (int d = 0; d < depth; d++) mbar_init(&full[d], 1);
    mbar_init_fence();
  }
  __syncthreads();
  const int ns = nstg;
  const size_t oq = 0, om = (size_t)64 * lw, og = om + (size_t)32 * ME * lw, oy = og + (size_t)8 * lw;
  const size_t od0 = (size_t)64 * lw, ok0 = (size_t)96 * lw;  // band-0 stage: direct quad, mask
  auto issue = [&](int s) {  // thread 0: stage s into slot s % depth
    const int4 e = stg[s];
    unsigned char* slot = b2s_ring + (size_t)(s % depth) * slot_bytes;
    if ((e.y & 3) == 2) {
      const int nqm = e.y >> 2;
      const uint32_t bd = 32u * nWin, bk = 16u * ME * nWin, bmq = 32u * nqm * nWin;
      uint64_t* bar = &full[s % depth];
      mbar_arrive_expect(bar, bd + bk + bmq);
      bulk_copy_g2s(slot + od0, J.Tw + (size_t)e.z * nWin * 4, bd, bar);
      bulk_copy_g2s(slot + ok0, J.masks + (size_t)e.z * nWin * 4 * ME, bk, bar);
      if (nqm) bulk_copy_g2s(slot, J.Tw + (size_t)e.w * nWin * 4, bmq, bar);
      return;
    }
    const int ab = e.x, a = ab / nPair, b = ab % nPair + 1, pos = e.y & 1, nq = e.y >> 2;
    const int comp = pos ? 2 * b : 2 * b - 1;
    const float2* src_q = J.Tw + ((size_t)(1 + ab) * nWin * nWin + (size_t)e.z * nWin * 4);
    const float* src_m = J.masks + ((size_t)(a * nC + comp) * nWin * nWin + (size_t)e.w * nWin * 4) * ME;
    const float2* src_g = J.G + (size_t)ab * nWin;
    const float2* src_y = J.nyq + (size_t)(ab * 2 + 1) * N;
    const uint32_t bq = 32u * nq * nWin, bm = 16u * ME * nq * nWin, bg = 8u * nWin, by = 8u * N;
    uint64_t* bar = &full[s % depth];
    mbar_arrive_expect(bar, bq + bm + bg + by);
    bulk_copy_g2s(slot + oq, src_q, bq, bar);
    bulk_copy_g2s(slot + om, src_m, bm, bar);
    bulk_copy_g2s(slot + og, src_g, bg, bar);
    bulk_copy_g2s(slot + oy, src_y, by, bar);
  };
  if (lt == 0) {
    fence_proxy_async();
    for (int s = 0; s < ns && s < depth; s++) issue(s);
  }
  float2 acc[EN];
#pragma unroll
  for (int i = 0; i < EN; i++) acc[i] = make_float2(0.f, 0.f);
  for (int s = 0; s < ns; s++) {
    uint64_t* bar = &full[s % depth];
    const uint32_t par = (uint32_t)(s / depth) & 1u;
    if (!bulk_wait(bar, par, B2S_WAIT_LIMIT)) {
      expired = 1;
      if (J.status && atomicOr(J.status, FSIM_STATUS_BULK_WAIT) == 0) {
        const unsigned long long w = *reinterpret_cast<volatile unsigned long long*>(bar);
        J.status[1] = (int)blockIdx.x | (s << 12) | (ns << 18) | (depth << 24);
        J.status[2] = (int)(w & 0xffffffffu);
        J.status[3] = (int)(w >> 32);
      }
    }
    const int4 e = stg[s];
    const unsigned char* slot = b2s_ring + (size_t)(s % depth) * slot_bytes;
    if ((e.y & 3) == 2) {  // band 0 from the staged direct and mirrored column quads
      const int xl = wrap(X - J.win[0]), xlm = wrap(Xm - J.win[0]);
      const bool mirror_in = xlm < nWin;
      const float2* tv = reinterpret_cast<const float2*>(slot + od0) + (xl & 3);
      const float2* tm = reinterpret_cast<const float2*>(slot) +
                         (mirror_in ? (size_t)((xlm >> 2) - e.w) * nWin * 4 + (xlm & 3) : 0);
      const float* mk = reinterpret_cast<const float*>(slot + ok0) + (xl & 3) * ME;
      b2_band0_px<N, T2, EN, CM, true>(acc, t, J.win[1], nWin, tv, tm, mirror_in, mk,
                                       reinterpret_cast<const float2*>(mk));
      __syncthreads();  // every thread is done with the slot
      if (lt == 0 && s + depth < ns) {
        fence_proxy_async();
        issue(s + depth);
      }
      continue;
    }
    const int ab = e.x, a = ab / nPair, b = ab % nPair + 1;
    const float2* Qx = J.nyq + (size_t)(ab * 2) * N;
    const float2* sq = reinterpret_cast<const float2*>(slot + oq);
    const float* smk = reinterpret_cast<const float*>(slot + om);
    const float2* sg = reinterpret_cast<const float2*>(slot + og);
    const float2* sy = reinterpret_cast<const float2*>(slot + oy);
    if ((e.y & 3) == 0) {
      const int xn = wrap(X - J.win[2 * (a * nC + 2 * b - 1)]);
      if (xn < nWin) {
        const size_t qo = (size_t)((xn >> 2) - e.z) * nWin * 4 + (xn & 3);
        const float* mk = smk + qo * ME;
        const float2 cxm = cmul(twW[Xm], __ldg(Qx + (Xm < N ? Xm : Xm - N)));
        b2_pair<N, T2, EN, CM, false, true>(acc, t, J.win[2 * (a * nC + 2 * b - 1) + 1], nWin, sq + qo, mk,
                                            reinterpret_cast<const float2*>(mk), sg, sy,
                                            J.Dy[(size_t)ab * nWin + xn], cxm, twW);
      }
    } else {
      const int xp = wrap(X - J.win[2 * (a * nC + 2 * b)]), xm = nWin - 1 - xp;
      const float* mk = smk + ((size_t)((xp >> 2) - e.w) * nWin * 4 + (xp & 3)) * ME;
      const float2 cx = cmul(twW[X], __ldg(Qx + (X < N ? X : X - N)));
      b2_pair<N, T2, EN, CM, true, true>(acc, t, J.win[2 * (a * nC + 2 * b) + 1], nWin,
                                         sq + (size_t)((xm >> 2) - e.z) * nWin * 4 + (xm & 3), mk,
                                         reinterpret_cast<const float2*>(mk), sg, sy,
                                         J.Dy[(size_t)ab * nWin + xm], cx, twW);
    }
    __syncthreads();  // every thread is done with the slot
    if (lt == 0 && s + depth < ns) {
      fence_proxy_async();
      issue(s + depth);
    }
  }
  // the ring is free (every issued stage was waited for and read): the FFT buffers alias it.
  // After an expired wait, the copies of each slot's last stage are waited for once more
  // (bounded) before the buffers are reused and the block exits.
  if (expired) {
    if (lt == 0)
      for (int s = ns - depth < 0 ? 0 : ns - depth; s < ns; s++)
        bulk_wait(&full[s % depth], (uint32_t)(s / depth) & 1u, B2S_WAIT_LIMIT);
    __syncthreads();
  }
  float2* bz = reinterpret_cast<float2*>(b2s_ring);
  float2* bh = bz + smem_line_elems(N, CB);
  b2_finish<N, T, CB, EN>(J, acc, bz, bh, lt, lane, t, X);
}

// ---- pass C: rows of the output (complex-to-real) ------------------------------------------------
// Row y of the image is out[x] = sum_X H[X] exp(+2 pi i x X/W) / W^2 with H[W-X] = conj H[X],
// H[0..N-1] = O[y][.] and H[N] = On[y]. Both halves of the output come from one N-point
// inverse FFT: Z[k] = (H[k] + conj H[N-k]) + i exp(+2 pi i k/W) (H[k] - conj H[N-k]) gives
// iFFT_N(Z)[n] = out[2n] + i out[2n+1] (the two sub-sequences' transforms are real).
// clip != 0 clips negative values (CLIPSCALE.CLIP); clip == 2 also records the image's
// maximum (CLIPSCALE.BOTH: k_scale_clip scales afterwards, before clipping).
template <int N>
__global__ void __launch_bounds__(Cfg<N>::GC* Cfg<N>::T) k_pass_c(const JobDesc* __restrict__ jobs) {
  using P = Cfg<N>;
  constexpr int W = P::W, T = P::T, G = P::GC, EN = P::EN;
  const JobDesc& J = jobs[blockIdx.y];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int y = blockIdx.x * G + g;
  __shared__ float2 sm[G * smem_line_elems(N, 1)];
  // stage twiddles through L1 (a per-block shared copy of the 511-entry table cost a 4 KB
  // copy and a barrier per pair of rows)
  const float2* tw = g_stw + stw_offset(N, EN);
  float2* s = sm + g * smem_line_elems(N, 1);
  const float2* twW = g_tw + tw_offset(W);
  const float2* row = J.O + (size_t)y * N;
  const float2 hn = J.On[y];
  float2 x[EN];  // element t + i*T of Z, in registers through the transform
#pragma unroll
  for (int i = 0; i < EN; i++) {
    const int k = t + i * T;
    const float2 h = row[k];
    const float2 hm = cconjf(k == 0 ? hn : row[N - k]);
    const float2 e = cadd(h, hm), d = cmul(csub(h, hm), cconjf(twW[k]));
    x[i] = make_float2(e.x - d.y, e.y + d.x);  // e + i d
  }
  line_fft_reg<N, T, 1, true>(x, s, 0, t, tw);
  const float scale = 1.f / ((float)W * (float)W);
  const int clip = J.clip;
  float2* out = reinterpret_cast<float2*>(J.out + (size_t)y * W);
  float mx = 0.f;
#pragma unroll
  for (int i = 0; i < EN; i++) {
    float2 v = make_float2(x[i].x * scale, x[i].y * scale);
    if (clip == 2) mx = fmaxf(mx, fmaxf(v.x, v.y));
    if (clip == 1) {
      if (v.x < 0) v.x = 0.f;
      if (v.y < 0) v.y = 0.f;
    }
    out[t + i * T] = v;
  }
  if (clip == 2) {  // non-negative floats order as their bit patterns
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0 && mx > 0.f) atomicMax(reinterpret_cast<unsigned int*>(J.clip_max), __float_as_uint(mx));
  }
}

// CLIPSCALE.BOTH (SimUtils.clipAndScale(vec, true, true), S/SimUtils.java:244-264): every pixel
// times 255/max (max over the image, starting at 0), then negative values set to 0.
static __global__ void k_scale_clip(const JobDesc* __restrict__ jobs, int W) {
  const JobDesc& J = jobs[blockIdx.y];
  if (J.clip != 2) return;
  const float f = __fdiv_rn(255.f, *J.clip_max);
  float* out = J.out;
  const size_t n = (size_t)W * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float v = __fmul_rn(out[i], f);
    if (v < 0) v = 0.f;
    out[i] = v;
  }
}

// ---- launch ----------------------------------------------------------------------------------------
// Each pass has its own launch-shape variants (autotuner: tuning.json); a batch launches
// A, G, B1, B2, C in order on one stream.
template <int N, int ENA>
static void launch_a(const JobDesc* d_jobs, int njobs, int maxA, int maxPair, cudaStream_t st) {
  using PAR = PassA<N, ENA>;
  // blockIdx.x: RB rows; blockIdx.y: the angles' band pairs, then (y == nA) the band-0 rows
  // of all angles
  k_pass_a<N, ENA><<<dim3(N / PAR::RB, maxA + 1, njobs), PAR::NT, 0, st>>>(d_jobs);
}

template <int N, int ENA>
static void launch_g(const JobDesc* d_jobs, int njobs, int maxA, int maxPair, cudaStream_t st) {
  using PA = Cfg<N, ENA>;
  k_pass_g<N, ENA><<<dim3(maxA * maxPair, njobs), PA::T, 0, st>>>(d_jobs);
}
template <int N, int ENB, int CBB>
static int launch_b1(const JobDesc* d_jobs, int njobs, int maxA, int maxPair, int maxWin, cudaStream_t st) {
  using PB = Cfg<N, ENB, CBB>;
  const size_t smem = sizeof(float2) * 2 * smem_line_elems(N, PB::CB);
  static bool attr = false;
  if (!attr) {
    FSIM_CUDA(cudaFuncSetAttribute(k_pass_b1<N, ENB, CBB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  k_pass_b1<N, ENB, CBB><<<dim3((maxWin + PB::CB - 1) / PB::CB, 1 + maxA * maxPair, njobs), PB::CB * PB::T, smem,
                           st>>>(d_jobs);
  return FSIM_OK;
}
template <int N, int ENB, int CBB, bool CM>
static int launch_b2_kind(const JobDesc* d_jobs, int njobs, cudaStream_t st) {
  using PB = Cfg<N, ENB, CBB>;
  const size_t smem = sizeof(float2) * 2 * smem_line_elems(N, PB::CB);
  static bool attr = false;
  if (!attr) {
    FSIM_CUDA(
        cudaFuncSetAttribute(k_pass_b2<N, ENB, CBB, CM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  // the Hermitian half: columns 0..N, 2T threads per column
  k_pass_b2<N, ENB, CBB, CM><<<dim3(N / PB::CB + 1, njobs), 2 * PB::CB * PB::T, smem, st>>>(d_jobs);
  return FSIM_OK;
}
// The bulk-copy variant where `depth` >= 2 stages of the launch's largest window fit in
// B2S_RING_BYTES (two blocks of 512 threads per SM) and every window is narrower than the grid;
// otherwise (and when b2_staging_enabled() is off) the variant with plain loads.
constexpr size_t B2S_RING_BYTES = 108 * 1024;
bool b2_staging_enabled();
template <int N, int ENB, int CBB, bool CM>
static int launch_b2s_kind(const JobDesc* d_jobs, int njobs, int maxWin, cudaStream_t st) {
  using PB = Cfg<N, ENB, CBB>;
  const size_t slot = b2s_slot_bytes(maxWin, N, CM);
  const int depth = (int)std::min<size_t>(B2S_MAX_DEPTH, B2S_RING_BYTES / slot);
  if (CBB != 4 || depth < 2 || maxWin >= 2 * N || !b2_staging_enabled())
    return launch_b2_kind<N, ENB, CBB, CM>(d_jobs, njobs, st);
  if constexpr (CBB == 4) {
    const size_t smem = std::max(depth * slot, sizeof(float2) * 2 * smem_line_elems(N, PB::CB));
    static size_t attr = 0;
    if (smem > attr) {
      FSIM_CUDA(cudaFuncSetAttribute(k_pass_b2s<N, ENB, CBB, CM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
      attr = smem;
    }
    k_pass_b2s<N, ENB, CBB, CM><<<dim3(N / PB::CB + 1, njobs), 2 * PB::CB * PB::T, smem, st>>>(
        d_jobs, maxWin, (int)slot, depth);
  }
  return FSIM_OK;
}
// masks: bit 0 launches the real-mask kind, bit 1 the complex-mask kind (measured OTFs)
template <int N, int ENB, int CBB>
static int launch_b2(const JobDesc* d_jobs, int njobs, int masks, int maxWin, cudaStream_t st) {
  int rc = FSIM_OK;
  if (masks & 1) rc = launch_b2s_kind<N, ENB, CBB, false>(d_jobs, njobs, maxWin, st);
  if (!rc && (masks & 2)) rc = launch_b2s_kind<N, ENB, CBB, true>(d_jobs, njobs, maxWin, st);
  return rc;
}

// tuned variants per size: index into the variant lists of launch_offline
extern int g_var_a[16], g_var_b[16], g_var_b2[16];
__host__ inline int size_slot(int n) {
  switch (n) {
    case 64: return 0;
    case 128: return 1;
    case 192: return 2;
    case 256: return 3;
    case 384: return 4;
    case 512: return 5;
    case 768: return 6;
    case 1024: return 7;
    case 2048: return 8;
  }
  return -1;
}

// variant lists: pass A (and G) elements/thread {E0, E1}; passes B1 and B2, each on its own,
// (elements, columns per block) {(E0,4), (E0,2), (E1,4), (E1,2)} with E0 = 8, E1 = 16
// (3*2^k sizes: 12, 24). The extremes (N <= 128, N >= 2048) have one variant.
template <int N>
int launch_offline(const JobDesc* d_jobs, int njobs, int maxA, int maxPair, int maxWin, bool scale_clip, int masks,
                   cudaStream_t st) {
  constexpr bool p3 = (N % 3 == 0);
  constexpr int E0 = p3 ? 12 : 8, E1 = p3 ? 24 : 16;
  constexpr bool single = (N <= 128 || N >= 2048);
  constexpr int CBX = N >= 2048 ? 2 : 4;
  const int k = size_slot(N);
  const int va = single ? 0 : g_var_a[k], vb1 = single ? 0 : g_var_b[k], vb2 = single ? 0 : g_var_b2[k];
  cudaEvent_t* ev = profile_events();
  if (ev) cudaEventRecord(ev[0], st);
  if (va == 0) launch_a<N, E0>(d_jobs, njobs, maxA, maxPair, st);
  else if constexpr (!single) launch_a<N, E1>(d_jobs, njobs, maxA, maxPair, st);
  if (ev) cudaEventRecord(ev[1], st);
  if (maxPair > 0) {
    if (va == 0) launch_g<N, E0>(d_jobs, njobs, maxA, maxPair, st);
    else if constexpr (!single) launch_g<N, E1>(d_jobs, njobs, maxA, maxPair, st);
  }
  int rc = FSIM_OK;
  if constexpr (single) {
    rc = launch_b1<N, E0, CBX>(d_jobs, njobs, maxA, maxPair, maxWin, st);
  } else {
    switch (vb1) {
      case 0: rc = launch_b1<N, E0, 4>(d_jobs, njobs, maxA, maxPair, maxWin, st); break;
      case 1: rc = launch_b1<N, E0, 2>(d_jobs, njobs, maxA, maxPair, maxWin, st); break;
      case 2: rc = launch_b1<N, E1, 4>(d_jobs, njobs, maxA, maxPair, maxWin, st); break;
      default: rc = launch_b1<N, E1, 2>(d_jobs, njobs, maxA, maxPair, maxWin, st); break;
    }
  }
  if (rc) return rc;
  if (ev) cudaEventRecord(ev[2], st);
  if constexpr (single) {
    rc = launch_b2<N, E0, CBX>(d_jobs, njobs, masks, maxWin, st);
  } else {
    switch (vb2) {
      case 0: rc = launch_b2<N, E0, 4>(d_jobs, njobs, masks, maxWin, st); break;
      case 1: rc = launch_b2<N, E0, 2>(d_jobs, njobs, masks, maxWin, st); break;
      case 2: rc = launch_b2<N, E1, 4>(d_jobs, njobs, masks, maxWin, st); break;
      default: rc = launch_b2<N, E1, 2>(d_jobs, njobs, masks, maxWin, st); break;
    }
  }
  if (rc) return rc;
  if (ev) cudaEventRecord(ev[3], st);
  using PC = Cfg<N>;
  k_pass_c<N><<<dim3(PC::W / PC::GC, njobs), PC::GC * PC::T, 0, st>>>(d_jobs);
  if (scale_clip) k_scale_clip<<<dim3(2 * N, njobs), 256, 0, st>>>(d_jobs, 2 * N);
  if (ev) {
    cudaEventRecord(ev[4], st);
    profile_mark(4);
  }
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

}  // namespace fsim
