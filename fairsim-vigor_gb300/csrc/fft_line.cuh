// Stockham line FFT for the GB300 kernels.
//
// A "line group" is C interleaved lines of length L held in shared memory
// (element k of line c at s[sidx(k*C + c)]) and transformed by C*T threads:
// thread lt -> line c = lt % C, lane t = lt / C. Each thread owns E = L/T elements per
// stage, kept in registers while it computes E/R radix-R butterflies; stages exchange
// through shared memory (one round trip per stage, __syncthreads on both sides).
//
// Radices 16, 8, 4, 2 (and one radix-3 stage for 3*2^k lengths) are picked at compile
// time so that R divides both the remaining length and E, giving 3 stages for 512..4096
// with E = 16. Twiddles come from per-stage tables (g_stw: one to three entries per
// butterfly, the other powers by products) computed in double on the host, not from
// fast-math intrinsics; the plain table g_tw (exp(-2 pi i m/L)) serves the callers' shift
// and window factors. Lines either stay in shared memory (line_fft_st) or enter and leave
// the transform in registers (line_fft_reg, the register-chained form below).
//
// Forward = exp(-2 pi i jk/L) (unscaled); inverse = exp(+2 pi i jk/L) (unscaled; callers
// apply 1/(w*h) where fairSIM's complexInverse(scale=true) does).
#pragma once

#include "common.cuh"
#include "fft_layouts.h"

namespace fsim {

// ---- radix choice (used by the table layouts below) ----------------------------
__host__ __device__ constexpr int pick_radix_fwd(int rem, int E) {
  return (rem % 3 == 0 && E % 3 == 0)      ? 3
         : (rem % 16 == 0 && E % 16 == 0) ? 16
         : (rem % 8 == 0 && E % 8 == 0)   ? 8
         : (rem % 4 == 0 && E % 4 == 0)   ? 4
                                          : 2;
}
__host__ __device__ constexpr bool plan_ok(int L, int T) {
  if (T <= 0 || L % T) return false;
  int E = L / T, rem = L;
  while (rem > 1) {
    int R = pick_radix_fwd(rem, E);
    if (rem % R || E % R) return false;
    rem /= R;
  }
  return true;
}

// ---- twiddle tables -----------------------------------------------------------
// Powers of two 16..8192 at [L-16, 2L-16); 3*2^k lengths 48..6144 after them.
constexpr int TW_POW2_END = 2 * 8192 - 16;
constexpr int TW_TOTAL = TW_POW2_END + 2 * 6144 - 48;
__host__ __device__ constexpr bool is_pow2(int L) { return L > 0 && (L & (L - 1)) == 0; }
__host__ __device__ constexpr int tw_offset(int L) {
  return is_pow2(L) ? (L - 16) : (TW_POW2_END + (L - 48));
}
__host__ __device__ constexpr bool supported_len(int L) {
  return (is_pow2(L) && L >= 16 && L <= 8192) || (L % 3 == 0 && is_pow2(L / 3) && L >= 48 && L <= 6144);
}
// Each translation unit that runs line FFTs holds its own copy of the table (no
// relocatable device code); the registrar below hands the copy's uploader to the runtime,
// which fills every registered copy once per device in ensure_init().
static __device__ float2 g_tw[TW_TOTAL];
void fill_twiddle_host(float2* host);  // TW_TOTAL entries, computed in double
typedef int (*tw_upload_fn)();
int register_twiddle_uploader(tw_upload_fn f);
static int upload_twiddles_this_tu() {
  static float2* host = nullptr;
  if (!host) {
    host = new float2[TW_TOTAL];
    fill_twiddle_host(host);
  }
  cudaError_t e = cudaMemcpyToSymbol(g_tw, host, sizeof(float2) * TW_TOTAL);
  return e == cudaSuccess ? 0 : -3;
}
static int g_tw_registered = register_twiddle_uploader(&upload_twiddles_this_tu);

// ---- per-stage twiddle tables --------------------------------------------------
// For a line FFT of length L with E elements per thread, stage s (radix R, stride NS)
// needs W_L^{r*k*L/(NS*R)} for r = 1..R-1, k = 0..NS-1. The tables store them as
// [stage][r-1][k]: threads of a warp read consecutive k, so the loads are conflict free
// (reading the plain table at index r*k*stride serialises on shared-memory banks).
constexpr int STW_NE = 6;
__host__ __device__ constexpr int stw_e(int i) { return i == 0 ? 4 : i == 1 ? 6 : i == 2 ? 8 : i == 3 ? 12 : i == 4 ? 16 : 24; }
__host__ __device__ constexpr int stw_len(int L, int E) {  // entries of one (L, E) table
  int n = 0, rem = L, NS = 1;
  while (rem > 1) {
    int R = pick_radix_fwd(rem, E);
    n += (R - 1) * NS;
    NS *= R;
    rem /= R;
  }
  return n;
}
__host__ __device__ constexpr bool stw_ok(int L, int E) { return supported_len(L) && L % E == 0 && plan_ok(L, L / E); }
__host__ __device__ constexpr int stw_offset(int L, int E) {  // position of (L, E) in g_stw
  int off = 0;
  for (int L2 = 16; L2 <= 8192; L2 *= 2)
    for (int e = 0; e < STW_NE; e++) {
      if (L2 == L && stw_e(e) == E) return off;
      if (stw_ok(L2, stw_e(e))) off += stw_len(L2, stw_e(e));
    }
  for (int L2 = 48; L2 <= 6144; L2 *= 2)
    for (int e = 0; e < STW_NE; e++) {
      if (L2 == L && stw_e(e) == E) return off;
      if (stw_ok(L2, stw_e(e))) off += stw_len(L2, stw_e(e));
    }
  return off;  // total size when (L, E) is not a table
}
constexpr int STW_TOTAL = stw_offset(0, 0);
static __device__ float2 g_stw[STW_TOTAL];
void fill_stage_twiddle_host(float2* host);  // STW_TOTAL entries
static int upload_stage_twiddles_this_tu() {
  static float2* host = nullptr;
  if (!host) {
    host = new float2[STW_TOTAL];
    fill_stage_twiddle_host(host);
  }
  cudaError_t e = cudaMemcpyToSymbol(g_stw, host, sizeof(float2) * STW_TOTAL);
  return e == cudaSuccess ? 0 : -3;
}
static int g_stw_registered = register_twiddle_uploader(&upload_stage_twiddles_this_tu);

// ---- shared-memory addressing -----------------------------------------------------
// Layouts of the line buffers as the callers address them around a transform: one padding
// element per 16 (SW false), or a permutation inside each 16-element group (SW true).
template <bool SW>
__device__ __forceinline__ int sidx_t(int a) {
  if constexpr (SW) return a ^ ((a >> 4) & 7) ^ (((a >> 6) & 1) << 3);
  else return a + (a >> 4);
}
__device__ __forceinline__ int sidx(int a) { return sidx_t<false>(a); }
// Layouts of the register-chained transform's inter-stage exchanges; fft_layouts.h picks
// one per exchange with a bank model (gen_fft_layouts.py): 0 a + a/16, 1 a + a/16 + 2(a/32),
// 2 a + a/16 + 4(a/64), 3 a + a/16 + 8(a/128), 4 the permutation of sidx_t<true>. Every
// layout stays below a + a/8 + 1 entries, the size of a line buffer. On 512-point lines of
// 8 elements per thread the second exchange pads by layout 1 (96 -> 64 modelled wavefronts
// per warp pair and transform), and the first exchange of four interleaved lines too
// (384 -> 256).
template <int LAY>
__device__ __forceinline__ int sidx_x(int a) {
  if constexpr (LAY == 1) return a + (a >> 4) + ((a >> 5) << 1);
  else if constexpr (LAY == 2) return a + (a >> 4) + ((a >> 6) << 2);
  else if constexpr (LAY == 3) return a + (a >> 4) + ((a >> 7) << 3);
  else if constexpr (LAY == 4) return sidx_t<true>(a);
  else return a + (a >> 4);
}
__host__ __device__ constexpr int smem_line_elems(int L, int C) { return L * C + (L * C) / 8 + 1; }

// ---- radix-R butterflies --------------------------------------------------------
template <bool INV>
__device__ __forceinline__ float2 rot_mi(float2 a) {  // times -i (forward) / +i (inverse)
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
template <bool INV>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}
template <bool INV>
__device__ __forceinline__ void dft4(float2& v0, float2& v1, float2& v2, float2& v3) {
  float2 t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3), t3 = rot_mi<INV>(csub(v1, v3));
  v0 = cadd(t0, t2);
  v2 = csub(t0, t2);
  v1 = cadd(t1, t3);
  v3 = csub(t1, t3);
}
template <bool INV>
__device__ __forceinline__ void dft3(float2& a, float2& b, float2& c) {
  const float h = 0.86602540378443864676f;  // sqrt(3)/2
  float2 s = cadd(b, c), d = csub(b, c);
  float2 m = make_float2(a.x - 0.5f * s.x, a.y - 0.5f * s.y);
  float2 r = rot_mi<INV>(d);
  a = cadd(a, s);
  b = make_float2(m.x + h * r.x, m.y + h * r.y);
  c = make_float2(m.x - h * r.x, m.y - h * r.y);
}
template <bool INV>
__device__ __forceinline__ void dft8(float2* v) {
  const float q = 0.70710678118654752440f;
  float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<INV>(e0, e1, e2, e3);
  dft4<INV>(o0, o1, o2, o3);
  // W8^1, W8^2, W8^3 (forward: e^{-i pi/4 k}; inverse conjugated)
  float2 w1 = INV ? make_float2(q, q) : make_float2(q, -q);
  float2 w3 = INV ? make_float2(-q, q) : make_float2(-q, -q);
  o1 = cmul(o1, w1);
  o2 = rot_mi<INV>(o2);
  o3 = cmul(o3, w3);
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1);
  v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2);
  v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3);
  v[7] = csub(e3, o3);
}
template <bool INV>
__device__ __forceinline__ void dft16(float2* v) {
  // 4 x 4: sub-DFTs over m for v[q + 4m], twiddle W16^{q*k1}, then DFT4 over q.
  float2 x[4][4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    x[q][0] = v[q];
    x[q][1] = v[q + 4];
    x[q][2] = v[q + 8];
    x[q][3] = v[q + 12];
    dft4<INV>(x[q][0], x[q][1], x[q][2], x[q][3]);
  }
  const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f, q = 0.70710678118654752440f;
  // W16^n for n = 1,2,3,4,6,9 (forward e^{-2 pi i n/16})
  const float sg = INV ? 1.f : -1.f;
  const float2 W1 = make_float2(c1, sg * s1), W2 = make_float2(q, sg * q), W3 = make_float2(s1, sg * c1);
  const float2 W6 = make_float2(-q, sg * q), W9 = make_float2(-c1, -sg * s1);
  x[1][1] = cmul(x[1][1], W1);
  x[1][2] = cmul(x[1][2], W2);
  x[1][3] = cmul(x[1][3], W3);
  x[2][1] = cmul(x[2][1], W2);
  x[2][2] = rot_mi<INV>(x[2][2]);
  x[2][3] = cmul(x[2][3], W6);
  x[3][1] = cmul(x[3][1], W3);
  x[3][2] = cmul(x[3][2], W6);
  x[3][3] = cmul(x[3][3], W9);
#pragma unroll
  for (int k1 = 0; k1 < 4; k1++) {
    float2 a = x[0][k1], b = x[1][k1], c = x[2][k1], d = x[3][k1];
    dft4<INV>(a, b, c, d);
    v[k1] = a;
    v[k1 + 4] = b;
    v[k1 + 8] = c;
    v[k1 + 12] = d;
  }
}
template <int R, bool INV>
__device__ __forceinline__ void dft(float2* v) {
  if constexpr (R == 2) dft2<INV>(v[0], v[1]);
  else if constexpr (R == 3) dft3<INV>(v[0], v[1], v[2]);
  else if constexpr (R == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 8) dft8<INV>(v);
  else if constexpr (R == 16) dft16<INV>(v);
}

// ---- radix choice ---------------------------------------------------------------
__host__ __device__ constexpr int pick_radix(int rem, int E) { return pick_radix_fwd(rem, E); }

// ---- one Stockham stage ---------------------------------------------------------
// C interleaved lines in shared memory (padded layout sidx), stage tables [r-1][k] of this
// stage (tw points at the stage's first entry).
template <int L, int T, int C, int R, int NS, bool INV>
__device__ __forceinline__ void fft_stage(float2* s, int c, int t, const float2* tw) {
  constexpr int E = L / T, NB = E / R, LR = L / R;
  // The twiddle loads depend only on the thread's index: issue them first, so that their
  // latency overlaps the shared-memory reads and the barrier.
  constexpr int NT = NS > 1 ? (R == 16 ? 3 : (R >= 8 || R == 3 ? 2 : 1)) : 1;
  float2 tl[NB][NT];
  if constexpr (NS > 1) {
#pragma unroll
    for (int b = 0; b < NB; b++) {
      const int k = (t + b * T) % NS;
      // stage table [r-1][k]: W^k, W^2k (radix 3), W^4k (radix 8/16), W^8k (radix 16)
      tl[b][0] = tw[k];
      if constexpr (R == 3) tl[b][1] = tw[NS + k];
      if constexpr (R >= 8) tl[b][1] = tw[3 * NS + k];
      if constexpr (R == 16) tl[b][2] = tw[7 * NS + k];
    }
  }
  float2 v[NB][R];
#pragma unroll
  for (int b = 0; b < NB; b++) {
    const int j = t + b * T;
#pragma unroll
    for (int r = 0; r < R; r++) v[b][r] = s[sidx((j + r * LR) * C + c)];
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < NB; b++) {
    const int j = t + b * T;
    const int k = j % NS;
    if constexpr (NS > 1) {
      // the remaining powers by products (at most three roundings beyond the table's)
      float2 w[R];
      w[1] = tl[b][0];
      if constexpr (R == 3) w[2] = tl[b][1];
      if constexpr (R == 4) {
        w[2] = cmul(w[1], w[1]);
        w[3] = cmul(w[2], w[1]);
      }
      if constexpr (R >= 8) {
        w[4] = tl[b][1];
        w[2] = cmul(w[1], w[1]);
        w[3] = cmul(w[2], w[1]);
#pragma unroll
        for (int r = 5; r < 8; r++) w[r] = cmul(w[4], w[r - 4]);
      }
      if constexpr (R == 16) {
        w[8] = tl[b][2];
#pragma unroll
        for (int r = 9; r < 16; r++) w[r] = cmul(w[8], w[r - 8]);
      }
#pragma unroll
      for (int r = 1; r < R; r++) {
        float2 ww = w[r];
        if (INV) ww.y = -ww.y;
        v[b][r] = cmul(v[b][r], ww);
      }
    }
    const int base = (j / NS) * NS * R + k;
    dft<R, INV>(v[b]);
#pragma unroll
    for (int r = 0; r < R; r++) s[sidx((base + r * NS) * C + c)] = v[b][r];
  }
  __syncthreads();
}

// ---- register-chained transform ------------------------------------------------------
// In this Stockham plan the first stage reads, and the last stage writes, exactly the
// elements t + i*T of the thread's line (stage input j + r*L/R with j = t + b*T is element
// t + T*(b + r*E/R); the last stage writes base + r*L/R with base = j). So a line can enter
// and leave the transform in registers, x[i] = element t + i*T, and chained transforms
// with pointwise products in between skip the shared-memory round trip at both ends:
// 2(S-1) shared-memory passes for S stages instead of 2(S+1), and 2(S-1) barriers.
// The caller must not be using `s` when the transform starts (the first stage writes it);
// `s` is free again when it returns.
template <int L, int T, int C, int R, int NS, bool INV, bool FIRST, bool LAST>
__device__ __forceinline__ void fft_stage_reg(float2 (&x)[L / T], float2* s, int c, int t, const float2* tw) {
  constexpr int E = L / T, NB = E / R, LR = L / R;
  constexpr int NT = NS > 1 ? (R == 16 ? 3 : (R >= 8 || R == 3 ? 2 : 1)) : 1;
  float2 tl[NB][NT];
  if constexpr (NS > 1) {
#pragma unroll
    for (int b = 0; b < NB; b++) {
      const int k = (t + b * T) % NS;
      tl[b][0] = tw[k];
      if constexpr (R == 3) tl[b][1] = tw[NS + k];
      if constexpr (R >= 8) tl[b][1] = tw[3 * NS + k];
      if constexpr (R == 16) tl[b][2] = tw[7 * NS + k];
    }
  }
  // the exchange that feeds this stage, and the one this stage feeds (bank-model layouts)
  constexpr int LIN = fft_xlay(L, E, C, NS), LOUT = fft_xlay(L, E, C, NS * R);
  float2 v[NB][R];
#pragma unroll
  for (int b = 0; b < NB; b++)
#pragma unroll
    for (int r = 0; r < R; r++) {
      if constexpr (FIRST) v[b][r] = x[b + NB * r];
      else v[b][r] = s[sidx_x<LIN>((t + b * T + r * LR) * C + c)];
    }
  if constexpr (!FIRST) __syncthreads();
#pragma unroll
  for (int b = 0; b < NB; b++) {
    const int j = t + b * T;
    const int k = j % NS;
    if constexpr (NS > 1) {
      float2 w[R];
      w[1] = tl[b][0];
      if constexpr (R == 3) w[2] = tl[b][1];
      if constexpr (R == 4) {
        w[2] = cmul(w[1], w[1]);
        w[3] = cmul(w[2], w[1]);
      }
      if constexpr (R >= 8) {
        w[4] = tl[b][1];
        w[2] = cmul(w[1], w[1]);
        w[3] = cmul(w[2], w[1]);
#pragma unroll
        for (int r = 5; r < 8; r++) w[r] = cmul(w[4], w[r - 4]);
      }
      if constexpr (R == 16) {
        w[8] = tl[b][2];
#pragma unroll
        for (int r = 9; r < 16; r++) w[r] = cmul(w[8], w[r - 8]);
      }
#pragma unroll
      for (int r = 1; r < R; r++) {
        float2 ww = w[r];
        if (INV) ww.y = -ww.y;
        v[b][r] = cmul(v[b][r], ww);
      }
    }
    dft<R, INV>(v[b]);
    if constexpr (LAST) {
#pragma unroll
      for (int r = 0; r < R; r++) x[b + NB * r] = v[b][r];
    } else {
      const int base = (j / NS) * NS * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) s[sidx_x<LOUT>((base + r * NS) * C + c)] = v[b][r];
    }
  }
  if constexpr (!LAST) __syncthreads();
}
template <int L, int T, int C, bool INV, int NS>
__device__ __forceinline__ void fft_stages_reg(float2 (&x)[L / T], float2* s, int c, int t, const float2* tw) {
  constexpr int R = pick_radix(L / NS, L / T);
  static_assert((L / NS) % R == 0 && (L / T) % R == 0, "bad radix plan");
  fft_stage_reg<L, T, C, R, NS, INV, NS == 1, NS * R == L>(x, s, c, t, tw);
  if constexpr (NS * R < L) fft_stages_reg<L, T, C, INV, NS * R>(x, s, c, t, tw + (R - 1) * NS);
}
// Transform line c of C interleaved lines held in registers (x[i] = element t + i*T),
// with `s` (C interleaved lines, shared memory) as scratch; stage tables (g_stw layout).
template <int L, int T, int C, bool INV>
__device__ __forceinline__ void line_fft_reg(float2 (&x)[L / T], float2* s, int c, int t, const float2* stw) {
  static_assert(supported_len(L) && plan_ok(L, T) && stw_ok(L, L / T), "no stage table for this plan");
  fft_stages_reg<L, T, C, INV, 1>(x, s, c, t, stw);
}

template <int L, int T, int C, bool INV, int NS>
__device__ __forceinline__ void fft_stages(float2* s, int c, int t, const float2* tw) {
  if constexpr (NS < L) {
    constexpr int R = pick_radix(L / NS, L / T);
    static_assert((L / NS) % R == 0 && (L / T) % R == 0, "bad radix plan");
    fft_stage<L, T, C, R, NS, INV>(s, c, t, tw);
    // stage tables: the next stage's entries follow this stage's (R-1)*NS entries
    fft_stages<L, T, C, INV, NS * R>(s, c, t, tw + (R - 1) * NS);
  }
}

// Transform C interleaved lines of length L in place in shared memory `s` (element k of
// line c at s[sidx(k*C + c)]) with per-stage twiddle tables (g_stw layout, read through L1).
// Called by exactly C*T threads (the whole block): it contains __syncthreads.
template <int L, int T, int C, bool INV>
__device__ __forceinline__ void line_fft_st(float2* s, int lt, const float2* stw) {
  static_assert(supported_len(L) && plan_ok(L, T) && stw_ok(L, L / T), "no stage table for this plan");
  fft_stages<L, T, C, INV, 1>(s, lt % C, lt / C, stw);
}

}  // namespace fsim
