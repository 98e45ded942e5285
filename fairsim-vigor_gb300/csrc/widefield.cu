// Widefield side outputs of the offline reconstruction (SimAlgorithm.runReconstruction's
// Wiener path, S/SimAlgorithm.java:533-576):
//   "Widefield"          = spatial(sum over directions a of placeFreq(band0_a))
//   "filtered Widefield" = spatial(placeFreq(sum_a band0_a) * conj(OTF_0) * 1/(2 |OTF_0|^2 + w^2)
//                          inside the OTF support)   (WienerFilter.getWidefieldDenominator,
//                          S/WienerFilter.java:129-139; OtfProvider.maskOtf at (0, 0));
//                          the product of the three factors is a resident per-plan table
// Band separation is linear, so sum_a band0_a = FFT_N(sum_{a,p} M^-1_a[0][p] * prep(raw_{a,p})):
// one N x N transform per dataset. The 2N x 2N inverse of the pasted spectrum splits into
// N-point inverse FFTs of the even and odd output samples (as in the main passes):
//   out[2m]   = iFFT_N(S)[m],   out[2m+1] = iFFT_N(S * s)[m],   s(k) = exp(+i pi k~/N)
// along each axis (k~ the pasted signed frequency), scaled by 1/W^2 once at the end. The
// filter of the pasted grid equals the filter of the N grid at the source index (both use
// the same signed coordinates and cycles per micron), so it is applied before pasting.
// Three passes per dataset, run after pass C in the job's own (then free) workspace:
//   WA rows:    band-0 mix over all frames, FFT_N along x            -> Wf [N][N]
//   WB columns: FFT_N along y, (filter), even/odd inverse along y    -> V_o [W][N], o = 0, 1
//   WC rows:    even/odd inverse along x (one transform: the two real parts
//               from the Hermitian halves), 1/W^2                     -> widefield / fwf [W][W]
// Algorithmic bytes per dataset (f32 raw): nA nP 4N^2 + 8N^2 | 8N^2 + 4N^2 + 2 x 16N^2 |
// 2 x (16N^2 + 16N^2).
#include "common.cuh"
#include "fft_line.cuh"
#include "filters.cuh"
#include "otf.cuh"
#include "recon.cuh"

namespace fsim {

template <int N>
struct WfCfg {
  static constexpr int W = 2 * N;
  static constexpr int E = (N % 3 == 0) ? 12 : 8;   // elements per thread of an N-length line
  static constexpr int T = N / E;                   // threads per line
  static constexpr int G = T >= 256 ? 1 : 256 / T;  // lines per block in the row passes
  // columns per block in WB: up to 512 threads (256 for the 12-element plans, whose
  // columns need more than 128 registers per thread)
  static constexpr int TB = (N % 3 == 0) ? 256 : 512;
  static constexpr int CB = T >= TB ? 1 : (TB / T < 8 ? TB / T : 8);
};

size_t widefield_ws_bytes(int n) {
  // Wf (N*N) then V_0 and V_1 (W*N each), complex
  return (size_t)n * n * sizeof(float2) * 5;
}

__device__ __forceinline__ void wf_load_job(JobDesc* dst, const JobDesc* src, int tid, int nthreads) {
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int i = tid; i < (int)(sizeof(JobDesc) / sizeof(int)); i += nthreads) d[i] = s[i];
}

// exp(+i pi k~ / N) for the pasted signed frequency k~ of index k (k < N/2: k, else k - N)
template <int N>
__device__ __forceinline__ float2 wf_half_shift(const float2* twW, int k) {
  const int ks = k < N / 2 ? k : k - N;
  return cconjf(twW[ks < 0 ? ks + 2 * N : ks]);
}

// WA: G rows per block; row y of sum_{a,p} c0[a][p] * prep(raw[a][p]), FFT_N along x.
template <int N>
__global__ void __launch_bounds__(WfCfg<N>::G* WfCfg<N>::T) k_wf_rows(const JobDesc* __restrict__ jobs) {
  using P = WfCfg<N>;
  constexpr int E = P::E, T = P::T, G = P::G, SL = smem_line_elems(N, 1);
  __shared__ JobDesc J;
  __shared__ float2 c0[FSIM_MAX_DIRS * FSIM_MAX_PHASES];
  extern __shared__ float2 sm[];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  wf_load_job(&J, jobs + blockIdx.y, threadIdx.x, G * T);
  __syncthreads();
  if (!J.widefield && !J.fwf) return;  // uniform per block
  const int nA = J.nA, nP = J.nP, nC = J.nC, nF = nA * nP;
  for (int i = threadIdx.x; i < nF; i += G * T) c0[i] = J.coef[((i / nP) * nC) * nP + i % nP];
  __syncthreads();
  const int y = blockIdx.x * G + g;  // N is a multiple of G
  const size_t frame = (size_t)N * N, row = (size_t)y * N;
  float2 x[E];
#pragma unroll
  for (int i = 0; i < E; i++) x[i] = make_float2(0.f, 0.f);
  for (int f = 0; f < nF; f++) {
    const float2 c = c0[f];
#pragma unroll
    for (int i = 0; i < E; i++) {
      const size_t at = f * frame + row + t + i * T;
      float v = J.input_u16 ? (float)__ldg((const uint16_t*)J.raw + at) : __ldg((const float*)J.raw + at);
      if (J.bgr != 0.f) {  // background clip and border damping, as the main passes
        v = v - J.bgr;
        if (v < 0) v = 0;
      }
      if (J.damp) v = v * __ldg(J.damp + row + t + i * T);
      x[i].x += c.x * v;
      x[i].y += c.y * v;
    }
  }
  line_fft_reg<N, T, 1, false>(x, sm + g * SL, 0, t, g_stw + stw_offset(N, E));
  float2* o = J.Wf + row;
#pragma unroll
  for (int i = 0; i < E; i++) o[t + i * T] = x[i];
}

// WB: CB columns per block. Column x: FFT_N along y gives the band-0 sum S(x, k); for each
// requested output, the even and odd rows of the 2N-point inverse along y go to V_o.
template <int N>
__global__ void __launch_bounds__(WfCfg<N>::CB* WfCfg<N>::T) k_wf_cols(const JobDesc* __restrict__ jobs) {
  using P = WfCfg<N>;
  constexpr int E = P::E, T = P::T, CB = P::CB, W = P::W;
  __shared__ JobDesc J;
  extern __shared__ float2 sm[];
  const int lane = threadIdx.x % CB, t = threadIdx.x / CB;
  wf_load_job(&J, jobs + blockIdx.y, threadIdx.x, CB * T);
  __syncthreads();
  if (!J.widefield && !J.fwf) return;  // uniform per block
  const int x = blockIdx.x * CB + lane;  // N is a multiple of CB
  const float2* twN = g_stw + stw_offset(N, E);
  const float2* twW = g_tw + tw_offset(W);
  float2 S[E], y[E];
#pragma unroll
  for (int i = 0; i < E; i++) S[i] = J.Wf[(size_t)(t + i * T) * N + x];
  line_fft_reg<N, T, CB, false>(S, sm, lane, t, twN);
  for (int o = 0; o < 2; o++) {
    if (!(o == 0 ? J.widefield : J.fwf)) continue;  // uniform per block
    if (o == 1) {  // the plan's resident filter (k_build_wff)
#pragma unroll
      for (int i = 0; i < E; i++) S[i] = cscale(S[i], __ldg(J.wff + (size_t)(t + i * T) * N + x));
    }
    float2* V = J.Wf + (size_t)N * N + (size_t)o * W * N + x;
#pragma unroll
    for (int i = 0; i < E; i++) y[i] = S[i];
    line_fft_reg<N, T, CB, true>(y, sm, lane, t, twN);
#pragma unroll
    for (int i = 0; i < E; i++) V[(size_t)(2 * (t + i * T)) * N] = y[i];
#pragma unroll
    for (int i = 0; i < E; i++) y[i] = cmul(S[i], wf_half_shift<N>(twW, t + i * T));
    line_fft_reg<N, T, CB, true>(y, sm, lane, t, twN);
#pragma unroll
    for (int i = 0; i < E; i++) V[(size_t)(2 * (t + i * T) + 1) * N] = y[i];
  }
}

// WC: G rows per block of output o = blockIdx.y. Row Y of V_o: even and odd columns of the
// 2N-point inverse along x, real part, scaled by 1/W^2 (JTransforms complexInverse, scale).
template <int N>
__global__ void __launch_bounds__(WfCfg<N>::G* WfCfg<N>::T) k_wf_out(const JobDesc* __restrict__ jobs) {
  using P = WfCfg<N>;
  constexpr int E = P::E, T = P::T, G = P::G, W = P::W, SL = smem_line_elems(N, 1);
  __shared__ JobDesc J;
  extern __shared__ float2 sm[];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  wf_load_job(&J, jobs + blockIdx.z, threadIdx.x, G * T);
  __syncthreads();
  const int o = blockIdx.y;
  float* out = o == 0 ? J.widefield : J.fwf;
  if (!out) return;  // uniform per block
  const int Y = blockIdx.x * G + g;  // W is a multiple of G
  const float2* twN = g_stw + stw_offset(N, E);
  const float2* twW = g_tw + tw_offset(W);
  const float2* V = J.Wf + (size_t)N * N + (size_t)o * W * N + (size_t)Y * N;
  float2* s = sm + g * SL;
  // Only the real parts of iFFT_N(a) (even columns, a = v) and iFFT_N(b) (odd columns,
  // b = v * s) are kept. Re(iFFT(a)) = iFFT(Ha), Ha[k] = (a[k] + conj(a[-k]))/2 is real, so
  // one transform of Ha + i Hb gives both: even columns in its real part, odd in its imaginary.
  float2 v[E], y[E];
#pragma unroll
  for (int i = 0; i < E; i++) {
    v[i] = V[t + i * T];
    s[sidx(t + i * T)] = v[i];
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < E; i++) {
    const int k = t + i * T, km = k == 0 ? 0 : N - k;
    const float2 vm = s[sidx(km)];
    const float2 a = v[i], am = vm;
    const float2 b = cmul(v[i], wf_half_shift<N>(twW, k)), bm = cmul(vm, wf_half_shift<N>(twW, km));
    const float2 ha = make_float2(0.5f * (a.x + am.x), 0.5f * (a.y - am.y));  // (a + conj(a_-k)) / 2
    const float2 hb = make_float2(0.5f * (b.x + bm.x), 0.5f * (b.y - bm.y));
    y[i] = make_float2(ha.x - hb.y, ha.y + hb.x);  // ha + i hb
  }
  __syncthreads();  // the mirrored reads are done before the transform writes the scratch
  line_fft_reg<N, T, 1, true>(y, s, 0, t, twN);
  const float sc = (float)(1.0 / ((double)W * (double)W));
  float2* orow = reinterpret_cast<float2*>(out + (size_t)Y * W);
#pragma unroll
  for (int i = 0; i < E; i++) orow[t + i * T] = make_float2(y[i].x * sc, y[i].y * sc);
}

// The filtered widefield's filter on the N grid, built once per plan: conj(OTF_0) (the OTF
// table is real), times 1/(|OTF_0|^2 + |OTF_0|^2 + (float)(wiener^2)), zero where the
// frequency lies beyond the cutoff: OtfProvider.otfToVector (S/OtfProvider.java:331-373, no
// attenuation), WienerFilter.getWidefieldDenominator (S/WienerFilter.java:129-139, from
// addWienerDenominator at band 0, java:46-79) and OtfProvider.maskOtf(0, 0) (java:538-559).
// Table positions as otf_pos_ff (the reference's double-precision radius, MTool.fhypot, at
// the boundaries of its tests); coordinates x~ = x < N/2 ? x : x - N, y~ = y < N/2 ? -y : N - y.
__global__ void k_build_wff(float* __restrict__ f, int N, const OtfTable* __restrict__ otf, float wp) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= N) return;
  float2 o;
  float v = 0.f;
  if (otf_at_fast(*otf, 0, freq_x(x, N), freq_y(y, N), FShift{0.f, 0.f, 0.f, 0.f}, 0, 0, false, &o)) {
    const float a2 = __fmul_rn(o.x, o.x);
    v = __fmul_rn(o.x, __frcp_rn(__fadd_rn(__fadd_rn(a2, a2), wp)));
  }
  f[(size_t)y * N + x] = v;
}

int build_widefield_filter(float* d_wff, int n, const OtfTable* d_otf, float wp, cudaStream_t st) {
  k_build_wff<<<dim3(div_up(n, 128), n), 128, 0, st>>>(d_wff, n, d_otf, wp);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

template <int N>
static int launch_wf(const JobDesc* d_jobs, int njobs, cudaStream_t st) {
  using P = WfCfg<N>;
  const size_t smem_rows = sizeof(float2) * (size_t)P::G * smem_line_elems(N, 1);
  const size_t smem_cols = sizeof(float2) * (size_t)smem_line_elems(N, P::CB);
  static bool attr = false;
  if (!attr) {
    FSIM_CUDA(cudaFuncSetAttribute(k_wf_rows<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_rows));
    FSIM_CUDA(cudaFuncSetAttribute(k_wf_cols<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cols));
    FSIM_CUDA(cudaFuncSetAttribute(k_wf_out<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_rows));
    attr = true;
  }
  k_wf_rows<N><<<dim3(N / P::G, njobs), P::G * P::T, smem_rows, st>>>(d_jobs);
  k_wf_cols<N><<<dim3(N / P::CB, njobs), P::CB * P::T, smem_cols, st>>>(d_jobs);
  k_wf_out<N><<<dim3(P::W / P::G, 2, njobs), P::G * P::T, smem_rows, st>>>(d_jobs);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int launch_widefield_size(int n, const JobDesc* d_jobs, int njobs, cudaStream_t st) {
  switch (n) {
#define CASE(v) \
  case v:       \
    return launch_wf<v>(d_jobs, njobs, st);
    CASE(64) CASE(128) CASE(192) CASE(256) CASE(384) CASE(512) CASE(768) CASE(1024) CASE(2048)
#undef CASE
  }
  set_error("widefield: unsupported image size %d", n);
  return FSIM_EINVAL;
}

}  // namespace fsim
