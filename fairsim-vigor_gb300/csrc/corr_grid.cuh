// The correlation grid of Correlation.fitPeak's inner loop (S/Correlation.java:43-136),
// shared by the allocating fit (estimate.cu) and the allocation-free sweep (noalloc.cu), so
// that both evaluate the same arithmetic and give the same bits.
//
// The shift phase ramp of fitPeak's fourierShift(kx, -ky) is separable, so
//   corr(xi, yi) = scal * sum_y ty[yi](y) * sum_x tx[xi](x) * b1(x,y) * conj(b0(x,y)),
// evaluated as NK row sums per image row (one warp per row), then nkx*nky column sums.
// Each lane adds its pixels of a row (N / 32 of them) in float, one sum per ramp; the warp
// sums those partials, and the column pass sums the rows, in FP64 in a fixed order
// (deterministic).
#pragma once

#include "common.cuh"

namespace fsim {
namespace {

// tab[j][x] = exp(+2 pi i k[j] x / N), the phase reduced modulo one turn in double
__global__ void k_ramp_table(float2* __restrict__ tab, const double* __restrict__ k, int nk, int N) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (x >= N || j >= nk) return;
  double f = k[j] * (double)x / (double)N;
  f -= floor(f);
  double s, c;
  sincospi(2.0 * f, &s, &c);
  tab[(size_t)j * N + x] = make_float2((float)c, (float)s);
}

// Q[j][y] = sum_x b1(x,y) conj(b0(x,y)) tx[j][x] for the nk <= NK ramps of the grid's x
// axis (rows j >= nk of Q are left untouched). One warp per image row: each lane sums its
// pixels x = lane + 32 m in float, one sum per ramp, and the warp adds the 32 partials in
// FP64 in a fixed order. (With 256 threads per row the FP64 reduction of 4-pixel partials
// took most of the time: GB300 runs FP64 at a small fraction of its FP32 rate.)
// eight rows per block: the warps of a block read the same ramp entries at the same x, so
// the ramp rows are served from L1 (two rows per block measured 3x slower at 1024^2)
constexpr int CORR_ROWS_PER_BLOCK = 8;
template <int NK>
__global__ void __launch_bounds__(32 * CORR_ROWS_PER_BLOCK)
    k_corr_rows(const float2* __restrict__ b0, const float2* __restrict__ b1, const float2* __restrict__ tx, int N,
                int nk, double2* __restrict__ Q) {
  const int lane = threadIdx.x % 32, y = blockIdx.x * CORR_ROWS_PER_BLOCK + threadIdx.x / 32;
  if (y >= N) return;  // uniform per warp
  float2 acc[NK];
#pragma unroll
  for (int j = 0; j < NK; j++) acc[j] = make_float2(0.f, 0.f);
  for (int x = lane; x < N; x += 32) {
    const size_t i = (size_t)y * N + x;
    const float2 p = cmulc(b1[i], b0[i]);  // b1 * conj(b0)
#pragma unroll
    for (int j = 0; j < NK; j++) {
      if (j < nk) {
        const float2 r = cmul(p, tx[(size_t)j * N + x]);
        acc[j].x += r.x;
        acc[j].y += r.y;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NK; j++) {
    double a = acc[j].x, b = acc[j].y;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (lane == 0 && j < nk) Q[(size_t)j * N + y] = make_double2(a, b);
  }
}

// corr[jy][jx] = scal * sum_y Q[jx][y] * ty[jy][y]: one block of CORR_COL_WARPS warps per grid
// point, warp w summing the rows y = w + CORR_COL_WARPS m (lanes strided) in FP64, the warps'
// sums added in a fixed order; scal = 1 / *n2 when n2 (a norm left on the device) is given
constexpr int CORR_COL_WARPS = 8;
__global__ void __launch_bounds__(32 * CORR_COL_WARPS)
    k_corr_cols(const double2* __restrict__ Q, const float2* __restrict__ ty, int N, int nkx, int nky, double scal,
                const double* __restrict__ n2, double2* __restrict__ out) {
  const int g = blockIdx.x, lane = threadIdx.x % 32, wp = threadIdx.x / 32;
  if (g >= nkx * nky) return;  // uniform per block
  const int jx = g % nkx, jy = g / nkx;
  double a = 0, b = 0;
  for (int y = wp * 32 + lane; y < N; y += 32 * CORR_COL_WARPS) {
    const double2 q = Q[(size_t)jx * N + y];
    const float2 t = ty[(size_t)jy * N + y];
    a += q.x * t.x - q.y * t.y;
    b += q.x * t.y + q.y * t.x;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  __shared__ double2 part[CORR_COL_WARPS];
  if (lane == 0) part[wp] = make_double2(a, b);
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0, sb = 0;
    for (int k = 0; k < CORR_COL_WARPS; k++) {
      sa += part[k].x;
      sb += part[k].y;
    }
    if (n2) scal = 1. / *n2;
    out[g] = make_double2(sa * scal, sb * scal);  // Cplx.mult(sum, (scal, 0))
  }
}

// The largest grid side of one sweep (fitPeak's 10 x 10).
constexpr int CORR_MAX_K = 10;

// Launches the sweep on stream st: tx, ty hold CORR_MAX_K ramp rows of N entries each, Q
// CORR_MAX_K rows of N, corr nkx*nky entries; kv holds the nkx x shifts at [0, nkx) and the
// nky y shifts, already negated for fourierShift(kx, -ky), at [CORR_MAX_K, CORR_MAX_K + nky).
// The normaliser is scal, or 1 / *n2 when n2 (device) is not null.
inline void launch_corr_grid(const float2* b0, const float2* b1, int N, const double* kv, int nkx, int nky, double scal,
                             const double* n2, float2* tx, float2* ty, double2* Q, double2* corr, cudaStream_t st) {
  k_ramp_table<<<dim3((N + 127) / 128, nkx), 128, 0, st>>>(tx, kv, nkx, N);
  k_ramp_table<<<dim3((N + 127) / 128, nky), 128, 0, st>>>(ty, kv + CORR_MAX_K, nky, N);
  const int rb = (N + CORR_ROWS_PER_BLOCK - 1) / CORR_ROWS_PER_BLOCK;
  if (nkx == 1)
    k_corr_rows<1><<<rb, 32 * CORR_ROWS_PER_BLOCK, 0, st>>>(b0, b1, tx, N, 1, Q);
  else
    k_corr_rows<CORR_MAX_K><<<rb, 32 * CORR_ROWS_PER_BLOCK, 0, st>>>(b0, b1, tx, N, nkx, Q);
  k_corr_cols<<<nkx * nky, 32 * CORR_COL_WARPS, 0, st>>>(Q, ty, N, nkx, nky, scal, n2, corr);
}

}  // namespace
}  // namespace fsim
