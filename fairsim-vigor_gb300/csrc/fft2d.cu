// 2D complex FFT (the replacement of the reference's cufftExecC2C path,
// accel/cuda_cplx.cu:475-514) built from the Stockham line FFT of fft_line.cuh:
//   pass 1: rows   - G rows per block, each row by T threads, coalesced row loads;
//   pass 2: columns - C adjacent columns per block interleaved in shared memory so that
//           every global access moves C*8 contiguous bytes (64 B for C = 8).
// Each pass reads and writes the array once (16 bytes per complex element per pass).
// Twiddles come from the per-stage tables (one to three loads per butterfly, the other
// powers by products), read through L1; lines enter and leave the transform in registers.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "fft_line.cuh"
#include "runtime.cuh"
#include "vec_ops.cuh"

namespace fsim {

// Lines up to 512: 8 elements per thread in 64 registers (32 resident warps per SM; 0.115 ->
// 0.111 ms for 64 x 512^2 on GB300); longer lines keep 16 (8 measured slower at 1024: 0.126
// -> 0.133 ms for 16 x 1024^2); 3*2^k lengths 12.
template <int L>
struct LinePlan {
  static constexpr int E = (L % 3 == 0) ? 12 : (L <= 512 ? (L >= 64 ? 8 : 4) : 16);
  static constexpr int T = L / E;
  static constexpr int G = T >= 256 ? 1 : 256 / T;  // rows per block in the row pass
  // column pass: columns per block (a block reads C * 8 bytes of each row; 16 columns of
  // 512 points, 1024 threads per block, measured slower: 0.115 -> 0.128 ms for 64 x 512^2)
  static constexpr int C = (E <= 8) ? (T >= 128 ? 4 : 8) : (L <= 1024 ? 8 : (L <= 3072 ? 4 : 2));
  static constexpr int MINB_R = (E <= 8) ? 4 : 1;  // blocks per SM the register budgets allow
  static constexpr int MINB_C = (E <= 8) ? 65536 / (C * T * 64) : 1;
};

template <int L, bool INV>
__global__ void __launch_bounds__(LinePlan<L>::G* LinePlan<L>::T, LinePlan<L>::MINB_R)
    k_fft_rows(float2* __restrict__ data, int nrows, size_t item_stride, float scale) {
  using P = LinePlan<L>;
  constexpr int T = P::T, E = P::E, G = P::G, SL = smem_line_elems(L, 1);
  extern __shared__ float2 sm[];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int row = blockIdx.x * G + g;
  float2* s = sm + g * SL;
  float2* base = data + blockIdx.y * item_stride + (size_t)row * L;
  float2 x[E];  // element t + i*T of the row: in and out of the transform in registers
#pragma unroll
  for (int i = 0; i < E; i++) x[i] = row < nrows ? base[t + i * T] : make_float2(0.f, 0.f);
  line_fft_reg<L, T, 1, INV>(x, s, 0, t, g_stw + stw_offset(L, E));
  if (row < nrows) {
#pragma unroll
    for (int i = 0; i < E; i++) base[t + i * T] = cscale(x[i], scale);
  }
}

template <int L, bool INV>
__device__ __forceinline__ void fft_cols_body(float2* __restrict__ data, int ncols, size_t item_stride, float scale) {
  using P = LinePlan<L>;
  constexpr int T = P::T, E = P::E, C = P::C;
  extern __shared__ float2 s[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int x = blockIdx.x * C + c;
  float2* base = data + blockIdx.y * item_stride;
  float2 v[E];  // element t + i*T of the column: in and out of the transform in registers
#pragma unroll
  for (int i = 0; i < E; i++) v[i] = (x < ncols) ? base[(size_t)(t + i * T) * ncols + x] : make_float2(0.f, 0.f);
  line_fft_reg<L, T, C, INV>(v, s, c, t, g_stw + stw_offset(L, E));
  if (x < ncols) {
#pragma unroll
    for (int i = 0; i < E; i++) base[(size_t)(t + i * T) * ncols + x] = cscale(v[i], scale);
  }
}
// 8 elements per thread: 64 registers for 32 resident warps per SM
template <int L, bool INV>
__global__ void __launch_bounds__(LinePlan<L>::C* LinePlan<L>::T, LinePlan<L>::MINB_C)
    k_fft_cols(float2* __restrict__ data, int ncols, size_t item_stride, float scale) {
  fft_cols_body<L, INV>(data, ncols, item_stride, scale);
}
// longer plans: the compiler's own register choice (a bound of 512 threads raised it from
// 96 to 121 registers at 1024 and slowed 16 x 1024^2 from 0.126 to 0.139 ms)
template <int L, bool INV>
__global__ void k_fft_cols_wide(float2* __restrict__ data, int ncols, size_t item_stride, float scale) {
  fft_cols_body<L, INV>(data, ncols, item_stride, scale);
}

template <int L, bool INV>
static int launch_rows(float2* d, int nrows, int batch, size_t stride, float scale, cudaStream_t st) {
  using P = LinePlan<L>;
  size_t smem = sizeof(float2) * (size_t)P::G * smem_line_elems(L, 1);
  static bool attr = false;
  if (!attr) {
    FSIM_CUDA(cudaFuncSetAttribute(k_fft_rows<L, INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  dim3 grid(div_up(nrows, P::G), batch);
  k_fft_rows<L, INV><<<grid, P::G * P::T, smem, st>>>(d, nrows, stride, scale);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

// Column pass with the next tile's loads in flight during this tile's transform: a
// persistent block (two per SM) walks tiles of C columns x L rows; while it transforms one,
// cp.async (16-byte copies, no registers held) fills the other of two shared-memory tile
// buffers. The plain column pass keeps only the loads of its own 8 elements per thread in
// flight and waits on them (long-scoreboard stalls, 45% of DRAM peak at 64 x 512^2).
// Requires C | ncols and 16-byte aligned rows (the launcher checks); used for 512-point
// columns (8 columns x 512 rows per tile, two 32 KB tile buffers per block).
template <int L>
struct ColPipe {
  static constexpr int C = LinePlan<L>::C, T = LinePlan<L>::T, NT = C * T;
  static constexpr int TILE = L * C;                           // float2 per tile buffer
  static constexpr int CHUNKS = TILE / 2;                      // 16-byte copies per tile
  static constexpr int PER_THREAD = CHUNKS / NT;               // copies per thread
  static constexpr size_t SMEM = sizeof(float2) * (2 * TILE + smem_line_elems(L, C));
  static_assert(CHUNKS % NT == 0 && (C * 8) % 16 == 0, "tile copies");
};
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
template <int L, bool INV>
__global__ void __launch_bounds__(ColPipe<L>::NT, 2)
    k_fft_cols_pipe(float2* __restrict__ data, int ncols, int batch, size_t item_stride, float scale) {
  using P = ColPipe<L>;
  constexpr int T = P::T, C = P::C, NT = P::NT, E = L / T;
  extern __shared__ float4 smem4[];
  float2* buf = reinterpret_cast<float2*>(smem4);  // [2][L][C]
  float2* s = buf + 2 * P::TILE;                  // exchanges of the transform
  const int lt = threadIdx.x, c = lt % C, t = lt / C;
  const int tiles_per_item = ncols / C, ntiles = tiles_per_item * batch;
  // copy k of a tile: row k / (C/2), 16-byte piece k % (C/2) of the row's C columns
  auto issue = [&](int tile, float2* dst) {
    const float2* base = data + (size_t)(tile / tiles_per_item) * item_stride + (size_t)(tile % tiles_per_item) * C;
#pragma unroll
    for (int j = 0; j < P::PER_THREAD; j++) {
      const int k = lt + j * NT, r = k / (C / 2), q = k % (C / 2);
      cp_async16(dst + r * C + 2 * q, base + (size_t)r * ncols + 2 * q);
    }
  };
  int tile = blockIdx.x, cur = 0;
  if (tile < ntiles) issue(tile, buf);
  cp_async_commit();
  for (; tile < ntiles; tile += gridDim.x, cur ^= 1) {
    const int next = tile + gridDim.x;
    if (next < ntiles) issue(next, buf + (cur ^ 1) * P::TILE);
    cp_async_commit();
    cp_async_wait<1>();  // this tile's copies (all but the group just committed) have landed
    __syncthreads();
    const float2* tb = buf + cur * P::TILE;
    float2 v[E];  // element t + i*T of column c of the tile
#pragma unroll
    for (int i = 0; i < E; i++) v[i] = tb[(t + i * T) * C + c];
    // the transform's barriers also order these reads before the tile buffer is refilled
    // (two tiles later)
    line_fft_reg<L, T, C, INV>(v, s, c, t, g_stw + stw_offset(L, E));
    float2* out = data + (size_t)(tile / tiles_per_item) * item_stride + (size_t)(tile % tiles_per_item) * C + c;
#pragma unroll
    for (int i = 0; i < E; i++) out[(size_t)(t + i * T) * ncols] = cscale(v[i], scale);
  }
  cp_async_wait<0>();
}

template <int L, bool INV>
constexpr auto cols_kernel() {
  if constexpr (LinePlan<L>::E <= 8) return k_fft_cols<L, INV>;
  else return k_fft_cols_wide<L, INV>;
}

template <int L, bool INV>
static int launch_cols(float2* d, int ncols, int batch, size_t stride, float scale, cudaStream_t st) {
  using P = LinePlan<L>;
  if constexpr (L == 512) {
    // the pipelined pass where its 16-byte copies are aligned and a batch has at least
    // as many tiles as two blocks per SM
    using Q = ColPipe<L>;
    const long long tiles = (long long)(ncols / Q::C) * batch;
    if (ncols % Q::C == 0 && ((uintptr_t)d % 16) == 0 && (stride * sizeof(float2)) % 16 == 0 &&
        ((size_t)ncols * sizeof(float2)) % 16 == 0 && tiles >= 2LL * ctx().num_sms) {
      static bool attr = false;
      if (!attr) {
        FSIM_CUDA(cudaFuncSetAttribute(k_fft_cols_pipe<L, INV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)Q::SMEM));
        attr = true;
      }
      const int grid = (int)std::min<long long>(tiles, 2LL * ctx().num_sms);
      k_fft_cols_pipe<L, INV><<<grid, Q::NT, Q::SMEM, st>>>(d, ncols, batch, stride, scale);
      FSIM_CHECK_LAUNCH();
      return FSIM_OK;
    }
  }
  size_t smem = sizeof(float2) * (size_t)smem_line_elems(L, P::C);
  auto kern = cols_kernel<L, INV>();
  static bool attr = false;
  if (!attr) {
    FSIM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  dim3 grid(div_up(ncols, P::C), batch);
  kern<<<grid, P::C * P::T, smem, st>>>(d, ncols, stride, scale);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

#define FSIM_FFT_LENGTHS(X) \
  X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) X(1536) X(2048) X(3072) X(4096)

static bool len_ok(int L) {
  switch (L) {
#define CASE(n) case n:
    FSIM_FFT_LENGTHS(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}

bool fft2d_supported(int w, int h) { return len_ok(w) && len_ok(h); }

static int rows_dispatch(int L, bool inv, float2* d, int nrows, int batch, size_t stride, float scale, cudaStream_t st) {
  switch (L) {
#define CASE(n)                                                                          \
  case n:                                                                                \
    return inv ? launch_rows<n, true>(d, nrows, batch, stride, scale, st)               \
               : launch_rows<n, false>(d, nrows, batch, stride, scale, st);
    FSIM_FFT_LENGTHS(CASE)
#undef CASE
  }
  set_error("unsupported FFT length %d", L);
  return FSIM_EINVAL;
}
static int cols_dispatch(int L, bool inv, float2* d, int ncols, int batch, size_t stride, float scale, cudaStream_t st) {
  switch (L) {
#define CASE(n)                                                                          \
  case n:                                                                                \
    return inv ? launch_cols<n, true>(d, ncols, batch, stride, scale, st)               \
               : launch_cols<n, false>(d, ncols, batch, stride, scale, st);
    FSIM_FFT_LENGTHS(CASE)
#undef CASE
  }
  set_error("unsupported FFT length %d", L);
  return FSIM_EINVAL;
}

int fft2d_device(float2* data, int w, int h, bool inverse, cudaStream_t stream, int batch) {
  FSIM_REQUIRE(fft2d_supported(w, h), FSIM_EINVAL,
               "fft2d: unsupported size %d x %d (lengths 2^k in 32..4096 and 3*2^k in 48..3072)", w, h);
  size_t stride = (size_t)w * h;
  int rc = rows_dispatch(w, inverse, data, h, batch, stride, 1.f, stream);
  if (rc) return rc;
  float scale = inverse ? (float)(1.0 / ((double)w * (double)h)) : 1.f;
  return cols_dispatch(h, inverse, data, w, batch, stride, scale, stream);
}

}  // namespace fsim

extern "C" int fsim_vec_fft2d(fsim_vec* v, int inverse) {
  int rc = fsim::ensure_init();
  if (rc) return rc;
  FSIM_REQUIRE(v && v->d && v->cplx, FSIM_EINVAL, "fft2d: complex vector required");
  return fsim::fft2d_device(reinterpret_cast<float2*>(v->d), v->w, v->h, inverse != 0, fsim::ctx().stream, 1);
}

extern "C" int fsim_fft2d_batch(void* data, int w, int h, int batch, int inverse, void* stream) {
  FSIM_REQUIRE(data && batch > 0, FSIM_EINVAL, "fft2d_batch: bad arguments");
  FSIM_REQUIRE(fsim::fft2d_supported(w, h), FSIM_EINVAL, "fft2d_batch: unsupported size %d x %d", w, h);
  int rc = fsim::ensure_init();
  if (rc) return rc;
  cudaStream_t st = stream ? (cudaStream_t)stream : fsim::ctx().stream;
  return fsim::fft2d_device(static_cast<float2*>(data), w, h, inverse != 0, st, batch);
}
