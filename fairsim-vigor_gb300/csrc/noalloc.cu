// fsim_corr_grid_noalloc: the parameter fit's correlation-grid sweep without any device
// allocation.
//
// Some callers cannot allocate device memory while they run this step: a real-time
// acquisition thread, whose latency budget has no room for the allocator and its
// synchronisation, or a host process (for example a JVM behind JNI) whose device memory
// was partitioned up front, so that an allocation in the middle of a run could fail or
// take memory another component counts on. The regular fit (fsim_fit_peak and the
// estimation entry points) allocates its scratch per call; this entry point keeps that
// scratch in one file-scope device array instead and touches no allocator.
//
// It evaluates, for real-space bands b0, b1 (the inverse FFTs of the common-region bands,
// as Correlation.fitPeak prepares them), the grid
//   out[yi][xi] = scal * sum_{x,y} b1(x,y) conj(b0(x,y)) exp(+2 pi i (kx[xi] x - ky[yi] y)/n)
// with the allocating fit's kernels (corr_grid.cuh), so its results equal the allocating
// path's bit for bit.
//
// Limits and sharing: n <= 2048, 1 <= nx, ny <= 10. The scratch (about 0.66 MB) is one
// static array per GPU that loads the library and stays allocated until the process
// exits. Every call reuses it and it keeps the previous call's contents; nothing in it
// needs to start at zero (each call rewrites every entry it reads). Calls whose work
// overlaps on the GPU (two host threads, or two streams in flight) race on the scratch and
// must be serialised by the caller. The call is synchronous: it returns once the grid is
// in `out`.
//
// Set-up: the first call on a device (with that device current) looks up the array's
// device address with cudaGetSymbolAddress and caches it per device; make that first call
// before any stream capture.
#include <cmath>
#include <mutex>

#include "common.cuh"
#include "corr_grid.cuh"

namespace {

constexpr int NA_MAX_N = 2048;
constexpr int NA_MAX_K = fsim::CORR_MAX_K;
constexpr size_t NA_TX = 0;                                              // float2 [K][N]
constexpr size_t NA_TY = NA_TX + sizeof(float2) * NA_MAX_K * NA_MAX_N;   // float2 [K][N]
constexpr size_t NA_Q = NA_TY + sizeof(float2) * NA_MAX_K * NA_MAX_N;    // double2 [K][N]
constexpr size_t NA_CORR = NA_Q + sizeof(double2) * NA_MAX_K * NA_MAX_N; // double2 [K][K]
constexpr size_t NA_KV = NA_CORR + sizeof(double2) * NA_MAX_K * NA_MAX_K;  // double [2K]
constexpr size_t NA_BYTES = NA_KV + sizeof(double) * 2 * NA_MAX_K;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

std::mutex g_na_mu;
void* g_na_addr[64] = {nullptr};

}  // namespace

extern "C" int fsim_corr_grid_noalloc(const void* b0, const void* b1, int n, const double* kx, int nx,
                                      const double* ky, int ny, double scal, double* out, void* stream) {
  using fsim::set_error;
  if (!b0 || !b1 || !kx || !ky || !out) {
    set_error("corr_grid_noalloc: null argument");
    return FSIM_EINVAL;
  }
  if (n < 1 || n > NA_MAX_N || nx < 1 || nx > NA_MAX_K || ny < 1 || ny > NA_MAX_K) {
    set_error("corr_grid_noalloc: size %d with a %d x %d grid is beyond the static scratch (n <= %d, grid <= %d x %d)",
              n, nx, ny, NA_MAX_N, NA_MAX_K, NA_MAX_K);
    return FSIM_EINVAL;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    set_error("corr_grid_noalloc: no current device (%s)", cudaGetErrorString(e));
    return FSIM_ENODEV;
  }
  unsigned char* s = nullptr;
  {
    std::lock_guard<std::mutex> g(g_na_mu);
    if (!g_na_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        set_error("corr_grid_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
      }
      g_na_addr[dev] = p;
    }
    s = static_cast<unsigned char*>(g_na_addr[dev]);
  }
  cudaStream_t st = (cudaStream_t)stream;
  float2* tx = reinterpret_cast<float2*>(s + NA_TX);
  float2* ty = reinterpret_cast<float2*>(s + NA_TY);
  double2* Q = reinterpret_cast<double2*>(s + NA_Q);
  double2* corr = reinterpret_cast<double2*>(s + NA_CORR);
  double* kv = reinterpret_cast<double*>(s + NA_KV);
  // fourierShift(xpos, -ypos): the y ramp uses -ky
  double k[2 * NA_MAX_K] = {0};
  for (int i = 0; i < nx; i++) k[i] = kx[i];
  for (int i = 0; i < ny; i++) k[NA_MAX_K + i] = -ky[i];
  FSIM_CUDA(cudaMemcpyAsync(kv, k, sizeof(k), cudaMemcpyHostToDevice, st));
  fsim::launch_corr_grid((const float2*)b0, (const float2*)b1, n, kv, nx, ny, scal, nullptr, tx, ty, Q, corr, st);
  FSIM_CHECK_LAUNCH();
  FSIM_CUDA(cudaMemcpyAsync(out, corr, sizeof(double2) * nx * ny, cudaMemcpyDeviceToHost, st));
  FSIM_CUDA(cudaStreamSynchronize(st));
  return FSIM_OK;
}
