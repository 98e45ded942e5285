// Library runtime: error state, device/stream context, FFT twiddle tables.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fft_line.cuh"
#include "runtime.cuh"

#include <cuda_profiler_api.h>

namespace fsim {

bool fft2d_supported(int w, int h);  // fft2d.cu

static thread_local char g_errbuf[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errbuf, sizeof(g_errbuf), fmt, ap);
  va_end(ap);
}
const char* last_error() { return g_errbuf; }

// Test hook: the n-th next device allocation of the library fails (fsim_debug_fail_alloc).
static std::atomic<int> g_fail_alloc{0};
// Pass B2's bulk-copy staging on (fsim_debug_b2_staging)
static std::atomic<int> g_b2_staging{1};
bool b2_staging_enabled() { return g_b2_staging.load(std::memory_order_relaxed) != 0; }

cudaError_t dev_alloc(void** p, size_t bytes) {
  int n = g_fail_alloc.load();
  while (n > 0) {
    if (g_fail_alloc.compare_exchange_weak(n, n - 1)) {
      if (n == 1) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
      }
      break;
    }
  }
  return cudaMalloc(p, bytes);
}

cudaError_t dev_alloc_async(void** p, size_t bytes, cudaStream_t st) {
  int n = g_fail_alloc.load();
  while (n > 0) {
    if (g_fail_alloc.compare_exchange_weak(n, n - 1)) {
      if (n == 1) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
      }
      break;
    }
  }
  return cudaMallocAsync(p, bytes, st);
}

static std::mutex g_mu;
static Ctx g_ctx;

Ctx& ctx() { return g_ctx; }

void fill_twiddle_host(float2* h) {
  auto fill = [&](int L) {
    int off = tw_offset(L);
    for (int m = 0; m < L; m++) {
      double a = -2.0 * M_PI * (double)m / (double)L;
      h[off + m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
  };
  for (int L = 16; L <= 8192; L *= 2) fill(L);
  for (int L = 48; L <= 6144; L *= 2) fill(L);
}

void fill_stage_twiddle_host(float2* h) {
  auto fill = [&](int L) {
    for (int e = 0; e < STW_NE; e++) {
      const int E = stw_e(e);
      if (!stw_ok(L, E)) continue;
      float2* t = h + stw_offset(L, E);
      int rem = L, NS = 1, pos = 0;
      while (rem > 1) {
        const int R = pick_radix_fwd(rem, E);
        for (int r = 1; r < R; r++)
          for (int k = 0; k < NS; k++) {
            double a = -2.0 * M_PI * (double)r * (double)k / ((double)NS * R);
            t[pos++] = make_float2((float)std::cos(a), (float)std::sin(a));
          }
        NS *= R;
        rem /= R;
      }
    }
  };
  for (int L = 16; L <= 8192; L *= 2) fill(L);
  for (int L = 48; L <= 6144; L *= 2) fill(L);
}

static std::vector<tw_upload_fn>& uploaders() {
  static std::vector<tw_upload_fn> v;
  return v;
}
int register_twiddle_uploader(tw_upload_fn f) {
  uploaders().push_back(f);
  return (int)uploaders().size();
}
static int upload_all_twiddles() {
  for (auto f : uploaders())
    if (f() != 0) {
      set_error("uploading FFT twiddle tables failed");
      return FSIM_ECUDA;
    }
  return FSIM_OK;
}

int ensure_init() {
  std::lock_guard<std::mutex> g(g_mu);
  if (g_ctx.ready) return FSIM_OK;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    set_error("no CUDA device: %s", cudaGetErrorString(e));
    return FSIM_ENODEV;
  }
  if (g_ctx.device < 0) g_ctx.device = 0;
  FSIM_CUDA(cudaSetDevice(g_ctx.device));
  int rc = upload_all_twiddles();
  if (rc) return rc;
  if (!g_ctx.stream) {
    FSIM_CUDA(cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking));
    g_ctx.own_stream = true;
  }
  FSIM_CUDA(fsim::dev_alloc(&g_ctx.red, sizeof(double) * RED_SLOTS));
  FSIM_CUDA(cudaMallocHost(&g_ctx.red_host, sizeof(double) * RED_SLOTS));
  FSIM_CUDA(fsim::dev_alloc((void**)&g_ctx.status, 4 * sizeof(int)));
  FSIM_CUDA(cudaMemset(g_ctx.status, 0, 4 * sizeof(int)));
  cudaDeviceProp prop;
  FSIM_CUDA(cudaGetDeviceProperties(&prop, g_ctx.device));
  g_ctx.num_sms = prop.multiProcessorCount;
  g_ctx.ready = true;
  return FSIM_OK;
}

int select_device(int device) {
  std::lock_guard<std::mutex> g(g_mu);
  if (g_ctx.ready && g_ctx.device != device) {
    set_error("fsim_init: library already initialised on device %d", g_ctx.device);
    return FSIM_EINVAL;
  }
  g_ctx.device = device;
  return FSIM_OK;
}

}  // namespace fsim

extern "C" {

const char* fsim_last_error(void) { return fsim::last_error(); }

int fsim_init(int device) {
  int rc = fsim::select_device(device);
  if (rc) return rc;
  return fsim::ensure_init();
}

int fsim_sync(void) {
  int rc = fsim::ensure_init();
  if (rc) return rc;
  FSIM_CUDA(cudaDeviceSynchronize());
  return FSIM_OK;
}

int fsim_device_status(int* bits, int* detail, int clear) {
  FSIM_REQUIRE(bits, FSIM_EINVAL, "device_status: null output");
  int rc = fsim::ensure_init();
  if (rc) return rc;
  FSIM_CUDA(cudaDeviceSynchronize());
  int w[4];
  FSIM_CUDA(cudaMemcpy(w, fsim::ctx().status, sizeof(w), cudaMemcpyDeviceToHost));
  *bits = w[0];
  if (detail)
    for (int i = 0; i < 3; i++) detail[i] = w[1 + i];
  if (clear) FSIM_CUDA(cudaMemset(fsim::ctx().status, 0, sizeof(w)));
  return FSIM_OK;
}

int fsim_version(void) { return 10000; }

int fsim_buffer_alloc(size_t bytes, int host, void** out) {
  FSIM_REQUIRE(out && bytes > 0, FSIM_EINVAL, "buffer_alloc: bad arguments");
  *out = nullptr;
  int rc = fsim::ensure_init();
  if (rc) return rc;
  if (host) {
    FSIM_CUDA(cudaMallocHost(out, bytes));
  } else {
    FSIM_CUDA(fsim::dev_alloc(out, bytes));
  }
  return FSIM_OK;
}

int fsim_buffer_free(void* p, int host) {
  if (!p) return FSIM_OK;
  FSIM_CUDA(host ? cudaFreeHost(p) : cudaFree(p));
  return FSIM_OK;
}

int fsim_profiler(int start) {
  int rc = fsim::ensure_init();
  if (rc) return rc;
  FSIM_CUDA(start ? cudaProfilerStart() : cudaProfilerStop());
  return FSIM_OK;
}

int fsim_fft_plan_2d(int w, int h, int64_t* plan) {
  FSIM_REQUIRE(plan, FSIM_EINVAL, "fft_plan_2d: null output");
  *plan = 0;
  FSIM_REQUIRE(fsim::fft2d_supported(w, h), FSIM_EINVAL,
               "fft_plan_2d: no line FFT for %d x %d", w, h);
  // nothing to build: the line FFTs use the resident twiddle tables; the handle carries
  // the shape for the vector that is transformed with it
  *plan = ((int64_t)w << 32) | (int64_t)(uint32_t)h;
  return FSIM_OK;
}

int fsim_debug_b2_staging(int on, int* prev) {
  const int p = fsim::g_b2_staging.exchange(on ? 1 : 0);
  if (prev) *prev = p;
  return FSIM_OK;
}

int fsim_debug_fail_alloc(int nth) {
  FSIM_REQUIRE(nth >= 0, FSIM_EINVAL, "debug_fail_alloc: nth must be >= 0");
  fsim::g_fail_alloc.store(nth);
  return FSIM_OK;
}

int fsim_set_stream(void* stream) {
  int rc = fsim::ensure_init();
  if (rc) return rc;
  fsim::Ctx& c = fsim::ctx();
  if (stream) {
    c.stream = (cudaStream_t)stream;
  } else {
    FSIM_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    c.own_stream = true;
  }
  return FSIM_OK;
}

}  // extern "C"
