// Vector API kernels: the replacements of the reference's JNI vector natives
// (accel/cuda_real.cu, accel/cuda_cplx.cu), written for sm_103a.
//
// Elementwise ops stream float4 (two complex values) per thread with grid-stride
// loops sized to the SM count; reductions are deterministic two-level FP64 sums
// (per-block partials in a fixed grid, then one block in fixed order) so that a result
// does not depend on scheduling.
#include <mutex>

#include "common.cuh"
#include "runtime.cuh"
#include "vec_ops.cuh"

namespace fsim {

static int grid_for(size_t n, int threads) {
  long long b = (long long)((n + threads - 1) / threads);
  long long cap = (long long)ctx().num_sms * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

// ---- elementwise -----------------------------------------------------------------
__global__ void k_add(float* __restrict__ y, const float* __restrict__ x, size_t nf) {
  size_t n4 = nf / 4;
  float4* y4 = reinterpret_cast<float4*>(y);
  const float4* x4 = reinterpret_cast<const float4*>(x);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
    float4 a = y4[i], b = __ldg(&x4[i]);
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
    a.w += b.w;
    y4[i] = a;
  }
  for (size_t i = n4 * 4 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf; i += (size_t)gridDim.x * blockDim.x)
    y[i] += x[i];
}

__global__ void k_addconst_c(float2* y, size_t n, float re, float im) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float2 v = y[i];
    v.x += re;
    v.y += im;
    y[i] = v;
  }
}
__global__ void k_addconst_r(float* y, size_t n, float a) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) y[i] += a;
}

// AbstractVectorCplx.axpy(Cplx.Float a, x): y += a*x (L/AbstractVectorCplx.java:185-195)
__global__ void k_axpy_c(float2* __restrict__ y, const float2* __restrict__ x, size_t n, float re, float im) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float2 a = y[i], b = __ldg(&x[i]);
    a.x = __fadd_rn(a.x, __fsub_rn(__fmul_rn(re, b.x), __fmul_rn(im, b.y)));
    a.y = __fadd_rn(a.y, __fadd_rn(__fmul_rn(im, b.x), __fmul_rn(re, b.y)));
    y[i] = a;
  }
}
__global__ void k_axpy_r(float* __restrict__ y, const float* __restrict__ x, size_t n, float a) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) y[i] = __fadd_rn(y[i], __fmul_rn(a, x[i]));
}

// times(in, conj): y = in .* y (L/AbstractVectorCplx.java:288-304)
__global__ void k_times_cc(float2* __restrict__ y, const float2* __restrict__ x, size_t n, int conj) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float2 b = __ldg(&x[i]), a = y[i];
    if (conj) b.y = -b.y;
    y[i] = make_float2(__fsub_rn(__fmul_rn(b.x, a.x), __fmul_rn(b.y, a.y)),
                       __fadd_rn(__fmul_rn(b.y, a.x), __fmul_rn(b.x, a.y)));
  }
}
__global__ void k_times_cr(float2* __restrict__ y, const float* __restrict__ x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float s = __ldg(&x[i]);
    float2 v = y[i];
    y[i] = make_float2(v.x * s, v.y * s);
  }
}
__global__ void k_times_rr(float* __restrict__ y, const float* __restrict__ x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) y[i] *= x[i];
}
// AbstractVectorCplx.scal(Cplx.Float): multReal / multImag with separate roundings
// (L/AbstractVectorCplx.java:228-236,402-408; no FMA contraction)
__global__ void k_scal_c(float2* y, size_t n, float re, float im) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float2 v = y[i];
    y[i] = make_float2(__fsub_rn(__fmul_rn(re, v.x), __fmul_rn(im, v.y)), __fadd_rn(__fmul_rn(im, v.x), __fmul_rn(re, v.y)));
  }
}
__global__ void k_scal_r(float* y, size_t n, float a) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) y[i] *= a;
}
__global__ void k_real_to_c(float2* __restrict__ y, const float* __restrict__ x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = make_float2(x[i], 0.f);
}
__global__ void k_c_to_real(float* __restrict__ y, const float2* __restrict__ x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) y[i] = x[i].x;
}
__global__ void k_u16_to_c(float2* __restrict__ y, const uint16_t* __restrict__ x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = make_float2((float)x[i], 0.f);
}
__global__ void k_u16_to_r(float* __restrict__ y, const uint16_t* __restrict__ x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) y[i] = (float)x[i];
}
// reciproc (L/AbstractVectorCplx.java:208-216)
__global__ void k_reciproc_c(float2* y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float2 v = y[i];
    float s = v.x * v.x + v.y * v.y;
    y[i] = make_float2(v.x / s, -v.y / s);
  }
}
__global__ void k_reciproc_r(float* y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) y[i] = 1.f / y[i];
}

// ---- reductions ---------------------------------------------------------------------
// mode 0: sum of float squares (norm2), 1: plain sum (real or complex pair), 2: <conj(x), y>
template <int MODE>
__global__ void k_reduce_partial(const float* __restrict__ x, const float* __restrict__ y, size_t nf, int cplx,
                                 double* __restrict__ part) {
  double a = 0, b = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if (MODE == 0) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf; i += stride) {
      float v = x[i];
      a += (double)(v * v);
    }
  } else if (MODE == 1) {
    if (cplx) {
      const float2* x2 = reinterpret_cast<const float2*>(x);
      for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf / 2; i += stride) {
        float2 v = x2[i];
        a += v.x;
        b += v.y;
      }
    } else {
      for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf; i += stride) a += x[i];
    }
  } else if (MODE == 2) {
    // dot: sum conj(x)*y (L/AbstractVectorCplx.java:258-270)
    const float2* x2 = reinterpret_cast<const float2*>(x);
    const float2* y2 = reinterpret_cast<const float2*>(y);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf / 2; i += stride) {
      float2 u = x2[i], v = y2[i];
      a += (double)(u.x * v.x - (-u.y) * v.y);
      b += (double)((-u.y) * v.x + u.x * v.y);
    }
  } else {
    // sum x*conj(y) with the products in double (Correlation.autoCorrelation: Cplx.Double
    // mult of the float values, S/Correlation.java:313-318)
    const float2* x2 = reinterpret_cast<const float2*>(x);
    const float2* y2 = reinterpret_cast<const float2*>(y);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nf / 2; i += stride) {
      const float2 u = x2[i], v = y2[i];
      const double ur = u.x, ui = u.y, vr = v.x, vi = -(double)v.y;
      a += __dsub_rn(__dmul_rn(ur, vr), __dmul_rn(ui, vi));
      b += __dadd_rn(__dmul_rn(ur, vi), __dmul_rn(ui, vr));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  __shared__ double sa[32], sb[32];
  int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if (l == 0) {
    sa[w] = a;
    sb[w] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0, tb = 0;
    for (int i = 0; i < (int)(blockDim.x / 32); i++) {
      ta += sa[i];
      tb += sb[i];
    }
    part[2 * blockIdx.x] = ta;
    part[2 * blockIdx.x + 1] = tb;
  }
}
__global__ void k_reduce_final(const double* __restrict__ part, int nblocks, double* __restrict__ out) {
  __shared__ double sa[256], sb[256];
  double a = 0, b = 0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
    a += part[2 * i];
    b += part[2 * i + 1];
  }
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sa[threadIdx.x] += sa[threadIdx.x + s];
      sb[threadIdx.x] += sb[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sa[0];
    out[1] = sb[0];
  }
}

static std::mutex g_red_mu;

// Deterministic FP64 reduction (synchronous on `st`). mode 0: norm2, 1: sum, 2: dot.
int reduce_device(int mode, const float* x, const float* y, size_t nf, int cplx, cudaStream_t st, double* a, double* b) {
  std::lock_guard<std::mutex> g(g_red_mu);
  Ctx& c = ctx();
  const int threads = 256;
  int blocks = grid_for(nf, threads);
  if (blocks > (RED_SLOTS - 8) / 2) blocks = (RED_SLOTS - 8) / 2;
  double* part = c.red;
  double* out = c.red + RED_SLOTS - 2;
  if (mode == 0)
    k_reduce_partial<0><<<blocks, threads, 0, st>>>(x, nullptr, nf, cplx, part);
  else if (mode == 1)
    k_reduce_partial<1><<<blocks, threads, 0, st>>>(x, nullptr, nf, cplx, part);
  else if (mode == 2)
    k_reduce_partial<2><<<blocks, threads, 0, st>>>(x, y, nf, 1, part);
  else
    k_reduce_partial<3><<<blocks, threads, 0, st>>>(x, y, nf, 1, part);
  k_reduce_final<<<1, 256, 0, st>>>(part, blocks, out);
  FSIM_CHECK_LAUNCH();
  FSIM_CUDA(cudaMemcpyAsync(c.red_host, out, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  FSIM_CUDA(cudaStreamSynchronize(st));
  if (a) *a = c.red_host[0];
  if (b) *b = c.red_host[1];
  return FSIM_OK;
}

static int reduce(int mode, const fsim_vec* x, const fsim_vec* y, double* a, double* b) {
  return reduce_device(mode, x->d, y ? y->d : nullptr, x->floats(), x->cplx, ctx().stream, a, b);
}

int norm2_device(const float2* v, size_t n, double* out, cudaStream_t st) {
  return reduce_device(0, reinterpret_cast<const float*>(v), nullptr, 2 * n, 1, st, out, nullptr);
}

// The same reduction (same blocks, same order, so the same bits) into the caller's RED_SLOTS
// doubles of scratch, left on the device at *result = scratch + RED_SLOTS - 2 (no sync).
int norm2_device_async(const float2* v, size_t n, double* scratch, const double** result, cudaStream_t st) {
  const int threads = 256;
  const size_t nf = 2 * n;
  int blocks = grid_for(nf, threads);
  if (blocks > (RED_SLOTS - 8) / 2) blocks = (RED_SLOTS - 8) / 2;
  k_reduce_partial<0><<<blocks, threads, 0, st>>>(reinterpret_cast<const float*>(v), nullptr, nf, 1, scratch);
  k_reduce_final<<<1, 256, 0, st>>>(scratch, blocks, scratch + RED_SLOTS - 2);
  FSIM_CHECK_LAUNCH();
  *result = scratch + RED_SLOTS - 2;
  return FSIM_OK;
}

int times_real_device(float2* y, const float* x, size_t n, cudaStream_t st) {
  k_times_cr<<<grid_for(n, 256), 256, 0, st>>>(y, x, n);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}
int times_cplx_device(float2* y, const float2* x, size_t n, bool conj, cudaStream_t st) {
  k_times_cc<<<grid_for(n, 256), 256, 0, st>>>(y, x, n, conj ? 1 : 0);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

// raw frames (u16 or f32) -> complex, times the damping vector (setFrom16bitPixels + times(dampBorder))
template <typename TIN>
__global__ void k_raw_damp(float2* __restrict__ y, const TIN* __restrict__ raw, const float* __restrict__ damp, size_t n,
                           size_t frames) {
  size_t total = n * frames;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    float v = (float)raw[i];
    if (damp) v = __fmul_rn(v, damp[i % n]);
    y[i] = make_float2(v, 0.f);
  }
}
int raw_to_cplx_device(float2* y, const void* raw, int input_u16, const float* damp, size_t n, size_t frames,
                       cudaStream_t st) {
  if (input_u16)
    k_raw_damp<uint16_t><<<grid_for(n * frames, 256), 256, 0, st>>>(y, (const uint16_t*)raw, damp, n, frames);
  else
    k_raw_damp<float><<<grid_for(n * frames, 256), 256, 0, st>>>(y, (const float*)raw, damp, n, frames);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

// ---- Fourier shift: v *= exp(i 2pi (kx x + ky y)/N) -------------------------------------
// The phase is reduced modulo one turn in double per row and per column (separable ramp)
// before the sine/cosine, instead of the reference's float-rounded full phase
// (L/BasicVectors.java:320-324); the ramp is then tx[x]*ty[y] in float.
__global__ void k_fourier_shift(float2* __restrict__ v, int N, double kx, double ky) {
  __shared__ float2 tx[32], ty[8];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  if (tid < 32) {
    int x = x0 + tid;
    double f = kx * (double)x / (double)N;
    f -= floor(f);
    double s, c;
    sincospi(2.0 * f, &s, &c);
    tx[tid] = make_float2((float)c, (float)s);
  } else if (tid < 40) {
    int y = y0 + tid - 32;
    double f = ky * (double)y / (double)N;
    f -= floor(f);
    double s, c;
    sincospi(2.0 * f, &s, &c);
    ty[tid - 32] = make_float2((float)c, (float)s);
  }
  __syncthreads();
  int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  if (x < N && y < N) {
    size_t i = (size_t)y * N + x;
    v[i] = cmul(v[i], cmul(tx[threadIdx.x], ty[threadIdx.y]));
  }
}

// ---- pasteFreq as a gather (L/BasicVectors.java:259-285) --------------------------------
// Every output element is written once; where two inputs land on the same output
// (wo < 2*wi) the one the reference's y-major loop writes last is taken.
__device__ __forceinline__ int paste_src(int o, int off, int ni, int no) {
  int p1 = ((o - off) % no + no) % no;           // from x < ni/2 (placed at x)
  int p2 = ((o - off - no / 2) % no + no) % no;  // from x >= ni/2 (placed at x + no/2)
  int best = -1;
  if (p1 < ni / 2) best = p1;
  if (p2 >= ni / 2 && p2 < ni && p2 > best) best = p2;
  return best;
}
__global__ void k_paste_freq(float2* __restrict__ out, int wo, int ho, const float2* __restrict__ in, int wi, int hi,
                             int xoff, int yoff) {
  int xo = blockIdx.x * blockDim.x + threadIdx.x, yo = blockIdx.y;
  if (xo >= wo || yo >= ho) return;
  int xs = paste_src(xo, xoff, wi, wo), ys = paste_src(yo, yoff, hi, ho);
  float2 v = make_float2(0.f, 0.f);
  if (xs >= 0 && ys >= 0) v = in[(size_t)ys * wi + xs];
  out[(size_t)yo * wo + xo] = v;
}

// ---- host wrappers ------------------------------------------------------------------------
int vec_add(fsim_vec* y, const fsim_vec* x) {
  Ctx& c = ctx();
  k_add<<<grid_for(y->floats() / 4 + 1, 256), 256, 0, c.stream>>>(y->d, x->d, y->floats());
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

}  // namespace fsim

using namespace fsim;

#define NEED_INIT()                \
  do {                             \
    int rc_ = ensure_init();       \
    if (rc_) return rc_;           \
  } while (0)
#define NEED_VEC(v) FSIM_REQUIRE((v) && (v)->d, FSIM_EINVAL, "null vector")
#define SAME_SIZE(a, b) FSIM_REQUIRE((a)->n == (b)->n, FSIM_EINVAL, "vector size mismatch %zu != %zu", (a)->n, (b)->n)

extern "C" {

int fsim_vec_create(fsim_vec** out, int w, int h, int is_complex) {
  NEED_INIT();
  FSIM_REQUIRE(out && w > 0 && h > 0, FSIM_EINVAL, "fsim_vec_create: bad size %d x %d", w, h);
  fsim_vec* v = new fsim_vec();
  v->w = w;
  v->h = h;
  v->cplx = is_complex ? 1 : 0;
  v->n = (size_t)w * h;
  size_t bytes = v->floats() * sizeof(float);
  cudaError_t e = fsim::dev_alloc(&v->d, bytes);
  if (e != cudaSuccess) {
    delete v;
    set_error("fsim_vec_create: device allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
    return FSIM_EOOM;
  }
  FSIM_CUDA(cudaMemsetAsync(v->d, 0, bytes, ctx().stream));
  *out = v;
  return FSIM_OK;
}

int fsim_vec_destroy(fsim_vec* v) {
  if (!v) return FSIM_OK;
  if (v->d) {
    cudaStreamSynchronize(ctx().stream);
    cudaFree(v->d);
  }
  delete v;
  return FSIM_OK;
}

int fsim_vec_info(const fsim_vec* v, int* w, int* h, int* is_complex, void** device_ptr) {
  NEED_VEC(v);
  if (w) *w = v->w;
  if (h) *h = v->h;
  if (is_complex) *is_complex = v->cplx;
  if (device_ptr) *device_ptr = v->d;
  return FSIM_OK;
}

int fsim_vec_reshape(fsim_vec* v, int w, int h) {
  NEED_VEC(v);
  FSIM_REQUIRE(w > 0 && h > 0 && (size_t)w * h == v->n, FSIM_EINVAL,
               "fsim_vec_reshape: %d x %d does not hold %zu elements", w, h, v->n);
  v->w = w;
  v->h = h;
  return FSIM_OK;
}

int fsim_vec_set_elem(fsim_vec* v, size_t index, float re, float im) {
  NEED_INIT();
  NEED_VEC(v);
  FSIM_REQUIRE(index < v->n, FSIM_EINVAL, "fsim_vec_set_elem: index %zu of %zu", index, v->n);
  const float val[2] = {re, im};
  // ordered after earlier work on the vector; the value is copied before the call returns
  FSIM_CUDA(cudaMemcpyAsync(v->d + (v->cplx ? 2 * index : index), val, (v->cplx ? 2 : 1) * sizeof(float),
                            cudaMemcpyHostToDevice, ctx().stream));
  FSIM_CUDA(cudaStreamSynchronize(ctx().stream));
  return FSIM_OK;
}

int fsim_vec_get_elem(const fsim_vec* v, size_t index, float* re, float* im) {
  NEED_INIT();
  NEED_VEC(v);
  FSIM_REQUIRE(index < v->n && re, FSIM_EINVAL, "fsim_vec_get_elem: index %zu of %zu", index, v->n);
  float val[2] = {0.f, 0.f};
  FSIM_CUDA(cudaMemcpyAsync(val, v->d + (v->cplx ? 2 * index : index), (v->cplx ? 2 : 1) * sizeof(float),
                            cudaMemcpyDeviceToHost, ctx().stream));
  FSIM_CUDA(cudaStreamSynchronize(ctx().stream));
  *re = val[0];
  if (im) *im = val[1];
  return FSIM_OK;
}

int fsim_vec_upload(fsim_vec* v, const float* host) {
  NEED_INIT();
  NEED_VEC(v);
  FSIM_CUDA(cudaMemcpyAsync(v->d, host, v->floats() * sizeof(float), cudaMemcpyHostToDevice, ctx().stream));
  FSIM_CUDA(cudaStreamSynchronize(ctx().stream));
  return FSIM_OK;
}

int fsim_vec_download(const fsim_vec* v, float* host) {
  NEED_INIT();
  NEED_VEC(v);
  FSIM_CUDA(cudaMemcpyAsync(host, v->d, v->floats() * sizeof(float), cudaMemcpyDeviceToHost, ctx().stream));
  FSIM_CUDA(cudaStreamSynchronize(ctx().stream));
  return FSIM_OK;
}

int fsim_vec_upload_u16(fsim_vec* v, const uint16_t* host) {
  NEED_INIT();
  NEED_VEC(v);
  Ctx& c = ctx();
  uint16_t* tmp = nullptr;
  FSIM_CUDA(fsim::dev_alloc_async(&tmp, v->n * sizeof(uint16_t), c.stream));
  FSIM_CUDA(cudaMemcpyAsync(tmp, host, v->n * sizeof(uint16_t), cudaMemcpyHostToDevice, c.stream));
  if (v->cplx)
    k_u16_to_c<<<grid_for(v->n, 256), 256, 0, c.stream>>>(reinterpret_cast<float2*>(v->d), tmp, v->n);
  else
    k_u16_to_r<<<grid_for(v->n, 256), 256, 0, c.stream>>>(v->d, tmp, v->n);
  FSIM_CHECK_LAUNCH();
  FSIM_CUDA(cudaFreeAsync(tmp, c.stream));
  FSIM_CUDA(cudaStreamSynchronize(c.stream));
  return FSIM_OK;
}

int fsim_vec_zero(fsim_vec* y) {
  NEED_INIT();
  NEED_VEC(y);
  FSIM_CUDA(cudaMemsetAsync(y->d, 0, y->floats() * sizeof(float), ctx().stream));
  return FSIM_OK;
}

int fsim_vec_add(fsim_vec* y, const fsim_vec* x) {
  NEED_INIT();
  NEED_VEC(y);
  NEED_VEC(x);
  SAME_SIZE(y, x);
  FSIM_REQUIRE(y->cplx == x->cplx, FSIM_EINVAL, "add: real/complex mismatch");
  return vec_add(y, x);
}

int fsim_vec_addconst(fsim_vec* y, float re, float im) {
  NEED_INIT();
  NEED_VEC(y);
  Ctx& c = ctx();
  if (y->cplx)
    k_addconst_c<<<grid_for(y->n, 256), 256, 0, c.stream>>>(reinterpret_cast<float2*>(y->d), y->n, re, im);
  else
    k_addconst_r<<<grid_for(y->n, 256), 256, 0, c.stream>>>(y->d, y->n, re);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int fsim_vec_axpy(fsim_vec* y, float re, float im, const fsim_vec* x) {
  NEED_INIT();
  NEED_VEC(y);
  NEED_VEC(x);
  SAME_SIZE(y, x);
  FSIM_REQUIRE(y->cplx == x->cplx, FSIM_EINVAL, "axpy: real/complex mismatch");
  Ctx& c = ctx();
  if (y->cplx)
    k_axpy_c<<<grid_for(y->n, 256), 256, 0, c.stream>>>(reinterpret_cast<float2*>(y->d),
                                                         reinterpret_cast<const float2*>(x->d), y->n, re, im);
  else
    k_axpy_r<<<grid_for(y->n, 256), 256, 0, c.stream>>>(y->d, x->d, y->n, re);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int fsim_vec_times(fsim_vec* y, const fsim_vec* x, int conj) {
  NEED_INIT();
  NEED_VEC(y);
  NEED_VEC(x);
  SAME_SIZE(y, x);
  Ctx& c = ctx();
  if (y->cplx && x->cplx)
    k_times_cc<<<grid_for(y->n, 256), 256, 0, c.stream>>>(reinterpret_cast<float2*>(y->d),
                                                           reinterpret_cast<const float2*>(x->d), y->n, conj);
  else if (y->cplx)
    k_times_cr<<<grid_for(y->n, 256), 256, 0, c.stream>>>(reinterpret_cast<float2*>(y->d), x->d, y->n);
  else if (!x->cplx)
    k_times_rr<<<grid_for(y->n, 256), 256, 0, c.stream>>>(y->d, x->d, y->n);
  else
    FSIM_REQUIRE(false, FSIM_EINVAL, "times: real vector times complex vector is not defined");
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int fsim_vec_scal(fsim_vec* y, float re, float im) {
  NEED_INIT();
  NEED_VEC(y);
  Ctx& c = ctx();
  if (y->cplx)
    k_scal_c<<<grid_for(y->n, 256), 256, 0, c.stream>>>(reinterpret_cast<float2*>(y->d), y->n, re, im);
  else
    k_scal_r<<<grid_for(y->n, 256), 256, 0, c.stream>>>(y->d, y->n, re);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int fsim_vec_copy(fsim_vec* y, const fsim_vec* x) {
  NEED_INIT();
  NEED_VEC(y);
  NEED_VEC(x);
  SAME_SIZE(y, x);
  Ctx& c = ctx();
  if (y->cplx == x->cplx) {
    FSIM_CUDA(cudaMemcpyAsync(y->d, x->d, y->floats() * sizeof(float), cudaMemcpyDeviceToDevice, c.stream));
  } else if (y->cplx) {
    k_real_to_c<<<grid_for(y->n, 256), 256, 0, c.stream>>>(reinterpret_cast<float2*>(y->d), x->d, y->n);
  } else {
    k_c_to_real<<<grid_for(y->n, 256), 256, 0, c.stream>>>(y->d, reinterpret_cast<const float2*>(x->d), y->n);
  }
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int fsim_vec_reciproc(fsim_vec* y) {
  NEED_INIT();
  NEED_VEC(y);
  Ctx& c = ctx();
  if (y->cplx)
    k_reciproc_c<<<grid_for(y->n, 256), 256, 0, c.stream>>>(reinterpret_cast<float2*>(y->d), y->n);
  else
    k_reciproc_r<<<grid_for(y->n, 256), 256, 0, c.stream>>>(y->d, y->n);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int fsim_vec_norm2(const fsim_vec* x, double* out) {
  NEED_INIT();
  NEED_VEC(x);
  return reduce(0, x, nullptr, out, nullptr);
}

int fsim_vec_sum(const fsim_vec* x, double* re, double* im) {
  NEED_INIT();
  NEED_VEC(x);
  int rc = reduce(1, x, nullptr, re, im);
  if (!x->cplx && im) *im = 0;
  return rc;
}

int fsim_vec_dot(const fsim_vec* x, const fsim_vec* y, double* re, double* im) {
  NEED_INIT();
  NEED_VEC(x);
  NEED_VEC(y);
  SAME_SIZE(x, y);
  FSIM_REQUIRE(x->cplx && y->cplx, FSIM_EINVAL, "dot: complex vectors only");
  return reduce(2, x, y, re, im);
}

int fsim_vec_fourier_shift(fsim_vec* v, double kx, double ky) {
  NEED_INIT();
  NEED_VEC(v);
  FSIM_REQUIRE(v->cplx, FSIM_EINVAL, "fourierShift: complex vector required");
  FSIM_REQUIRE(v->w == v->h, FSIM_EINVAL, "Vector len mismatch %d %d", v->w, v->h);  // Vec2d.checkSquare
  dim3 g(div_up(v->w, 32), div_up(v->h, 8));
  k_fourier_shift<<<g, dim3(32, 8), 0, ctx().stream>>>(reinterpret_cast<float2*>(v->d), v->w, kx, ky);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int fsim_vec_paste_freq(fsim_vec* out, const fsim_vec* in, int x_off, int y_off) {
  NEED_INIT();
  NEED_VEC(out);
  NEED_VEC(in);
  FSIM_REQUIRE(out->cplx && in->cplx, FSIM_EINVAL, "pasteFreq: complex vectors required");
  FSIM_REQUIRE(out->w >= in->w && out->h >= in->h, FSIM_EINVAL, "pasteFreq: output smaller than input");
  dim3 g(div_up(out->w, 256), out->h);
  k_paste_freq<<<g, 256, 0, ctx().stream>>>(reinterpret_cast<float2*>(out->d), out->w, out->h,
                                            reinterpret_cast<const float2*>(in->d), in->w, in->h, x_off, y_off);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

}  // extern "C"
