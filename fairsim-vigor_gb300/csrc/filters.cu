// Per-pixel filter builders and band separation on device vectors:
// OtfProvider.otfToVector / writeApoVector / writeAttenuationVector / maskOtf,
// WienerFilter.getDenominator, BandSeparation.separateBands.
// These run once per parameter change (or once per op in the op-by-op path), so radii are
// computed in double exactly as the reference does.
#include <cmath>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "filters.cuh"
#include "otf.cuh"
#include "runtime.cuh"
#include "sim_host.h"

namespace fsim {

double ideal_otf_host(double d) {
  if (d < 0 || d > 1) return 0;
  return (2 / M_PI) * (std::acos(d) - d * std::sqrt(1 - d * d));
}

// OtfProvider.valAttenuation (java:234-236)
static float val_attenuation(double dist, double str, double fwhm) {
  return (float)(1 - str * std::exp(-(std::pow(dist, 2)) / (2 * std::pow(fwhm / 2.355, 2))));
}

void build_otf_table(const fsim_sim_param* p, OtfTable* t) {
  t->cutoff = 1000 / (p->em_wavelength / p->na / 2);
  t->cycles_per_sample = t->cutoff / OTF_SAMPLES;
  t->vec_cpm = 1 / (p->w * p->microns_per_pixel);
  t->measured = otf_measured(p) ? 1 : 0;
  t->multi_band = 0;
  t->n_bands = t->n_samples = 0;
  if (t->measured) {
    // loadFromConfig with band data, then setAttenuation per band (java:588-621, 276-287)
    t->cycles_per_sample = p->otf_cycles;
    t->n_bands = p->otf_bands;
    t->n_samples = p->otf_samples;
    t->multi_band = p->otf_bands > 1;
    for (int b = 0; b < t->n_bands; b++)
      for (int v = 0; v < t->n_samples; v++) {
        const float re = p->otf_data[2 * ((size_t)b * t->n_samples + v)];
        const float im = p->otf_data[2 * ((size_t)b * t->n_samples + v) + 1];
        const float a = val_attenuation(v * t->cycles_per_sample, p->att_strength, p->att_fwhm);
        t->mvals[b][v] = make_float2(re, im);
        t->monly_att[b][v] = a;
        t->mvals_att[b][v] = make_float2(re * a, im * a);
      }
  }
  for (int i = 0; i < OTF_SAMPLES; i++) {
    double v = i / (double)OTF_SAMPLES;
    t->vals[i] = (float)(ideal_otf_host(v) * std::pow(p->otf_a, v));
  }
  for (int v = 0; v < OTF_SAMPLES; v++) {
    double dist = v * t->cycles_per_sample;
    t->only_att[v] = (float)(1 - p->att_strength * std::exp(-(std::pow(dist, 2)) / (2 * std::pow(p->att_fwhm / 2.355, 2))));
    t->vals_att[v] = t->vals[v] * t->only_att[v];
  }
  auto split = [](double v, float* o) {
    o[0] = (float)v;
    o[1] = (float)(v - (double)o[0]);
  };
  split(t->vec_cpm, t->ff_cpm);
  split(t->vec_cpm / t->cycles_per_sample, t->ff_pos);
  split(t->cutoff, t->ff_cut);
}

// ---- kernels ------------------------------------------------------------------------
__global__ void k_otf_to_vector(float2* __restrict__ v, int w, int h, const OtfTable* __restrict__ t, int band,
                                double kx, double ky, int att, int write) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  size_t i = (size_t)y * w + x;
  if (t->measured) {
    float2 c;
    if (!otf_at_c(*t, band, (double)freq_x(x, w), (double)freq_y(y, h), kx, ky, att != 0, &c)) {
      v[i] = make_float2(0.f, 0.f);
    } else if (write) {
      v[i] = c;
    } else {  // Cplx.Float.mult(a, c.conj())
      const float2 a = v[i];
      const float cr = c.x, ci = -c.y;
      v[i] = make_float2(__fsub_rn(__fmul_rn(a.x, cr), __fmul_rn(a.y, ci)),
                         __fadd_rn(__fmul_rn(a.x, ci), __fmul_rn(a.y, cr)));
    }
    return;
  }
  float val;
  if (!otf_at(*t, (double)freq_x(x, w), (double)freq_y(y, h), kx, ky, att != 0, &val)) {
    v[i] = make_float2(0.f, 0.f);
  } else if (write) {
    v[i] = make_float2(val, 0.f);
  } else {
    float2 a = v[i];  // a * conj(val): im part of the OTF is zero for estimates
    v[i] = make_float2(__fmul_rn(a.x, val), __fmul_rn(a.y, val));
  }
}

__global__ void k_apo_vector(float* __restrict__ v, int cplx, int w, int h, double vec_cpm, double cutoff,
                             double bend) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  double rad = d_hypot_java((double)freq_x(x, w), (double)freq_y(y, h));
  double cycl = __dmul_rn(rad, vec_cpm);
  double frac = cycl / cutoff;
  float val = (float)pow(ideal_otf_dev(frac), bend);
  size_t i = (size_t)y * w + x;
  if (cplx)
    reinterpret_cast<float2*>(v)[i] = make_float2(val, 0.f);
  else
    v[i] = val;
}

__global__ void k_att_vector(float* __restrict__ v, int w, int h, double vec_cpm, double str, double fwhm, double kx,
                             double ky) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  double rad = d_hypot_java(__dsub_rn((double)freq_x(x, w), kx), __dsub_rn((double)freq_y(y, h), ky));
  double dist = __dmul_rn(rad, vec_cpm);
  const double s = fwhm / 2.355;  // Java's separate roundings (no FMA contraction)
  const double g = exp(-__dmul_rn(dist, dist) / __dmul_rn(2.0, __dmul_rn(s, s)));
  v[(size_t)y * w + x] = (float)__dsub_rn(1.0, __dmul_rn(str, g));
}

__global__ void k_mask_otf(float2* __restrict__ v, int w, int h, double vec_cpm, double cutoff, double kx, double ky) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  double rad = __dmul_rn(d_hypot_java(__dsub_rn((double)freq_x(x, w), kx), __dsub_rn((double)freq_y(y, h), ky)), vec_cpm);
  if (rad > cutoff) v[(size_t)y * w + x] = make_float2(0.f, 0.f);
}

// WienerFilter.updateCache + getDenominator (WienerFilter.java:46-122): in float, in the
// reference's accumulation order (directions outer, bands inner, +otf(r-k) then +otf(r+k)).
__global__ void k_wiener_denominator(float* __restrict__ out, int W, int H, const OtfTable* __restrict__ t,
                                     ShiftSet shifts, int use_att, float wp, int reciprocal) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= W) return;
  const double xh = freq_x(x, W), yh = freq_y(y, H);
  const double cpm = t->vec_cpm;
  float acc = 0.f;
  for (int d = 0; d < shifts.n_dirs; d++)
    for (int b = 0; b < shifts.n_bands; b++) {
      const double kx = shifts.px[d] * b, ky = shifts.py[d] * b;
      double r1 = __dmul_rn(d_hypot_java(__dsub_rn(xh, kx), __dsub_rn(yh, ky)), cpm);
      double r2 = __dmul_rn(d_hypot_java(__dadd_rn(xh, kx), __dadd_rn(yh, ky)), cpm);
      float v1, v2;
      if (t->measured) {  // Cplx.Float.absSq of the band's value
        v1 = abs_sq(otf_val_c(*t, b, r1, false));
        v2 = abs_sq(otf_val_c(*t, b, r2, false));
        if (use_att) {
          v1 = __fmul_rn(v1, att_val_b(*t, b, r1));
          v2 = __fmul_rn(v2, att_val_b(*t, b, r2));
        }
      } else {
        float o1 = otf_val(*t, r1, false), o2 = otf_val(*t, r2, false);
        v1 = __fmul_rn(o1, o1);
        v2 = __fmul_rn(o2, o2);
        if (use_att) {
          v1 = __fmul_rn(v1, att_val(*t, r1));
          v2 = __fmul_rn(v2, att_val(*t, r2));
        }
      }
      acc = __fadd_rn(__fadd_rn(acc, v1), v2);
    }
  out[(size_t)y * W + x] = reciprocal ? __fdiv_rn(1.f, __fadd_rn(acc, wp)) : acc;
}

// separateBands: out[b] = sum_p M[b][p] * in[p] with the reference's axpy rounding
// (L/AbstractVectorCplx.java:185-195); in/out are arrays of device pointers.
__global__ void k_separate(const SepArgs a, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float2 in[FSIM_MAX_PHASES];
    for (int p = 0; p < a.n_in; p++) in[p] = a.in[p][i];
    for (int b = 0; b < a.n_out; b++) {
      float re = 0.f, im = 0.f;
      for (int p = 0; p < a.n_in; p++) {
        const float2 c = a.coef[b * a.n_in + p];
        re = __fadd_rn(re, __fsub_rn(__fmul_rn(c.x, in[p].x), __fmul_rn(c.y, in[p].y)));
        im = __fadd_rn(im, __fadd_rn(__fmul_rn(c.y, in[p].x), __fmul_rn(c.x, in[p].y)));
      }
      a.out[b][i] = make_float2(re, im);
    }
  }
}

// ---- host helpers ------------------------------------------------------------------------
static std::mutex g_otf_mu;
std::mutex& otf_table_mutex() { return g_otf_mu; }

// The caller holds otf_table_mutex() from this call until the kernel that reads the table
// is enqueued: another thread's upload waits for the device before it overwrites the
// staging table, and only enqueued work is waited for.
int upload_otf_table(const fsim_sim_param* p, OtfTable** dev, cudaStream_t st) {
  Ctx& c = ctx();
  static OtfTable* buf = nullptr;
  static OtfTable* host = nullptr;
  static double key[7] = {0, 0, 0, 0, 0, 0, 0};
  if (!buf) FSIM_CUDA(fsim::dev_alloc(&buf, sizeof(OtfTable)));
  if (!host) FSIM_CUDA(cudaMallocHost(&host, sizeof(OtfTable)));
  const double k[7] = {p->na, p->em_wavelength, p->otf_a, p->att_strength, p->att_fwhm, (double)p->w,
                       p->microns_per_pixel};
  // estimates are cached by their parameters; measured tables (whose samples the key does
  // not cover) are rebuilt on every call and leave the cache invalid
  const bool measured = otf_measured(p);
  bool same = !measured;
  for (int i = 0; i < 7; i++) same = same && (k[i] == key[i]);
  if (!same) {
    // wait for the previous user of the staging copy before overwriting it
    FSIM_CUDA(cudaDeviceSynchronize());
    build_otf_table(p, host);
    FSIM_CUDA(cudaMemcpyAsync(buf, host, sizeof(OtfTable), cudaMemcpyHostToDevice, st ? st : c.stream));
    FSIM_CUDA(cudaStreamSynchronize(st ? st : c.stream));
    for (int i = 0; i < 7; i++) key[i] = measured ? std::nan("") : k[i];
  }
  *dev = buf;
  return FSIM_OK;
}

FShiftSet fshift_set(const ShiftSet& s) {
  FShiftSet f{};
  for (int d = 0; d < s.n_dirs && d < FSIM_MAX_DIRS; d++)
    for (int b = 0; b < s.n_bands && b < FSIM_MAX_BANDS; b++) f.k[d][b] = fshift_host(s.px[d] * b, s.py[d] * b);
  return f;
}

__global__ void k_apo_octant(float* __restrict__ q, int n, double vec_cpm, double cutoff_abs, double bend) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j > i) return;
  const double frac = __dmul_rn(d_hypot_java((double)i, (double)j), vec_cpm) / cutoff_abs;
  const double io = ideal_otf_dev(frac);
  q[(size_t)i * (n + 1) + j] = (float)(bend == 1.0 ? io : pow(io, bend));  // Math.pow(x, 1.0) is x
}

int apo_octant_device(float* q, int n, double vec_cpm, double cutoff_abs, double bend, cudaStream_t st) {
  k_apo_octant<<<dim3(div_up(n + 1, 128), n + 1), 128, 0, st>>>(q, n, vec_cpm, cutoff_abs, bend);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

ShiftSet shift_set(const fsim_sim_param* p) {
  ShiftSet s{};
  s.n_dirs = p->nr_dirs;
  s.n_bands = p->nr_bands;
  for (int d = 0; d < p->nr_dirs; d++) {
    s.px[d] = p->px[d];
    s.py[d] = p->py[d];
  }
  return s;
}

int wiener_denominator_device(float* out, const fsim_sim_param* p, double wiener, const OtfTable* t, bool reciprocal,
                              cudaStream_t st) {
  const int W = 2 * p->w;
  dim3 g(div_up(W, 128), W);
  k_wiener_denominator<<<g, 128, 0, st>>>(out, W, W, t, shift_set(p), p->use_attenuation, (float)(wiener * wiener),
                                          reciprocal ? 1 : 0);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int apo_device(float* out, int cplx, int W, int H, double vec_cpm, double cutoff_abs, double bend, cudaStream_t st) {
  dim3 g(div_up(W, 128), H);
  k_apo_vector<<<g, 128, 0, st>>>(out, cplx, W, H, vec_cpm, cutoff_abs, bend);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

// Unshifted on a square grid the attenuation depends on (|x~|, |y~|) only, symmetrically:
// evaluated in double once per octant point 0 <= j <= i <= n/2 (the same expression as
// k_att_vector, so the same bits) and spread over the grid.
__global__ void k_att_octant(float* __restrict__ q, int h2, double vec_cpm, double str, double fwhm) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j > i) return;
  const double rad = d_hypot_java((double)i, (double)j);
  const double dist = __dmul_rn(rad, vec_cpm);
  const double s = fwhm / 2.355;
  const double g = exp(-__dmul_rn(dist, dist) / __dmul_rn(2.0, __dmul_rn(s, s)));
  q[(size_t)i * (h2 + 1) + j] = (float)__dsub_rn(1.0, __dmul_rn(str, g));
}
__global__ void k_att_expand(float* __restrict__ v, int n, const float* __restrict__ q) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= n) return;
  const int ax = abs(freq_x(x, n)), ay = abs(freq_y(y, n));
  v[(size_t)y * n + x] = __ldg(q + (size_t)max(ax, ay) * (n / 2 + 1) + min(ax, ay));
}

int att_device(float* out, int w, int h, double vec_cpm, double str, double fwhm, double kx, double ky, cudaStream_t st) {
  dim3 g(div_up(w, 128), h);
  if (w == h && w % 2 == 0 && kx == 0 && ky == 0) {
    const int h2 = w / 2;
    float* q = nullptr;
    FSIM_CUDA(fsim::dev_alloc_async(&q, sizeof(float) * (size_t)(h2 + 1) * (h2 + 1), st));
    k_att_octant<<<dim3(div_up(h2 + 1, 128), h2 + 1), 128, 0, st>>>(q, h2, vec_cpm, str, fwhm);
    k_att_expand<<<g, 128, 0, st>>>(out, w, q);
    FSIM_CHECK_LAUNCH();
    FSIM_CUDA(cudaFreeAsync(q, st));
    return FSIM_OK;
  }
  k_att_vector<<<g, 128, 0, st>>>(out, w, h, vec_cpm, str, fwhm, kx, ky);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int otf_vector_device(float2* v, int w, int h, const OtfTable* t, int band, double kx, double ky, bool att, bool write,
                      cudaStream_t st) {
  dim3 g(div_up(w, 128), h);
  k_otf_to_vector<<<g, 128, 0, st>>>(v, w, h, t, band, kx, ky, att ? 1 : 0, write ? 1 : 0);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int separate_device(const SepArgs& a, size_t n, cudaStream_t st) {
  int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)ctx().num_sms * 8);
  k_separate<<<blocks, 256, 0, st>>>(a, n);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

}  // namespace fsim

using namespace fsim;

#define NEED_INIT()          \
  do {                       \
    int rc_ = ensure_init(); \
    if (rc_) return rc_;     \
  } while (0)

extern "C" {

int fsim_otf_to_vector(fsim_vec* v, const fsim_sim_param* p, int band, double kx, double ky, int use_att, int write) {
  NEED_INIT();
  // band: a measured multi-band table's band; an estimated (single-band) OTF ignores it
  // (OtfProvider.java:191-192)
  FSIM_REQUIRE(v && v->cplx, FSIM_EINVAL, "otfToVector: complex vector required");
  int rc = validate_param(p);
  if (rc) return rc;
  // getOtfVal's check (OtfProvider.java:191-194): a multi-band measured table indexes its
  // bands with `band`, so it must name one of them; other tables collapse it to band 0
  FSIM_REQUIRE(!(otf_measured(p) && p->otf_bands > 1) || (band >= 0 && band < p->otf_bands), FSIM_EINVAL,
               "otfToVector: band idx too high or <0 (%d of %d bands)", band, p->otf_bands);
  OtfTable* t;
  std::lock_guard<std::mutex> g(otf_table_mutex());
  rc = upload_otf_table(p, &t, ctx().stream);
  if (rc) return rc;
  return otf_vector_device(reinterpret_cast<float2*>(v->d), v->w, v->h, t, band, kx, ky, use_att != 0, write != 0,
                           ctx().stream);
}

int fsim_apo_vector(fsim_vec* v, const fsim_sim_param* p, double bend, double cutoff) {
  NEED_INIT();
  FSIM_REQUIRE(v, FSIM_EINVAL, "null vector");
  int rc = validate_param(p);
  if (rc) return rc;
  double cut = 1000 / (p->em_wavelength / p->na / 2);
  return apo_device(v->d, v->cplx, v->w, v->h, 1 / (p->w * p->microns_per_pixel), cut * cutoff, bend, ctx().stream);
}

int fsim_attenuation_vector(fsim_vec* v, const fsim_sim_param* p, double str, double fwhm, double kx, double ky) {
  NEED_INIT();
  FSIM_REQUIRE(v && !v->cplx, FSIM_EINVAL, "attenuation vector must be real");
  int rc = validate_param(p);
  if (rc) return rc;
  return att_device(v->d, v->w, v->h, 1 / (p->w * p->microns_per_pixel), str, fwhm, kx, ky, ctx().stream);
}

int fsim_mask_otf(fsim_vec* v, const fsim_sim_param* p, double kx, double ky) {
  NEED_INIT();
  FSIM_REQUIRE(v && v->cplx, FSIM_EINVAL, "maskOtf: complex vector required");
  int rc = validate_param(p);
  if (rc) return rc;
  double cut = 1000 / (p->em_wavelength / p->na / 2);
  dim3 g(div_up(v->w, 128), v->h);
  k_mask_otf<<<g, 128, 0, ctx().stream>>>(reinterpret_cast<float2*>(v->d), v->w, v->h,
                                          1 / (p->w * p->microns_per_pixel), cut, kx, ky);
  FSIM_CHECK_LAUNCH();
  return FSIM_OK;
}

int fsim_wiener_denominator(fsim_vec* out, const fsim_sim_param* p, double wiener) {
  NEED_INIT();
  int rc = validate_param(p);
  if (rc) return rc;
  FSIM_REQUIRE(out && !out->cplx && out->w == 2 * p->w && out->h == 2 * p->w, FSIM_EINVAL,
               "Wiener denominator: real 2w x 2w vector required");
  OtfTable* t;
  std::lock_guard<std::mutex> g(otf_table_mutex());
  rc = upload_otf_table(p, &t, ctx().stream);
  if (rc) return rc;
  return wiener_denominator_device(out->d, p, wiener, t, true, ctx().stream);
}

int fsim_separate_bands(fsim_vec* const* in, int n_in, fsim_vec* const* out, int n_out, const double* phases,
                        int bands, const double* fac) {
  NEED_INIT();
  FSIM_REQUIRE(in && out && phases && n_in > 0 && n_in <= FSIM_MAX_PHASES, FSIM_EINVAL, "separateBands: bad arguments");
  FSIM_REQUIRE(n_out == 2 * bands - 1, FSIM_EINVAL, "#output images != #bands*2-1");
  FSIM_REQUIRE(n_in >= 2 * bands - 1, FSIM_EINVAL, "not enough phases for #bands");
  for (int i = 0; i < n_in; i++)
    FSIM_REQUIRE(in[i] && in[i]->cplx && in[i]->n == in[0]->n, FSIM_EINVAL, "separateBands: input size mismatch");
  for (int i = 0; i < n_out; i++)
    FSIM_REQUIRE(out[i] && out[i]->cplx && out[i]->n == in[0]->n, FSIM_EINVAL, "separateBands: output size mismatch");
  std::vector<double> ph(phases, phases + n_in), f;
  if (fac) f.assign(fac, fac + bands);
  std::vector<cd> m = separation_matrix(ph, bands, f);
  SepArgs a{};
  a.n_in = n_in;
  a.n_out = n_out;
  for (int i = 0; i < n_in; i++) a.in[i] = reinterpret_cast<const float2*>(in[i]->d);
  for (int i = 0; i < n_out; i++) a.out[i] = reinterpret_cast<float2*>(out[i]->d);
  for (int b = 0; b < n_out; b++)
    for (int p = 0; p < n_in; p++)
      a.coef[b * n_in + p] = make_float2((float)m[b * n_in + p].real(), (float)m[b * n_in + p].imag());
  return separate_device(a, in[0]->n, ctx().stream);
}

}  // extern "C"
