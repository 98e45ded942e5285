// ORACLE — test infrastructure only (see refcpu.hpp). Flat C entry points over the
// templated restatement so that Python tests (ctypes) and bench.py's CPU-baseline leg can
// call it. Every function returns 0 on success, -1 on a reference-style exception (the
// message is available from ref_last_error()).
#include <cstdio>
#include <string>

#include "refcpu.hpp"

extern "C" {

#define REF_MAXD 8
#define REF_MAXB 4
#define REF_MAXP 16

typedef struct {
  int w;  // raw image width (= height)
  int nrDirs, nrBands, nrPhases;
  double micronsPerPixel;
  double na, lambda, otfA;  // OtfProvider.fromEstimate
  int useAtt;
  double attStr, attFWHM;
  double wiener, apoCutoff, apoBend;
  double pX[REF_MAXD], pY[REF_MAXD], phaOff[REF_MAXD];
  double modul[REF_MAXD][REF_MAXB];
  int hasPhases;
  double phases[REF_MAXD][REF_MAXP];
  int filterStyle;   // SimParam.FilterStyle ordinal
  int rlIterations;
  const float* otfData;  // measured OTF: otfBands x otfSamples complex (re, im); NULL = estimate
  int otfBands, otfSamples;
  double otfCycles;
} ref_param;
}

static thread_local std::string g_err;

template <class T>
static ref::SimParam<T> make_param(const ref_param* p) {
  ref::SimParam<T> sp;
  sp.nrDirs = p->nrDirs;
  sp.nrBands = p->nrBands;
  sp.nrPhases = p->nrPhases;
  sp.wiener = p->wiener;
  sp.apoCutOff = p->apoCutoff;
  sp.filterStyle = p->filterStyle;
  sp.rlIterations = p->rlIterations;
  sp.otf = (p->otfData && p->otfSamples > 0)
               ? ref::Otf<T>::fromData(p->na, p->lambda, p->otfBands, p->otfSamples, p->otfCycles, p->otfData)
               : ref::Otf<T>::fromEstimate(p->na, p->lambda, p->otfA);
  sp.otf.setAttenuation(p->attStr, p->attFWHM);
  sp.otf.useAtt = p->useAtt != 0;
  sp.setPxlSize(p->w, p->micronsPerPixel);
  sp.dirs.clear();
  for (int d = 0; d < p->nrDirs; d++) {
    ref::Dir dir(p->nrBands, p->nrPhases);
    dir.pX = p->pX[d];
    dir.pY = p->pY[d];
    dir.phaOff = p->phaOff[d];
    for (int b = 0; b < p->nrBands; b++) dir.modul[b] = p->modul[d][b];
    if (p->hasPhases)
      for (int i = 0; i < p->nrPhases; i++) dir.phases[i] = p->phases[d][i];
    sp.dirs.push_back(dir);
  }
  return sp;
}
template <class T>
static void store_param(const ref::SimParam<T>& sp, ref_param* p) {
  for (int d = 0; d < sp.nrDirs; d++) {
    p->pX[d] = sp.dirs[d].pX;
    p->pY[d] = sp.dirs[d].pY;
    p->phaOff[d] = sp.dirs[d].phaOff;
    for (int b = 0; b < sp.nrBands; b++) p->modul[d][b] = sp.dirs[d].modul[b];
  }
}

template <class T>
static std::vector<std::vector<ref::CVec<T>>> load_spectra(const ref_param* p, const T* in) {
  const int w = p->w;
  std::vector<std::vector<ref::CVec<T>>> v(p->nrDirs, std::vector<ref::CVec<T>>(p->nrPhases, ref::CVec<T>(w, w)));
  size_t n = (size_t)2 * w * w;
  for (int a = 0; a < p->nrDirs; a++)
    for (int ph = 0; ph < p->nrPhases; ph++)
      std::copy(in + n * (a * p->nrPhases + ph), in + n * (a * p->nrPhases + ph + 1), v[a][ph].d.begin());
  return v;
}

// GUI input preparation (org/fairsim/sim_gui/ImageControl.java:819-836): optional
// background subtraction (SimUtils.subtractBackground), fadeBorderCos(10), forward FFT.
template <class T>
static std::vector<std::vector<ref::CVec<T>>> prepare_raw(const ref_param* p, const T* raw, double bgr, int fade) {
  const int w = p->w;
  std::vector<std::vector<ref::CVec<T>>> v(p->nrDirs, std::vector<ref::CVec<T>>(p->nrPhases, ref::CVec<T>(w, w)));
  size_t n = (size_t)w * w;
  for (int a = 0; a < p->nrDirs; a++)
    for (int ph = 0; ph < p->nrPhases; ph++) {
      ref::RVec<T> img(w, w);
      std::copy(raw + n * (a * p->nrPhases + ph), raw + n * (a * p->nrPhases + ph + 1), img.d.begin());
      if (bgr != 0) {
        for (auto& x : img.d) {
          x -= (T)bgr;
          if (x < 0) x = 0;
        }
      }
      if (fade > 0) ref::fade_border_cos(img, fade);
      ref::CVec<T>& c = v[a][ph];
      for (size_t i = 0; i < n; i++) {
        c.d[2 * i] = img.d[i];
        c.d[2 * i + 1] = 0;
      }
      ref::fft2d(c, false);
    }
  return v;
}

#define GUARD(...)               \
  try {                          \
    __VA_ARGS__;                 \
    return 0;                    \
  } catch (std::exception & e) { \
    g_err = e.what();            \
    return -1;                   \
  }

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }
int ref_set_threads(int n) {
  ref::Pool::get().set_threads(n);
  return ref::Pool::get().threads();
}
double ref_fsin(double x) { return ref::fsin(x); }
double ref_fcos(double x) { return ref::fcos(x); }

#define FFT_API(SUF, T)                                         \
  int ref_fft2d_##SUF(T* d, int w, int h, int inverse) {        \
    GUARD({                                                     \
      ref::CVec<T> v(w, h);                                     \
      std::copy(d, d + (size_t)2 * w * h, v.d.begin());         \
      ref::fft2d(v, inverse != 0);                              \
      std::copy(v.d.begin(), v.d.end(), d);                     \
    })                                                          \
  }                                                             \
  int ref_fourier_shift_##SUF(T* d, int n, double kx, double ky) { \
    GUARD({                                                     \
      ref::CVec<T> v(n, n);                                     \
      std::copy(d, d + (size_t)2 * n * n, v.d.begin());         \
      ref::fourier_shift(v, kx, ky);                            \
      std::copy(v.d.begin(), v.d.end(), d);                     \
    })                                                          \
  }                                                             \
  int ref_paste_freq_##SUF(T* out, int wo, int ho, const T* in, int wi, int hi, int xo, int yo) { \
    GUARD({                                                     \
      ref::CVec<T> o(wo, ho), i(wi, hi);                        \
      std::copy(in, in + (size_t)2 * wi * hi, i.d.begin());     \
      ref::paste_freq(o, i, xo, yo);                            \
      std::copy(o.d.begin(), o.d.end(), out);                   \
    })                                                          \
  }

FFT_API(f32, float)
FFT_API(f64, double)

// Inverse separation matrix (nC x nP, complex double, row-major) for the given phases
// of band 1 (higher bands use multiples) and raw modulations (clamped here as
// SimParam.Dir.getModulations does); fac==NULL reproduces the estimation call.
int ref_separation_matrix(const double* phases, int nPhases, int bands, const double* modul, double* out) {
  GUARD({
    std::vector<std::vector<double>> pha(bands - 1, std::vector<double>(nPhases));
    for (int b = 1; b < bands; b++)
      for (int p = 0; p < nPhases; p++) pha[b - 1][p] = phases[p] * b;
    std::vector<double> fac;
    if (modul) {
      fac.assign(modul, modul + bands);
      for (auto& m : fac) {
        if (m < 0.3) m = 0.3;
        if (m > 1.1) m = 1.1;
      }
    }
    ref::Mat M = ref::separation_matrix(pha, bands, fac);
    for (int i = 0; i < M.m; i++)
      for (int j = 0; j < M.n; j++) {
        out[2 * (i * M.n + j)] = M(i, j).re;
        out[2 * (i * M.n + j) + 1] = M(i, j).im;
      }
  })
}

int ref_matrix_inverse(const double* in, int n, double* out, int pseudo, int m) {
  GUARD({
    int rows = pseudo ? m : n;
    ref::Mat A(rows, n);
    for (int i = 0; i < rows; i++)
      for (int j = 0; j < n; j++) A(i, j) = {in[2 * (i * n + j)], in[2 * (i * n + j) + 1]};
    ref::Mat R = pseudo ? ref::mat_pseudo_inverse(A) : ref::mat_inverse(A);
    for (int i = 0; i < R.m; i++)
      for (int j = 0; j < R.n; j++) {
        out[2 * (i * R.n + j)] = R(i, j).re;
        out[2 * (i * R.n + j) + 1] = R(i, j).im;
      }
  })
}

#define SIM_API(SUF, T)                                                                               \
  int ref_separate_bands_##SUF(const ref_param* p, int dir, const T* inFFT, T* out) {                 \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      const int w = p->w;                                                                             \
      size_t n = (size_t)2 * w * w;                                                                   \
      std::vector<ref::CVec<T>> in(p->nrPhases, ref::CVec<T>(w, w));                                  \
      for (int i = 0; i < p->nrPhases; i++) std::copy(inFFT + n * i, inFFT + n * (i + 1), in[i].d.begin()); \
      int nc = 2 * p->nrBands - 1;                                                                    \
      std::vector<ref::CVec<T>> o(nc, ref::CVec<T>(w, w));                                            \
      ref::separate_bands(in, o, sp.dirs[dir].getPhases(), p->nrBands, sp.dirs[dir].getModulations()); \
      for (int i = 0; i < nc; i++) std::copy(o[i].d.begin(), o[i].d.end(), out + n * i);               \
    })                                                                                                \
  }                                                                                                   \
  /* which: 0 writeOtfVector, 1 writeOtfWithAttVector, 2 applyOtf (multiply), 3 maskOtf */            \
  int ref_otf_vector_##SUF(const ref_param* p, T* vec, int vw, int vh, double kx, double ky, int which,  \
                           int band) {                                                                \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      ref::CVec<T> v(vw, vh);                                                                         \
      std::copy(vec, vec + (size_t)2 * vw * vh, v.d.begin());                                         \
      if (which == 0) sp.otf.writeOtfVector(v, band, kx, ky);                                         \
      if (which == 1) sp.otf.writeOtfWithAttVector(v, band, kx, ky);                                  \
      if (which == 2) sp.otf.applyOtf(v, band, kx, ky);                                               \
      if (which == 3) sp.otf.maskOtf(v, kx, ky);                                                      \
      std::copy(v.d.begin(), v.d.end(), vec);                                                         \
    })                                                                                                \
  }                                                                                                   \
  int ref_apo_vector_##SUF(const ref_param* p, T* vec, int vw, int vh, double bend, double cutoff) {  \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      ref::RVec<T> v(vw, vh);                                                                         \
      sp.otf.writeApoVector(v, bend, cutoff);                                                         \
      std::copy(v.d.begin(), v.d.end(), vec);                                                         \
    })                                                                                                \
  }                                                                                                   \
  int ref_attenuation_vector_##SUF(const ref_param* p, T* vec, int vw, int vh, double str, double fwhm, \
                                   double kx, double ky) {                                            \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      ref::RVec<T> v(vw, vh);                                                                         \
      sp.otf.writeAttenuationVector(v, str, fwhm, kx, ky);                                            \
      std::copy(v.d.begin(), v.d.end(), vec);                                                         \
    })                                                                                                \
  }                                                                                                   \
  int ref_wiener_denominator_##SUF(const ref_param* p, T* out) {                                      \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      ref::RVec<T> v = ref::wiener_denominator(sp, p->wiener);                                        \
      std::copy(v.d.begin(), v.d.end(), out);                                                         \
    })                                                                                                \
  }                                                                                                   \
  int ref_recon_##SUF(const ref_param* p, const T* inFFT, int otfBeforeShift, int clipScale, T* out) { \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      auto in = load_spectra<T>(p, inFFT);                                                            \
      ref::RVec<T> r = ref::run_reconstruction(sp, in, otfBeforeShift != 0, clipScale, p->apoBend);   \
      std::copy(r.d.begin(), r.d.end(), out);                                                         \
    })                                                                                                \
  }                                                                                                   \
  int ref_prepare_raw_##SUF(const ref_param* p, const T* raw, double bgr, int fade, T* outFFT) {      \
    GUARD({                                                                                           \
      auto v = prepare_raw<T>(p, raw, bgr, fade);                                                     \
      size_t n = (size_t)2 * p->w * p->w;                                                             \
      for (int a = 0; a < p->nrDirs; a++)                                                             \
        for (int ph = 0; ph < p->nrPhases; ph++)                                                      \
          std::copy(v[a][ph].d.begin(), v[a][ph].d.end(), outFFT + n * (a * p->nrPhases + ph));       \
    })                                                                                                \
  }                                                                                                   \
  int ref_recon_raw_##SUF(const ref_param* p, const T* raw, double bgr, int fade, int clipScale, T* out) { \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      auto in = prepare_raw<T>(p, raw, bgr, fade);                                                    \
      ref::RVec<T> r = ref::run_reconstruction(sp, in, false, clipScale, p->apoBend);                 \
      std::copy(r.d.begin(), r.d.end(), out);                                                         \
    })                                                                                                \
  }                                                                                                   \
  int ref_rl_deconvolve_##SUF(T* img, const T* otf, int w, int h, int steps, int inFreq) {                \
    GUARD({                                                                                           \
      ref::CVec<T> v(w, h), o(w, h);                                                                  \
      std::copy(img, img + (size_t)2 * w * h, v.d.begin());                                           \
      std::copy(otf, otf + (size_t)2 * w * h, o.d.begin());                                           \
      ref::rl_deconvolve(v, o, steps, inFreq != 0);                                                   \
      std::copy(v.d.begin(), v.d.end(), img);                                                         \
    })                                                                                                \
  }                                                                                                   \
  int ref_auto_correlation_##SUF(const T* band, int w, double kx, double ky, double* out2) {         \
    GUARD({                                                                                           \
      ref::CVec<T> v(w, w);                                                                           \
      std::copy(band, band + (size_t)2 * w * w, v.d.begin());                                         \
      ref::C<double> r = ref::auto_correlation(v, kx, ky);                                            \
      out2[0] = r.re;                                                                                 \
      out2[1] = r.im;                                                                                 \
    })                                                                                                \
  }                                                                                                   \
  int ref_widefield_raw_##SUF(const ref_param* p, const T* raw, double bgr, int fade, int clipScale,   \
                              T* wf, T* fwf) {                                                        \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      auto in = prepare_raw<T>(p, raw, bgr, fade);                                                    \
      ref::RVec<T> a, b;                                                                              \
      ref::widefield_outputs(sp, in, clipScale, a, b);                                                \
      std::copy(a.d.begin(), a.d.end(), wf);                                                          \
      std::copy(b.d.begin(), b.d.end(), fwf);                                                         \
    })                                                                                                \
  }                                                                                                   \
  int ref_estimate_##SUF(ref_param* p, const T* inFFT, int fitBand, double fitExclude, double* peaks, \
                         double* coarse) {                                                            \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      auto in = load_spectra<T>(p, inFFT);                                                            \
      ref::estimate_parameters(sp, in, fitBand, fitExclude, peaks, coarse);                           \
      store_param(sp, p);                                                                             \
    })                                                                                                \
  }                                                                                                   \
  int ref_common_region_##SUF(const ref_param* p, T* b0, T* b1, double kx, double ky, double dist,   \
                              double wl, int divide) {                                                \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      const int w = p->w;                                                                             \
      ref::CVec<T> v0(w, w), v1(w, w);                                                                \
      std::copy(b0, b0 + (size_t)2 * w * w, v0.d.begin());                                           \
      std::copy(b1, b1 + (size_t)2 * w * w, v1.d.begin());                                            \
      ref::common_region(v0, v1, 0, 1, sp.otf, kx, ky, dist, wl, divide != 0);                              \
      std::copy(v0.d.begin(), v0.d.end(), b0);                                                        \
      std::copy(v1.d.begin(), v1.d.end(), b1);                                                        \
    })                                                                                                \
  }                                                                                                   \
  int ref_locate_peak_##SUF(const T* vec, int w, int h, double kMin, double* out4) {                  \
    GUARD({                                                                                           \
      ref::CVec<T> v(w, h);                                                                           \
      std::copy(vec, vec + (size_t)2 * w * h, v.d.begin());                                           \
      ref::locate_peak(v, kMin, out4);                                                                \
    })                                                                                                \
  }                                                                                                   \
  int ref_fit_peak_##SUF(const ref_param* p, const T* band0, const T* band1, double kx, double ky,    \
                         double wl, double search, double* out4, double* grid) {                      \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      const int w = p->w;                                                                             \
      ref::CVec<T> v0(w, w), v1(w, w);                                                                \
      std::copy(band0, band0 + (size_t)2 * w * w, v0.d.begin());                                      \
      std::copy(band1, band1 + (size_t)2 * w * w, v1.d.begin());                                      \
      ref::fit_peak(v0, v1, 0, 1, sp.otf, kx, ky, wl, search, out4, grid);                                  \
    })                                                                                                \
  }                                                                                                   \
  int ref_get_peak_##SUF(const ref_param* p, const T* band0, const T* band1, double kx, double ky,    \
                         double wl, double* out2) {                                                   \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      const int w = p->w;                                                                             \
      ref::CVec<T> v0(w, w), v1(w, w);                                                                \
      std::copy(band0, band0 + (size_t)2 * w * w, v0.d.begin());                                      \
      std::copy(band1, band1 + (size_t)2 * w * w, v1.d.begin());                                      \
      ref::C<double> r = ref::get_peak(v0, v1, 0, 1, sp.otf, kx, ky, wl);                                   \
      out2[0] = r.re;                                                                                 \
      out2[1] = r.im;                                                                                 \
    })                                                                                                \
  }                                                                                                   \
  int ref_live_recon_##SUF(const ref_param* p, const uint16_t* raw, int nStacks, T* out, T* widefield) { \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      auto f = ref::live_setup_filters(sp, p->useAtt != 0, p->attStr, p->attFWHM, p->wiener);         \
      const int w = p->w;                                                                             \
      size_t nraw = (size_t)w * w * p->nrDirs * p->nrPhases;                                          \
      for (int s = 0; s < nStacks; s++)                                                               \
        ref::live_reconstruct(sp, f, raw + nraw * s, out ? out + (size_t)4 * w * w * s : nullptr,     \
                              widefield ? widefield + (size_t)w * w * s : nullptr);                   \
    })                                                                                                \
  }                                                                                                   \
  int ref_live_refit_##SUF(ref_param* p, const uint16_t* raw, double* peaks) {                        \
    GUARD({                                                                                           \
      ref::SimParam<T> sp = make_param<T>(p);                                                         \
      ref::live_refit(sp, raw, peaks);                                                                \
      store_param(sp, p);                                                                             \
    })                                                                                                \
  }

SIM_API(f32, float)
SIM_API(f64, double)

}  // extern "C"
