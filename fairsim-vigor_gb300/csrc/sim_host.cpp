// Host-side SimParam logic. The matrix inverse follows MatrixComplex
// (org/fairsim/linalg/MatrixComplex.java:56-264): a pivot permutation computed once on the
// original columns, Doolittle LU on the pivoted matrix, forward/back substitution for
// every unit vector; the pseudo-inverse is (A*A)^-1 A*.
#include "sim_host.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>

namespace fsim {

void set_error(const char* fmt, ...);

namespace {
struct M {
  int m, n;
  std::vector<cd> v;
  M(int m_, int n_) : m(m_), n(n_), v((size_t)m_ * n_, cd(0, 0)) {}
  cd& operator()(int i, int j) { return v[(size_t)i * n + j]; }
  cd operator()(int i, int j) const { return v[(size_t)i * n + j]; }
};
// complex ops with the reference's formulas (Cplx.Double mult/reciproc/div)
inline cd mul(cd a, cd b) { return cd(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real()); }
inline cd div_(cd a, cd b) {
  double s = b.real() * b.real() + b.imag() * b.imag();
  return mul(a, cd(b.real() / s, -b.imag() / s));
}
M mat_mul(const M& a, const M& b) {
  M c(a.m, b.n);
  for (int i = 0; i < a.m; i++)
    for (int k = 0; k < a.n; k++)
      for (int j = 0; j < b.n; j++) c(i, j) += mul(a(i, k), b(k, j));
  return c;
}
M unity(int n) {
  M r(n, n);
  for (int i = 0; i < n; i++) r(i, i) = cd(1, 0);
  return r;
}
M pivot(const M& a) {
  int n = a.n;
  M p = unity(n);
  for (int i = 0; i < n; i++) {
    int mj = i;
    for (int j = i; j < n; j++)
      if (std::hypot(a(j, i).real(), a(j, i).imag()) > std::hypot(a(mj, i).real(), a(mj, i).imag())) mj = j;
    if (mj != i)
      for (int k = 0; k < n; k++) std::swap(p(i, k), p(mj, k));
  }
  return p;
}
M inverse(const M& a) {
  int n = a.n;
  M U(n, n), L = unity(n), P = pivot(a);
  M Ap = mat_mul(P, a);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      if (j <= i) {
        cd s(0, 0);
        for (int k = 0; k < j; k++) s += mul(L(j, k), U(k, i));
        U(j, i) = Ap(j, i) - s;
      }
      if (j >= i) {
        cd s(0, 0);
        for (int k = 0; k < i; k++) s += mul(L(j, k), U(k, i));
        L(j, i) = div_(Ap(j, i) - s, U(i, i));
      }
    }
  M y(n, n), x(n, n);
  for (int k = 0; k < n; k++)
    for (int i = 0; i < n; i++) {
      cd r = P(i, k);
      for (int j = 0; j < i; j++) r -= mul(L(i, j), y(j, k));
      y(i, k) = div_(r, L(i, i));
    }
  for (int k = 0; k < n; k++)
    for (int i = n - 1; i >= 0; i--) {
      cd r = y(i, k);
      for (int j = i + 1; j < n; j++) r -= mul(U(i, j), x(j, k));
      x(i, k) = div_(r, U(i, i));
    }
  return x;
}
M pseudo_inverse(const M& a) {
  M adj(a.n, a.m);
  for (int i = 0; i < a.m; i++)
    for (int j = 0; j < a.n; j++) adj(j, i) = std::conj(a(i, j));
  return mat_mul(inverse(mat_mul(adj, a)), adj);
}
}  // namespace

std::vector<double> dir_phases(const fsim_sim_param* p, int d) {
  std::vector<double> r(p->nr_phases);
  for (int i = 0; i < p->nr_phases; i++) {
    double base = p->has_phases ? p->phases[d][i] : (2 * M_PI / p->nr_phases) * i;
    r[i] = base + p->pha_off[d];
  }
  return r;
}

std::vector<double> dir_modulations(const fsim_sim_param* p, int d) {
  std::vector<double> r(p->nr_bands);
  for (int b = 0; b < p->nr_bands; b++) {
    double m = p->modulation[d][b];
    if (m < 0.3) m = 0.3;
    if (m > 1.1) m = 1.1;
    r[b] = m;
  }
  return r;
}

std::vector<cd> separation_matrix(const std::vector<double>& phases, int bands, std::vector<double> fac) {
  const int nP = (int)phases.size(), nC = 2 * bands - 1;
  if (fac.empty()) {
    fac.assign(bands, .5);
    fac[0] = 1.0;
  } else {
    for (int i = 1; i < bands; i++) fac[i] *= 0.5;
  }
  M A(nP, nC);
  for (int i = 0; i < nP; i++) {
    A(i, 0) = cd(fac[0], 0);
    for (int j = 0; j < bands - 1; j++) {
      double ph = phases[i] * (j + 1);
      A(i, 2 * j + 1) = cd(fac[j + 1] * std::cos(ph), fac[j + 1] * std::sin(ph));
      A(i, 2 * j + 2) = cd(fac[j + 1] * std::cos(-ph), fac[j + 1] * std::sin(-ph));
    }
  }
  M inv = (nP == nC) ? inverse(A) : pseudo_inverse(A);
  return inv.v;
}

std::vector<std::complex<float>> separation_coeffs(const fsim_sim_param* p, int d, bool estimation) {
  std::vector<double> ph, fac;
  if (estimation) {  // separateBands(in, out, phaOff=0, bands, fac=null)
    ph.resize(p->nr_phases);
    for (int i = 0; i < p->nr_phases; i++) ph[i] = (2 * M_PI * i) / p->nr_phases;
  } else {
    ph = dir_phases(p, d);
    fac = dir_modulations(p, d);
  }
  std::vector<cd> m = separation_matrix(ph, p->nr_bands, fac);
  std::vector<std::complex<float>> r(m.size());
  for (size_t i = 0; i < m.size(); i++) r[i] = std::complex<float>((float)m[i].real(), (float)m[i].imag());
  return r;
}

int validate_param(const fsim_sim_param* p) {
  if (!p) {
    set_error("null SimParam");
    return FSIM_EINVAL;
  }
  if (p->nr_dirs < 1 || p->nr_dirs > FSIM_MAX_DIRS || p->nr_bands < 2 || p->nr_bands > FSIM_MAX_BANDS ||
      p->nr_phases < 2 * p->nr_bands - 1 || p->nr_phases > FSIM_MAX_PHASES) {
    set_error("SimParam: bad dirs/bands/phases %d/%d/%d", p->nr_dirs, p->nr_bands, p->nr_phases);
    return FSIM_EINVAL;
  }
  if (p->otf_a < 0 || p->otf_a > 1 || p->na < 0.3 || p->na > 2.2 || p->em_wavelength < 300 || p->em_wavelength > 1500) {
    set_error("unphysical input parameters");  // OtfProvider.fromEstimate's IllegalArgumentException
    return FSIM_EINVAL;
  }
  if (p->w < 8 || p->microns_per_pixel <= 0) {
    set_error("SimParam: bad image size %d / pixel size %g", p->w, p->microns_per_pixel);
    return FSIM_EINVAL;
  }
  if (p->otf_data && p->otf_samples > 0) {
    // measured OTF: getOtfVal throws for a band beyond a multi-band table (OtfProvider.java:192-193)
    if (p->otf_bands < 1 || p->otf_bands > FSIM_MAX_BANDS || p->otf_samples > 1024 || !(p->otf_cycles > 0) ||
        (p->otf_bands > 1 && p->nr_bands > p->otf_bands)) {
      set_error("SimParam: bad measured OTF (%d bands, %d samples, %g cycles/micron per sample)", p->otf_bands,
                p->otf_samples, p->otf_cycles);
      return FSIM_EINVAL;
    }
  }
  if (p->filter_style < FSIM_FILTER_WIENER || p->filter_style > FSIM_FILTER_RL_BOTH ||
      (p->filter_style != FSIM_FILTER_WIENER && p->rl_iterations < 0)) {
    set_error("SimParam: bad filter style %d / RL iterations %d", p->filter_style, p->rl_iterations);
    return FSIM_EINVAL;
  }
  return FSIM_OK;
}

}  // namespace fsim

// BandSeparation.createSeparationMatrix (S/BandSeparation.java:40-114) for the phases of
// band 1 (band b's phases are b times them): the inverse (nP == 2*bands-1) or pseudo-inverse
// of the phase matrix, [component][phase] interleaved complex doubles. Host-only.
extern "C" int fsim_separation_matrix(const double* phases, int n_phases, int bands, const double* fac,
                                      double* out) {
  if (!phases || !out) {
    fsim::set_error("separation_matrix: null argument");
    return FSIM_EINVAL;
  }
  if (bands < 2 || bands > FSIM_MAX_BANDS) {
    fsim::set_error("#bands < 2, not useful");
    return FSIM_EINVAL;
  }
  if (n_phases < 2 * bands - 1 || n_phases > FSIM_MAX_PHASES) {
    fsim::set_error("not enough phases for #bands");
    return FSIM_EINVAL;
  }
  std::vector<double> ph(phases, phases + n_phases), fc;
  if (fac) fc.assign(fac, fac + bands);
  const std::vector<fsim::cd> m = fsim::separation_matrix(ph, bands, fc);
  for (size_t i = 0; i < m.size(); i++) {
    out[2 * i] = m[i].real();
    out[2 * i + 1] = m[i].imag();
  }
  return FSIM_OK;
}
