// ORACLE — test infrastructure only. Not part of the product.
//
// CPU restatement of fairSIM's 2D SIM reconstruction path (the Java code under
// org/fairsim/{linalg,sim_algorithm,livemode}), used by the tests, by smoke() and by
// the CPU-baseline leg of bench.py to compare against. The GPU library never links it.
//
// Two instantiations:
//   T = float   reproduces the reference's single-precision semantics: float vectors,
//               float-rounded Fourier-shift phases fed to MTool.fsin/fcos, floor-indexed
//               OTF lookup, Java float operation order (compile with -ffp-contract=off).
//   T = double  the same algorithm carried out in double precision with libm sin/cos
//               and unrounded phases: the "FP64 oracle" that error figures are quoted
//               against.
//
// Parity status: the Java reference cannot run in this environment (no JVM, and its FFT
// lives in the absent JTransforms 3.1 jar), and the reference ships no golden vectors.
// This restatement is therefore "parity unpinned" against the reference's own outputs;
// it is pinned instead by known-answer tests (FFT vs numpy, MTool.fsin error bound of
// L/MTool.java:33, MatrixComplex inverse identity, band-separation recovery, integer
// Fourier shift == circular roll, parameter-estimation recovery of seeded k0).
//
// Citations are relative to the reference project root:
//   L/ = org/fairsim/linalg/, S/ = org/fairsim/sim_algorithm/, LM/ = org/fairsim/livemode/
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <vector>

namespace ref {

// ---------------------------------------------------------------------------
// Row-splitting thread pool: the same work split as SimpleMT.PFor
// (org/fairsim/utils/SimpleMT.java:124-155): a loop range cut into one chunk per thread.
// ---------------------------------------------------------------------------
class Pool {
 public:
  static Pool& get() {
    static Pool p;
    return p;
  }
  void set_threads(int n) {
    n = std::max(1, n);
    if (n == nthreads_) return;
    shutdown();
    nthreads_ = n;
    start();
  }
  int threads() const { return nthreads_; }

  template <class F>
  void pfor(int begin, int end, F&& f) {
    int n = end - begin;
    if (n <= 0) return;
    if (nthreads_ <= 1 || n == 1) {
      for (int i = begin; i < end; i++) f(i);
      return;
    }
    std::function<void(int)> body = [&](int i) { f(i); };
    run(begin, end, body);
  }

  ~Pool() { shutdown(); }

 private:
  Pool() { start(); }
  void start() {
    stop_ = false;
    for (int t = 1; t < nthreads_; t++) workers_.emplace_back([this, t] { loop(t); });
  }
  void shutdown() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
      gen_++;
    }
    cv_.notify_all();
    for (auto& w : workers_) w.join();
    workers_.clear();
  }
  void chunk(int t) {
    int n = end_ - begin_;
    int per = (n + nthreads_ - 1) / nthreads_;
    int b = begin_ + t * per, e = std::min(end_, b + per);
    for (int i = b; i < e; i++) (*body_)(i);
  }
  void loop(int t) {
    int seen = 0;
    for (;;) {
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] { return gen_ != seen; });
      seen = gen_;
      if (stop_) return;
      lk.unlock();
      chunk(t);
      if (remaining_.fetch_sub(1) == 1) {
        std::lock_guard<std::mutex> g(dm_);
        dcv_.notify_all();
      }
    }
  }
  void run(int begin, int end, std::function<void(int)>& body) {
    std::lock_guard<std::mutex> serial(run_m_);
    {
      std::lock_guard<std::mutex> g(m_);
      begin_ = begin;
      end_ = end;
      body_ = &body;
      remaining_ = nthreads_ - 1;
      gen_++;
    }
    cv_.notify_all();
    chunk(0);
    std::unique_lock<std::mutex> lk(dm_);
    dcv_.wait(lk, [&] { return remaining_.load() == 0; });
  }

  int nthreads_ = 1;
  std::vector<std::thread> workers_;
  std::mutex m_, dm_, run_m_;
  std::condition_variable cv_, dcv_;
  int gen_ = 0;
  bool stop_ = false;
  int begin_ = 0, end_ = 0;
  std::function<void(int)>* body_ = nullptr;
  std::atomic<int> remaining_{0};
};

template <class F>
inline void pfor(int b, int e, F&& f) {
  Pool::get().pfor(b, e, std::forward<F>(f));
}

// ---------------------------------------------------------------------------
// MTool (L/MTool.java:34-64)
// ---------------------------------------------------------------------------
inline double aproxSin01(double x) {
  double x2 = x * x;
  return ((((.00015148419 * x2 - .00467376557) * x2 + .07968967928) * x2 - .64596371106) * x2 +
          1.57079631847) *
         x;
}
inline double fsin(double x) {
  x = x / (M_PI / 2);
  x -= std::floor(0.25 * x) * 4;
  if (x > 3) return -aproxSin01(4 - x);
  if (x > 1) return aproxSin01(2 - x);
  return aproxSin01(x);
}
inline double fcos(double x) { return fsin(x + M_PI / 2); }
inline double fhypot(double x, double y) { return std::sqrt(x * x + y * y); }

// Java's (float) cast for T=float, identity for the FP64 oracle.
template <class T>
inline T rnd(double v) {
  return (T)v;
}

// ---------------------------------------------------------------------------
// Complex helpers with Java's operation order (L/Cplx.java:262-332)
// ---------------------------------------------------------------------------
template <class T>
struct C {
  T re, im;
};
template <class T>
inline C<T> cmul(C<T> a, C<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class T>
inline C<T> cconj(C<T> a) {
  return {a.re, -a.im};
}
template <class T>
inline C<T> cadd(C<T> a, C<T> b) {
  return {a.re + b.re, a.im + b.im};
}
template <class T>
inline C<T> crecip(C<T> a) {
  T s = a.re * a.re + a.im * a.im;
  return {a.re / s, -a.im / s};
}
template <class T>
inline C<T> cdiv(C<T> a, C<T> b) {
  return cmul(a, crecip(b));
}
// Cplx.Float.abs(): (float)Math.sqrt((double)re*re+(double)im*im)  (L/Cplx.java:159-161)
template <class T>
inline T cabs_f(C<T> a) {
  return (T)std::sqrt((double)a.re * a.re + (double)a.im * a.im);
}

// ---------------------------------------------------------------------------
// Vectors: row-major x + w*y, complex interleaved (L/Vec2d.java:23-24)
// ---------------------------------------------------------------------------
template <class T>
struct RVec {
  int w = 0, h = 0;
  std::vector<T> d;
  RVec() = default;
  RVec(int w_, int h_) : w(w_), h(h_), d((size_t)w_ * h_, T(0)) {}
  T& at(int x, int y) { return d[(size_t)x + (size_t)w * y]; }
  T at(int x, int y) const { return d[(size_t)x + (size_t)w * y]; }
};
template <class T>
struct CVec {
  int w = 0, h = 0;
  std::vector<T> d;
  CVec() = default;
  CVec(int w_, int h_) : w(w_), h(h_), d((size_t)2 * w_ * h_, T(0)) {}
  size_t n() const { return (size_t)w * h; }
  C<T> get(int x, int y) const {
    size_t i = (size_t)x + (size_t)w * y;
    return {d[2 * i], d[2 * i + 1]};
  }
  void set(int x, int y, C<T> v) {
    size_t i = (size_t)x + (size_t)w * y;
    d[2 * i] = v.re;
    d[2 * i + 1] = v.im;
  }
  void zero() { std::fill(d.begin(), d.end(), T(0)); }
};

// AbstractVectorCplx ops (L/AbstractVectorCplx.java:156-373)
template <class T>
inline void v_add(CVec<T>& y, const CVec<T>& x) {
  for (size_t j = 0; j < y.d.size(); j++) y.d[j] += x.d[j];
}
template <class T>
inline void v_axpy(CVec<T>& y, C<T> a, const CVec<T>& x) {
  size_t n = y.n();
  for (size_t i = 0; i < n; i++) {
    T xr = x.d[2 * i], xi = x.d[2 * i + 1];
    y.d[2 * i] += a.re * xr - a.im * xi;
    y.d[2 * i + 1] += a.im * xr + a.re * xi;
  }
}
// times(in, conj): y = in * y  (multReal(x, y) with x = in) (L/AbstractVectorCplx.java:288-304)
template <class T>
inline void v_times(CVec<T>& y, const CVec<T>& in, bool conj) {
  size_t n = y.n();
  for (size_t i = 0; i < n; i++) {
    T xr = in.d[2 * i], xi = conj ? -in.d[2 * i + 1] : in.d[2 * i + 1];
    T yr = y.d[2 * i], yi = y.d[2 * i + 1];
    y.d[2 * i] = xr * yr - xi * yi;
    y.d[2 * i + 1] = xi * yr + xr * yi;
  }
}
template <class T>
inline void v_times_real(CVec<T>& y, const RVec<T>& in) {
  size_t n = y.n();
  for (size_t i = 0; i < n; i++) {
    y.d[2 * i] *= in.d[i];
    y.d[2 * i + 1] *= in.d[i];
  }
}
template <class T>
inline void v_scal(CVec<T>& y, T a) {
  for (auto& v : y.d) v *= a;
}
// norm2: sum of float squares accumulated in double (L/AbstractVectorCplx.java:241-247)
template <class T>
inline double v_norm2(const CVec<T>& y) {
  double r = 0;
  for (auto v : y.d) r += (T)(v * v);
  return r;
}
// sumElements in double (L/AbstractVectorCplx.java:353-362)
template <class T>
inline C<double> v_sum(const CVec<T>& y) {
  double re = 0, im = 0;
  size_t n = y.n();
  for (size_t i = 0; i < n; i++) {
    re += y.d[2 * i];
    im += y.d[2 * i + 1];
  }
  return {re, im};
}

// reciproc: conj(z)/|z|^2 in float (L/AbstractVectorCplx.java:208-216)
template <class T>
inline void v_reciproc(CVec<T>& y) {
  size_t n = y.n();
  for (size_t i = 0; i < n; i++) {
    T s = y.d[2 * i] * y.d[2 * i] + y.d[2 * i + 1] * y.d[2 * i + 1];
    y.d[2 * i] = y.d[2 * i] / s;
    y.d[2 * i + 1] = -y.d[2 * i + 1] / s;
  }
}

// ---------------------------------------------------------------------------
// FFT: mixed-radix (2,3,4,5) Stockham, the stand-in for JTransforms 3.1
// (L/JTransformsConnector.java:76-92): FloatFFT_2D(rows=h, cols=w), in place on
// interleaved complex data, forward exp(-2 pi i), inverse exp(+2 pi i) scaled 1/(w*h).
// ---------------------------------------------------------------------------
template <class T>
struct FFT1 {
  int n = 0;
  std::vector<int> radix;
  std::vector<T> tw;  // exp(-2 pi i m / n), m in [0,n)
  explicit FFT1(int n_) : n(n_) {
    int m = n;
    while (m > 1) {
      if (m % 4 == 0) {
        radix.push_back(4);
        m /= 4;
      } else if (m % 2 == 0) {
        radix.push_back(2);
        m /= 2;
      } else if (m % 3 == 0) {
        radix.push_back(3);
        m /= 3;
      } else if (m % 5 == 0) {
        radix.push_back(5);
        m /= 5;
      } else {
        throw std::runtime_error("FFT size must be 2^a 3^b 5^c");
      }
    }
    tw.resize(2 * (size_t)n);
    for (int k = 0; k < n; k++) {
      double a = -2.0 * M_PI * (double)k / (double)n;
      tw[2 * k] = (T)std::cos(a);
      tw[2 * k + 1] = (T)std::sin(a);
    }
  }
  // x: n complex, stride 1. scratch: n complex. Result in x.
  void exec(T* x, T* scratch, bool inverse) const {
    T* in = x;
    T* out = scratch;
    int Ns = 1;
    const T sg = inverse ? T(1) : T(-1);
    for (int R : radix) {
      int nr = n / R;
      for (int j = 0; j < nr; j++) {
        int k = j % Ns;
        T vr[5], vi[5];
        for (int r = 0; r < R; r++) {
          T a = in[2 * (j + r * nr)], b = in[2 * (j + r * nr) + 1];
          if (r && k) {
            int m = (r * k * (n / (Ns * R)));
            T c = tw[2 * m], s = inverse ? -tw[2 * m + 1] : tw[2 * m + 1];
            T ar = a * c - b * s, ai = a * s + b * c;
            a = ar;
            b = ai;
          }
          vr[r] = a;
          vi[r] = b;
        }
        T yr[5], yi[5];
        if (R == 2) {
          yr[0] = vr[0] + vr[1];
          yi[0] = vi[0] + vi[1];
          yr[1] = vr[0] - vr[1];
          yi[1] = vi[0] - vi[1];
        } else if (R == 4) {
          T ar = vr[0] + vr[2], ai = vi[0] + vi[2];
          T br = vr[0] - vr[2], bi = vi[0] - vi[2];
          T cr = vr[1] + vr[3], ci = vi[1] + vi[3];
          T dr = vr[1] - vr[3], di = vi[1] - vi[3];
          // forward: y1 = b - i d ; inverse: y1 = b + i d
          yr[0] = ar + cr;
          yi[0] = ai + ci;
          yr[2] = ar - cr;
          yi[2] = ai - ci;
          yr[1] = br - sg * di;
          yi[1] = bi + sg * dr;
          yr[3] = br + sg * di;
          yi[3] = bi - sg * dr;
        } else {
          for (int q = 0; q < R; q++) {
            double sr = 0, si = 0;
            for (int r = 0; r < R; r++) {
              double ang = sg * 2.0 * M_PI * (double)((q * r) % R) / R;
              double c = std::cos(ang), s = std::sin(ang);
              sr += vr[r] * c - vi[r] * s;
              si += vr[r] * s + vi[r] * c;
            }
            yr[q] = (T)sr;
            yi[q] = (T)si;
          }
        }
        int base = (j / Ns) * Ns * R + k;
        for (int r = 0; r < R; r++) {
          out[2 * (base + r * Ns)] = yr[r];
          out[2 * (base + r * Ns) + 1] = yi[r];
        }
      }
      std::swap(in, out);
      Ns *= R;
    }
    if (in != x) std::memcpy(x, in, sizeof(T) * 2 * n);
  }
};

template <class T>
inline void fft2d(CVec<T>& v, bool inverse) {
  const int w = v.w, h = v.h;
  FFT1<T> fx(w), fy(h);
  T* d = v.d.data();
  // rows
  pfor(0, h, [&](int y) {
    std::vector<T> s(2 * (size_t)w);
    fx.exec(d + 2 * (size_t)w * y, s.data(), inverse);
  });
  // columns, in blocks of 8 gathered into contiguous lines
  const int B = 8;
  int nb = (w + B - 1) / B;
  pfor(0, nb, [&](int b) {
    std::vector<T> line(2 * (size_t)h), s(2 * (size_t)h);
    for (int x = b * B; x < std::min(w, b * B + B); x++) {
      for (int y = 0; y < h; y++) {
        line[2 * y] = d[2 * ((size_t)x + (size_t)w * y)];
        line[2 * y + 1] = d[2 * ((size_t)x + (size_t)w * y) + 1];
      }
      fy.exec(line.data(), s.data(), inverse);
      for (int y = 0; y < h; y++) {
        d[2 * ((size_t)x + (size_t)w * y)] = line[2 * y];
        d[2 * ((size_t)x + (size_t)w * y) + 1] = line[2 * y + 1];
      }
    }
  });
  if (inverse) {
    T sc = (T)(1.0 / ((double)w * (double)h));
    size_t n = v.d.size();
    pfor(0, h, [&](int y) {
      size_t b = 2 * (size_t)w * y, e = std::min(n, b + 2 * (size_t)w);
      for (size_t i = b; i < e; i++) d[i] *= sc;
    });
  }
}

// ---------------------------------------------------------------------------
// BasicVectors.BCplx2D.pasteFreq / fourierShift (L/BasicVectors.java:259-339)
// ---------------------------------------------------------------------------
template <class T>
inline void paste_freq(CVec<T>& out, const CVec<T>& in, int xOff, int yOff) {
  const int wi = in.w, hi = in.h, wo = out.w, ho = out.h;
  out.zero();
  for (int y = 0; y < hi; y++)
    for (int x = 0; x < wi; x++) {
      int xo = (x < wi / 2) ? x : x + wo / 2;
      int yo = (y < hi / 2) ? y : y + ho / 2;
      xo = (xo + xOff + wo) % wo;
      yo = (yo + yOff + ho) % ho;
      out.d[2 * ((size_t)xo + (size_t)wo * yo)] = in.d[2 * ((size_t)x + (size_t)wi * y)];
      out.d[2 * ((size_t)xo + (size_t)wo * yo) + 1] = in.d[2 * ((size_t)x + (size_t)wi * y) + 1];
    }
}

template <class T>
inline void fourier_shift(CVec<T>& v, double kx, double ky) {
  if (v.w != v.h) throw std::runtime_error("fourierShift needs a square vector");
  const int N = v.w;
  T* val = v.d.data();
  pfor(0, N, [&](int y) {
    for (int x = 0; x < N; x++) {
      T co, si;
      if (sizeof(T) == 4) {
        float pha = (float)(2 * M_PI * (kx * x + ky * y) / N);
        co = (T)fcos(pha);
        si = (T)fsin(pha);
      } else {
        double pha = 2 * M_PI * (kx * x + ky * y) / N;
        co = (T)std::cos(pha);
        si = (T)std::sin(pha);
      }
      size_t i = (size_t)y * N + x;
      T re = val[2 * i], im = val[2 * i + 1];
      val[2 * i] = re * co - im * si;
      val[2 * i + 1] = im * co + re * si;
    }
  });
}

// ---------------------------------------------------------------------------
// MatrixComplex (L/MatrixComplex.java:56-264): pivot computed on the original matrix,
// Doolittle LU, forward/back substitution, pseudo-inverse (A*A)^-1 A*.
// ---------------------------------------------------------------------------
struct Mat {
  int m = 0, n = 0;
  std::vector<C<double>> v;
  Mat() = default;
  Mat(int m_, int n_) : m(m_), n(n_), v((size_t)m_ * n_, C<double>{0, 0}) {}
  C<double>& operator()(int i, int j) { return v[(size_t)i * n + j]; }
  C<double> operator()(int i, int j) const { return v[(size_t)i * n + j]; }
  static Mat unity(int n) {
    Mat r(n, n);
    for (int i = 0; i < n; i++) r(i, i) = {1, 0};
    return r;
  }
};
inline double chypot(C<double> a) { return std::hypot(a.re, a.im); }
inline C<double> csub(C<double> a, C<double> b) { return {a.re - b.re, a.im - b.im}; }
inline Mat mat_mult(const Mat& a, const Mat& b) {
  Mat c(a.m, b.n);
  for (int i = 0; i < a.m; i++)
    for (int k = 0; k < a.n; k++)
      for (int j = 0; j < b.n; j++) c(i, j) = cadd(c(i, j), cmul(a(i, k), b(k, j)));
  return c;
}
inline Mat mat_pivot(const Mat& a) {
  int n = a.n;
  Mat p = Mat::unity(n);
  for (int i = 0; i < n; i++) {
    int max_j = i;
    for (int j = i; j < n; j++)
      if (chypot(a(j, i)) > chypot(a(max_j, i))) max_j = j;
    if (max_j != i)
      for (int k = 0; k < n; k++) std::swap(p(i, k), p(max_j, k));
  }
  return p;
}
inline Mat mat_inverse(const Mat& a) {
  if (a.m != a.n) throw std::runtime_error("not a square matrix");
  int n = a.n;
  Mat U(n, n), L = Mat::unity(n), P = mat_pivot(a);
  Mat Ap = mat_mult(P, a);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      if (j <= i) {
        C<double> s{0, 0};
        for (int k = 0; k < j; k++) s = cadd(s, cmul(L(j, k), U(k, i)));
        U(j, i) = csub(Ap(j, i), s);
      }
      if (j >= i) {
        C<double> s{0, 0};
        for (int k = 0; k < i; k++) s = cadd(s, cmul(L(j, k), U(k, i)));
        L(j, i) = cdiv(csub(Ap(j, i), s), U(i, i));
      }
    }
  Mat y(n, n), x(n, n);
  for (int k = 0; k < n; k++)
    for (int i = 0; i < n; i++) {
      C<double> res = P(i, k);
      for (int j = 0; j < i; j++) res = csub(res, cmul(L(i, j), y(j, k)));
      y(i, k) = cdiv(res, L(i, i));
    }
  for (int k = 0; k < n; k++)
    for (int i = n - 1; i >= 0; i--) {
      C<double> res = y(i, k);
      for (int j = i + 1; j < n; j++) res = csub(res, cmul(U(i, j), x(j, k)));
      x(i, k) = cdiv(res, U(i, i));
    }
  return x;
}
inline Mat mat_pseudo_inverse(const Mat& a) {
  Mat adj(a.n, a.m);
  for (int i = 0; i < a.m; i++)
    for (int j = 0; j < a.n; j++) adj(j, i) = cconj(a(i, j));
  Mat axa = mat_mult(adj, a);
  Mat inv = mat_inverse(axa);
  return mat_mult(inv, adj);
}

// BandSeparation.createSeparationMatrix (S/BandSeparation.java:40-114).
// phases[b-1][p]; fac may be empty (then [1,.5,.5,...]); returns inverse (nC x nP).
inline Mat separation_matrix(const std::vector<std::vector<double>>& phases, int bands,
                             std::vector<double> fac) {
  if (bands < 2) throw std::runtime_error("#bands < 2, not useful");
  if ((int)phases.size() != bands - 1 || (!fac.empty() && (int)fac.size() != bands))
    throw std::runtime_error("#factors or #phases+1 != #bands");
  int nrPhases = (int)phases[0].size();
  if (nrPhases < bands * 2 - 1) throw std::runtime_error("not enough phases for #bands");
  if (fac.empty()) {
    fac.resize(bands);
    for (int i = 0; i < bands; i++) fac[i] = (i == 0) ? 1.0 : .5;
  } else {
    for (int i = 1; i < bands; i++) fac[i] *= 0.5;
  }
  Mat M(nrPhases, bands * 2 - 1);
  for (int i = 0; i < nrPhases; i++) {
    M(i, 0) = {fac[0], 0};
    for (int j = 0; j < bands - 1; j++) {
      M(i, 2 * j + 1) = {fac[j + 1] * std::cos(phases[j][i]), fac[j + 1] * std::sin(phases[j][i])};
      M(i, 2 * j + 2) = {fac[j + 1] * std::cos(-phases[j][i]), fac[j + 1] * std::sin(-phases[j][i])};
    }
  }
  if (nrPhases == bands * 2 - 1) return mat_inverse(M);
  return mat_pseudo_inverse(M);
}

// BandSeparation.separateBands (S/BandSeparation.java:131-165)
template <class T>
inline void separate_bands(const std::vector<CVec<T>>& in, std::vector<CVec<T>>& out,
                           const std::vector<double>& phases, int bands, const std::vector<double>& fac) {
  if (in.size() != phases.size()) throw std::runtime_error("#input images != phases per band");
  if ((int)out.size() != bands * 2 - 1) throw std::runtime_error("#output images != #bands*2-1");
  std::vector<std::vector<double>> pha(bands - 1, std::vector<double>(phases.size()));
  for (int b = 1; b < bands; b++)
    for (size_t p = 0; p < phases.size(); p++) pha[b - 1][p] = phases[p] * b;
  Mat S = separation_matrix(pha, bands, fac);
  for (auto& o : out) o.zero();
  for (size_t p = 0; p < phases.size(); p++)
    for (int b = 0; b < bands * 2 - 1; b++) {
      C<T> a{(T)S(b, (int)p).re, (T)S(b, (int)p).im};  // toFlt()
      v_axpy(out[b], a, in[p]);
    }
}
template <class T>
inline void separate_bands_eq(const std::vector<CVec<T>>& in, std::vector<CVec<T>>& out, double phaOff,
                              int bands, const std::vector<double>& fac) {
  int n = (int)in.size();
  std::vector<double> ph(n);
  for (int p = 0; p < n; p++) ph[p] = (2 * M_PI * p) / n + phaOff;
  separate_bands(in, out, ph, bands, fac);
}

// ---------------------------------------------------------------------------
// OtfProvider, estimate form (S/OtfProvider.java:74-559)
// ---------------------------------------------------------------------------
inline double val_ideal_otf(double dist) {
  if (dist < 0 || dist > 1) return 0;
  return (2 / M_PI) * (std::acos(dist) - dist * std::sqrt(1 - dist * dist));
}
template <class T>
inline T val_attenuation(double dist, double str, double fwhm) {
  return rnd<T>(1 - str * std::exp(-(std::pow(dist, 2)) / (2 * std::pow(fwhm / 2.355, 2))));
}

template <class T>
struct Otf {
  // estimates: one real band of 512 samples up to the cutoff (OtfProvider.fromEstimate,
  // S/OtfProvider.java:96-127); measured: maxBand complex bands of samplesLateral samples at
  // cyclesPerMicron spacing (loadFromConfig with band data, :588-621)
  double na = 0, lambda = 0, cutOff = 0, cyclesPerMicron = 0, a = 1;
  double attStrength = .99, attFWHM = 1.2;
  bool useAtt = false;
  bool isMultiBand = false;
  int maxBand = 1, samplesLateral = 512;
  double vecCyclesPerMicron = -1;
  std::vector<std::vector<C<T>>> vals, valsAtt;
  std::vector<std::vector<T>> valsOnlyAtt;

  static Otf fromEstimate(double na, double lambda, double a) {
    if (a < 0 || a > 1 || na < 0.3 || na > 2.2 || lambda < 300 || lambda > 1500)
      throw std::runtime_error("unphysical input parameters");
    Otf o;
    o.na = na;
    o.lambda = lambda;
    o.a = a;
    o.cutOff = 1000 / (lambda / na / 2);
    o.samplesLateral = 512;
    o.cyclesPerMicron = o.cutOff / o.samplesLateral;
    o.alloc(1);
    for (int i = 0; i < o.samplesLateral; i++) {
      double v = i / (double)o.samplesLateral;
      o.vals[0][i] = {rnd<T>(val_ideal_otf(v) * std::pow(a, v)), T(0)};
    }
    o.setAttenuation(o.attStrength, o.attFWHM);
    o.useAtt = false;
    return o;
  }
  // loadFromConfig with a "data" folder: data = bands x samples complex (re, im) floats
  static Otf fromData(double na, double lambda, int bands, int samples, double cycles, const float* data) {
    if (bands < 1 || samples < 1 || cycles <= 0) throw std::runtime_error("bad OTF data");
    Otf o;
    o.na = na;
    o.lambda = lambda;
    o.cutOff = 1000 / (lambda / na / 2);
    o.samplesLateral = samples;
    o.cyclesPerMicron = cycles;
    o.isMultiBand = bands > 1;
    o.alloc(bands);
    for (int b = 0; b < bands; b++)
      for (int i = 0; i < samples; i++)
        o.vals[b][i] = {(T)data[2 * ((size_t)b * samples + i)], (T)data[2 * ((size_t)b * samples + i) + 1]};
    o.setAttenuation(o.attStrength, o.attFWHM);
    o.useAtt = false;
    return o;
  }
  void alloc(int bands) {
    maxBand = bands;
    vals.assign(bands, std::vector<C<T>>(samplesLateral));
    valsAtt.assign(bands, std::vector<C<T>>(samplesLateral));
    valsOnlyAtt.assign(bands, std::vector<T>(samplesLateral));
  }
  void setAttenuation(double str, double fwhm) {  // :276-287
    attStrength = str;
    attFWHM = fwhm;
    for (int b = 0; b < maxBand; b++)
      for (int v = 0; v < samplesLateral; v++) {
        double dist = v * cyclesPerMicron;
        valsOnlyAtt[b][v] = val_attenuation<T>(dist, attStrength, attFWHM);
        valsAtt[b][v] = {vals[b][v].re * valsOnlyAtt[b][v], vals[b][v].im * valsOnlyAtt[b][v]};
      }
  }
  int bandIdx(int band) const {
    if (!isMultiBand) band = 0;
    if (band >= maxBand || band < 0) throw std::runtime_error("band idx too high or <0");
    return band;
  }
  // getOtfVal: floor-indexed, "interpolation" weights both on lPos (S/OtfProvider.java:189-222)
  C<T> getOtfVal(int band, double cycl, bool att) const {
    band = bandIdx(band);
    if (cycl < 0) throw std::runtime_error("cylc negative!");
    if (cycl >= cutOff) return {0, 0};
    const double pos = cycl / cyclesPerMicron;
    if (std::ceil(pos) >= samplesLateral) return {0, 0};
    int lPos = (int)std::floor(pos);
    T f = (T)(pos - lPos);
    C<T> v = att ? valsAtt[band][lPos] : vals[band][lPos];
    T g = T(1) - f;
    return {v.re * g + v.re * f, v.im * g + v.im * f};  // Cplx.add(v.mult(1-f), v.mult(f))
  }
  // getAttVal (:246-269); beyond the table the reference indexes out of its arrays
  T getAttVal(int band, double cycl) const {
    band = bandIdx(band);
    if (cycl >= cutOff) return T(1);
    double pos = cycl / cyclesPerMicron;
    int lPos = (int)std::floor(pos);
    if (lPos >= samplesLateral) throw std::runtime_error("attenuation beyond the OTF table");
    T f = (T)(pos - lPos);
    T retl = valsOnlyAtt[band][lPos] * f;
    T reth = valsOnlyAtt[band][lPos] * (T(1) - f);
    return retl + reth;
  }
  // otfToVector (S/OtfProvider.java:331-373): write the OTF, or multiply by its conjugate
  void otfToVector(CVec<T>& vec, int band, double kx, double ky, bool att, bool write) const {
    if (vecCyclesPerMicron <= 0) throw std::runtime_error("Vector pixel size not initialized");
    const int w = vec.w, h = vec.h;
    pfor(0, h, [&](int y) {
      for (int x = 0; x < w; x++) {
        double xh = (x < w / 2) ? x : x - w;
        double yh = (y < h / 2) ? -y : h - y;
        double rad = fhypot(xh - kx, yh - ky);
        double cycl = rad * vecCyclesPerMicron;
        if (cycl > cutOff) {
          vec.set(x, y, {0, 0});
        } else {
          C<T> val = getOtfVal(band, cycl, att);
          if (!write) {
            C<T> a = vec.get(x, y);
            C<T> b{val.re, -val.im};  // val.conj()
            vec.set(x, y, cmul(a, b));
          } else {
            vec.set(x, y, val);
          }
        }
      }
    });
  }
  void applyOtf(CVec<T>& vec, int band, double kx, double ky) const { otfToVector(vec, band, kx, ky, useAtt, false); }
  void writeOtfVector(CVec<T>& vec, int band, double kx, double ky) const {
    otfToVector(vec, band, kx, ky, false, true);
  }
  void writeOtfWithAttVector(CVec<T>& vec, int band, double kx, double ky) const {
    otfToVector(vec, band, kx, ky, useAtt, true);
  }
  // writeApoVector, real form (S/OtfProvider.java:469-492)
  void writeApoVector(RVec<T>& vec, double bend, double cutoffFac) const {
    const int w = vec.w, h = vec.h;
    pfor(0, h, [&](int y) {
      for (int x = 0; x < w; x++) {
        double xh = (x < w / 2) ? x : x - w;
        double yh = (y < h / 2) ? -y : h - y;
        double rad = fhypot(xh, yh);
        double cycl = rad * vecCyclesPerMicron;
        double frac = cycl / (cutOff * cutoffFac);
        double val = std::pow(val_ideal_otf(frac), bend);
        vec.at(x, y) = rnd<T>(val);
      }
    });
  }
  // writeAttenuationVector (S/OtfProvider.java:503-529)
  void writeAttenuationVector(RVec<T>& out, double str, double fwhm, double kx, double ky) const {
    const int w = out.w, h = out.h;
    pfor(0, h, [&](int y) {
      for (int x = 0; x < w; x++) {
        double xh = (x < w / 2) ? x : x - w;
        double yh = (y < h / 2) ? -y : h - y;
        double rad = fhypot(xh - kx, yh - ky);
        out.at(x, y) = val_attenuation<T>(rad * vecCyclesPerMicron, str, fwhm);
      }
    });
  }
  void maskOtf(CVec<T>& vec, double kx, double ky) const {
    const int w = vec.w, h = vec.h;
    for (int y = 0; y < h; y++)
      for (int x = 0; x < w; x++) {
        double xh = (x < w / 2) ? x : x - w;
        double yh = (y < h / 2) ? -y : h - y;
        double rad = fhypot(xh - kx, yh - ky) * vecCyclesPerMicron;
        if (rad > cutOff) vec.set(x, y, {0, 0});
      }
  }
};

// ---------------------------------------------------------------------------
// SimParam (S/SimParam.java:31-615), 2D subset
// ---------------------------------------------------------------------------
struct Dir {
  int nrBands = 2, nrPhases = 3;
  double pX = 0, pY = 0, phaOff = 0;
  std::vector<double> phases, modul;
  Dir() = default;
  Dir(int nb, int np) : nrBands(nb), nrPhases(np), phases(np), modul(nb, 1.0) { resetPhases(); }
  void resetPhases() {
    for (int i = 0; i < nrPhases; i++) phases[i] = (2 * M_PI / nrPhases) * i;
  }
  void setPxPy(double x, double y) {
    pX = x / (nrBands - 1);
    pY = y / (nrBands - 1);
  }
  double px(int b) const { return pX * b; }
  double py(int b) const { return pY * b; }
  std::vector<double> getPhases() const {
    std::vector<double> r(nrPhases);
    for (int i = 0; i < nrPhases; i++) r[i] = phases[i] + phaOff;
    return r;
  }
  std::vector<double> getModulations(double lo = 0.3, double hi = 1.1) const {
    std::vector<double> r = modul;
    for (auto& m : r) {
      if (m < lo) m = lo;
      if (m > hi) m = hi;
    }
    return r;
  }
};

template <class T>
struct SimParam {
  int nrDirs = 3, nrBands = 2, nrPhases = 3;
  int imgSize = 0;
  double micronsPerPixel = 0, cyclesPerMicron = 0;
  double wiener = 0.05, apoCutOff = 2;
  int filterStyle = 0;  // SimParam.FilterStyle: 0 Wiener, 1 RLin, 2 RLout, 3 RLboth (S/SimParam.java:33-43)
  int rlIterations = 5;
  bool useWienerFilter() const { return filterStyle == 0 || filterStyle == 1; }  // S/SimParam.java:287-290
  bool useRLonInput() const { return filterStyle == 3 || filterStyle == 1; }     // :295-298
  bool useRLonOutput() const { return filterStyle == 3 || filterStyle == 2; }    // :301-304
  std::vector<Dir> dirs;
  Otf<T> otf;
  int vectorWidth() const { return imgSize; }
  void setPxlSize(int pxl, double microns) {
    imgSize = pxl;
    micronsPerPixel = microns;
    cyclesPerMicron = 1 / (pxl * microns);
    otf.vecCyclesPerMicron = cyclesPerMicron;
  }
};

// ---------------------------------------------------------------------------
// WienerFilter (S/WienerFilter.java:46-122)
// ---------------------------------------------------------------------------
template <class T>
inline void add_wiener_denominator(const SimParam<T>& sp, RVec<T>& vec, int d, int b, bool useAtt) {
  const int w = vec.w, h = vec.h;
  const Dir& dir = sp.dirs[d];
  const double cyclMicron = sp.cyclesPerMicron;
  pfor(0, h, [&](int y) {
    for (int x = 0; x < w; x++) {
      double xh = (x < w / 2) ? x : x - w;
      double yh = (y < h / 2) ? -y : h - y;
      double rad1 = fhypot(xh - dir.px(b), yh - dir.py(b)) * cyclMicron;
      double rad2 = fhypot(xh + dir.px(b), yh + dir.py(b)) * cyclMicron;
      C<T> o1 = sp.otf.getOtfVal(b, rad1, false), o2 = sp.otf.getOtfVal(b, rad2, false);
      T v1 = o1.re * o1.re + o1.im * o1.im, v2 = o2.re * o2.re + o2.im * o2.im;  // Cplx.Float.absSq
      if (useAtt) {
        v1 *= sp.otf.getAttVal(b, rad1);
        v2 *= sp.otf.getAttVal(b, rad2);
      }
      vec.at(x, y) = vec.at(x, y) + v1 + v2;
    }
  });
}
template <class T>
inline RVec<T> wiener_denominator(const SimParam<T>& sp, double wParam) {
  const int w = sp.imgSize;
  RVec<T> wd(2 * w, 2 * w);
  for (int d = 0; d < sp.nrDirs; d++)
    for (int b = 0; b < sp.nrBands; b++) add_wiener_denominator(sp, wd, d, b, sp.otf.useAtt);
  T wp = rnd<T>(wParam * wParam);
  for (auto& v : wd.d) v = T(1) / (v + wp);
  return wd;
}

// ---------------------------------------------------------------------------
// SimUtils (S/SimUtils.java:33-264)
// ---------------------------------------------------------------------------
template <class T>
inline void fade_border_cos(RVec<T>& img, int px) {
  const int w = img.w, h = img.h;
  const double fac = 1. / px * M_PI / 2.;
  for (int y = 0; y < px; y++)
    for (int x = 0; x < w; x++) img.at(x, y) = rnd<T>(img.at(x, y) * std::pow(std::sin(y * fac), 2));
  for (int y = h - px; y < h; y++)
    for (int x = 0; x < w; x++) img.at(x, y) = rnd<T>(img.at(x, y) * std::pow(std::sin((h - y - 1) * fac), 2));
  for (int y = 0; y < h; y++)
    for (int x = 0; x < px; x++) img.at(x, y) = rnd<T>(img.at(x, y) * std::pow(std::sin(x * fac), 2));
  for (int y = 0; y < h; y++)
    for (int x = w - px; x < w; x++) img.at(x, y) = rnd<T>(img.at(x, y) * std::pow(std::sin((w - x - 1) * fac), 2));
}
// fourierShift via real space (S/SimUtils.java:43-50)
template <class T>
inline void sim_fourier_shift(CVec<T>& v, double kx, double ky) {
  fft2d(v, true);
  fourier_shift(v, kx, -ky);
  fft2d(v, false);
}
// pasteAndFourierShift (S/SimUtils.java:65-91); modifies inV in fast mode
template <class T>
inline void paste_and_fourier_shift(CVec<T>& inV, CVec<T>& outV, double kx, double ky, bool fast) {
  if (!fast) {
    paste_freq(outV, inV, 0, 0);
    fft2d(outV, true);
    fourier_shift(outV, kx, -ky);
    fft2d(outV, false);
  } else {
    double xFrac = kx - std::floor(kx);
    double yFrac = -ky - std::floor(-ky);
    fft2d(inV, true);
    fourier_shift(inV, xFrac, yFrac);
    fft2d(inV, false);
    int xInt = (int)std::floor(kx);
    int yInt = (int)std::floor(-ky);
    paste_freq(outV, inV, xInt, yInt);
  }
}
// spatial(): inverse FFT of a copy, real part (S/SimUtils.java:124-130)
template <class T>
inline RVec<T> spatial(const CVec<T>& in) {
  CVec<T> tmp = in;
  fft2d(tmp, true);
  RVec<T> out(in.w, in.h);
  for (size_t i = 0; i < out.d.size(); i++) out.d[i] = tmp.d[2 * i];
  return out;
}
// clipAndScale (S/SimUtils.java:244-264)
template <class T>
inline void clip_and_scale(RVec<T>& v, bool clip, bool scale) {
  if (scale) {
    T mx = 0;
    for (auto x : v.d)
      if (x > mx) mx = x;
    T f = T(255) / mx;
    for (auto& x : v.d) x *= f;
  }
  if (clip)
    for (auto& x : v.d)
      if (x < 0) x = 0;
}

// ---------------------------------------------------------------------------
// RLDeconvolution.deconvolve (S/RLDeconvolution.java:45-103): u_{j+1} = u_j x [(d / (u_j * psf)) * psf]
// with the convolutions as products with `otf` in frequency space; starting guess u_0 = d.
// ---------------------------------------------------------------------------
template <class T>
inline void rl_deconvolve(CVec<T>& img, const CVec<T>& otf, int steps, bool inputIsInFreqSpace) {
  if (inputIsInFreqSpace) fft2d(img, true);
  CVec<T> deconv = img, next = img;
  for (int i = 0; i < steps; i++) {
    fft2d(next, false);
    v_times(next, otf, false);
    fft2d(next, true);
    v_reciproc(next);
    v_times(next, img, false);
    fft2d(next, false);
    v_times(next, otf, false);
    fft2d(next, true);
    v_times(next, deconv, false);
    deconv = next;
  }
  img = deconv;
  if (inputIsInFreqSpace) fft2d(img, false);
}

// ---------------------------------------------------------------------------
// SimAlgorithm.runReconstruction (S/SimAlgorithm.java:268-686): Wiener path, RL on the input
// (RLin / RLboth, :318-361), RL on the output with the effective SIM OTF (RLout / RLboth, :587-641)
// clipScale: 0 NONE, 1 CLIP, 2 BOTH
// ---------------------------------------------------------------------------
template <class T>
inline RVec<T> run_reconstruction(const SimParam<T>& param, const std::vector<std::vector<CVec<T>>>& inFFT,
                                  bool otfBeforeShift, int clipScale, double apoBend = .9) {
  const int w = inFFT[0][0].w, h = inFFT[0][0].h;
  const double apoB = apoBend, apoF = param.apoCutOff;
  const Otf<T>& otf = param.otf;
  RVec<T> denom = wiener_denominator(param, param.wiener);
  CVec<T> fullResult(2 * w, 2 * h);
  const bool useWiener = param.useWienerFilter();
  CVec<T> inputOtf;  // zero-band OTF for RL on the input (:313-321)
  if (param.useRLonInput()) {
    inputOtf = CVec<T>(w, h);
    otf.writeOtfVector(inputOtf, 0, 0, 0);
  }
  for (int a = 0; a < param.nrDirs; a++) {
    const Dir& par = param.dirs[a];
    int nc = par.nrBands * 2 - 1;
    std::vector<CVec<T>> sep(nc, CVec<T>(w, h));
    if (param.useRLonInput()) {
      // the reference deconvolves the first nrBand*2-1 input images only and separates those
      // (:331-354): with more phases than components, separateBands throws
      if ((int)inFFT[a].size() != nc) throw std::runtime_error("#input images != phases per band");
      std::vector<CVec<T>> tmp(inFFT[a].begin(), inFFT[a].begin() + nc);
      for (int i = 0; i < nc; i++) rl_deconvolve(tmp[i], inputOtf, param.rlIterations, true);
      separate_bands(tmp, sep, par.getPhases(), par.nrBands, par.getModulations());
    } else {
      separate_bands(inFFT[a], sep, par.getPhases(), par.nrBands, par.getModulations());
    }
    if (otfBeforeShift && useWiener)
      for (int i = 0; i < nc; i++) otf.applyOtf(sep[i], (i + 1) / 2, 0, 0);
    std::vector<CVec<T>> shifted(std::max(5, nc), CVec<T>(2 * w, 2 * h));
    paste_freq(shifted[0], sep[0], 0, 0);
    for (int b = 1; b < par.nrBands; b++) {
      int pos = b * 2, neg = b * 2 - 1;
      paste_freq(shifted[pos], sep[pos], 0, 0);
      paste_freq(shifted[neg], sep[neg], 0, 0);
      sim_fourier_shift(shifted[pos], par.px(b), par.py(b));
      sim_fourier_shift(shifted[neg], -par.px(b), -par.py(b));
    }
    if (useWiener && !otfBeforeShift) {
      otf.applyOtf(shifted[0], 0, 0, 0);
      for (int b = 1; b < par.nrBands; b++) {
        int pos = b * 2, neg = b * 2 - 1;
        otf.applyOtf(shifted[pos], b, par.px(b), par.py(b));
        otf.applyOtf(shifted[neg], b, -par.px(b), -par.py(b));
      }
    } else if (useWiener) {
      // the reference passes (angIdx, component) as the mask centre (S/SimAlgorithm.java:407-409)
      for (int i = 0; i < nc; i++) otf.maskOtf(shifted[i], a, i);
    }
    if (param.useRLonOutput()) v_scal(shifted[0], rnd<T>(1.0 / param.nrDirs));  // scal(1.f / nrDir())
    for (int i = 0; i < nc; i++) v_add(fullResult, shifted[i]);
  }
  if (!useWiener) {
    // RL on the output with the effective SIM OTF: band 0 once (1/nrDir per direction), the
    // other bands at +-k of every direction (S/SimAlgorithm.java:591-611, 630-631)
    CVec<T> otfSim(2 * w, 2 * h), pos(2 * w, 2 * h), neg(2 * w, 2 * h);
    for (int a = 0; a < param.nrDirs; a++) {
      const Dir& par = param.dirs[a];
      for (int b = 0; b < par.nrBands; b++) {
        otf.writeOtfVector(pos, b, par.px(b), par.py(b));
        otf.writeOtfVector(neg, b, -par.px(b), -par.py(b));
        if (b == 0) {
          v_scal(pos, rnd<T>(1.0 / param.nrDirs));
          v_add(otfSim, pos);
        } else {
          v_add(otfSim, pos);
          v_add(otfSim, neg);
        }
      }
    }
    rl_deconvolve(fullResult, otfSim, param.rlIterations, true);
    RVec<T> res = spatial(fullResult);
    if (clipScale == 1) clip_and_scale(res, true, false);
    if (clipScale == 2) clip_and_scale(res, true, true);
    return res;
  }
  CVec<T> apo(2 * w, 2 * h);
  {
    RVec<T> apoR(2 * w, 2 * h);
    otf.writeApoVector(apoR, apoB, apoF);
    for (size_t i = 0; i < apoR.d.size(); i++) {
      apo.d[2 * i] = apoR.d[i];
      apo.d[2 * i + 1] = 0;
    }
  }
  v_times_real(fullResult, denom);
  v_times(fullResult, apo, false);
  RVec<T> res = spatial(fullResult);
  if (clipScale == 1) clip_and_scale(res, true, false);
  if (clipScale == 2) clip_and_scale(res, true, true);
  return res;
}

// WienerFilter.getWidefieldDenominator (S/WienerFilter.java:129-139): band 0 of direction 0,
// no attenuation, on the 2w x 2h grid, then 1/(v + (float)(w^2))
template <class T>
inline RVec<T> widefield_denominator(const SimParam<T>& sp, double wParam) {
  const int w = sp.imgSize;
  RVec<T> wd(2 * w, 2 * w);
  add_wiener_denominator(sp, wd, 0, 0, false);
  T wp = rnd<T>(wParam * wParam);
  for (auto& v : wd.d) v = T(1) / (v + wp);
  return wd;
}

// The two side outputs of runReconstruction's Wiener path (S/SimAlgorithm.java:533-576):
// "Widefield" = spatial(sum over directions of placeFreq(separated band 0)), and
// "filtered Widefield" = the same spectrum times conj(OTF band 0) (no attenuation), times the
// widefield Wiener denominator, masked to the OTF support, then spatial. clipScale as above.
template <class T>
inline void widefield_outputs(const SimParam<T>& param, const std::vector<std::vector<CVec<T>>>& inFFT,
                              int clipScale, RVec<T>& wf, RVec<T>& fwf) {
  const int w = inFFT[0][0].w, h = inFFT[0][0].h;
  CVec<T> low(2 * w, 2 * h);
  for (int a = 0; a < param.nrDirs; a++) {
    const Dir& par = param.dirs[a];
    std::vector<CVec<T>> sep(par.nrBands * 2 - 1, CVec<T>(w, h));
    separate_bands(inFFT[a], sep, par.getPhases(), par.nrBands, par.getModulations());
    CVec<T> tmp(2 * w, 2 * h);
    paste_freq(tmp, sep[0], 0, 0);
    v_add(low, tmp);
  }
  auto finish = [&](RVec<T>& r) {
    if (clipScale == 1) clip_and_scale(r, true, false);
    if (clipScale == 2) clip_and_scale(r, true, true);
  };
  wf = spatial(low);
  finish(wf);
  if (param.useRLonOutput()) {
    // RL styles: the widefield deconvolved with the zero-order OTF (S/SimAlgorithm.java:669-672)
    CVec<T> zeroOrderOtf(2 * w, 2 * h);
    param.otf.writeOtfVector(zeroOrderOtf, 0, 0, 0);
    rl_deconvolve(low, zeroOrderOtf, param.rlIterations, true);
  } else {
    param.otf.otfToVector(low, 0, 0, 0, false, false);
    v_times_real(low, widefield_denominator(param, param.wiener));
    param.otf.maskOtf(low, 0, 0);
  }
  fwf = spatial(low);
  finish(fwf);
}

// Correlation.autoCorrelation (S/Correlation.java:294-325): Wicker's non-iterative phase
// estimate. The band pasted to 2w, one copy shifted by (kx, ky), sum of a * conj(b) in double,
// divided by norm2 of the unshifted copy.
template <class T>
inline C<double> auto_correlation(const CVec<T>& inV, double kx, double ky) {
  const int N = inV.w * 2;
  CVec<T> aV(N, N), bV(N, N);
  paste_freq(aV, inV, 0, 0);
  paste_freq(bV, inV, 0, 0);
  sim_fourier_shift(bV, kx, ky);
  double re = 0, im = 0;
  for (size_t i = 0; i < aV.n(); i++) {
    const double ar = aV.d[2 * i], ai = aV.d[2 * i + 1], br = bV.d[2 * i], bi = -(double)bV.d[2 * i + 1];
    re += ar * br - ai * bi;
    im += ar * bi + ai * br;
  }
  const double n2 = v_norm2(aV);
  return {re / n2, im / n2};
}

// ---------------------------------------------------------------------------
// Correlation (S/Correlation.java:43-288)
// ---------------------------------------------------------------------------
template <class T>
inline void common_region(CVec<T>& band0, CVec<T>& band1, int bn0, int bn1, const Otf<T>& otf, double kx, double ky,
                          double dist, double weightLimit, bool divideByOtf) {
  const int w = band0.w, h = band0.h;
  CVec<T> weight0(w, h), weight1(w, h), wt0(w, h), wt1(w, h);
  otf.writeOtfVector(weight0, bn0, 0, 0);
  otf.writeOtfVector(weight1, bn1, 0, 0);
  otf.writeOtfVector(wt0, bn0, kx, ky);
  otf.writeOtfVector(wt1, bn1, -kx, -ky);
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      double rad = std::sqrt((double)(((x < w / 2) ? (x * x) : ((x - w) * (x - w))) +
                                      ((y < h / 2) ? (y * y) : ((y - h) * (y - h)))));
      double max = std::sqrt(kx * kx + ky * ky);
      double ratio = rad / max;
      if (cabs_f(weight0.get(x, y)) < weightLimit || cabs_f(wt0.get(x, y)) < weightLimit)
        band0.set(x, y, {0, 0});
      else if (divideByOtf)
        band0.set(x, y, cdiv(band0.get(x, y), weight0.get(x, y)));
      if (cabs_f(weight1.get(x, y)) < weightLimit || cabs_f(wt1.get(x, y)) < weightLimit)
        band1.set(x, y, {0, 0});
      else if (divideByOtf)
        band1.set(x, y, cdiv(band1.get(x, y), weight1.get(x, y)));
      if ((ratio < dist) || (ratio > (1 - dist))) {
        band0.set(x, y, {0, 0});
        band1.set((x - (int)kx + w) % w, (y + (int)ky + h) % h, {0, 0});
      }
    }
}

// locatePeak: returns {xPos, yPos, max, phase} (S/Correlation.java:144-167)
template <class T>
inline void locate_peak(const CVec<T>& vec, double kMin, double out[4]) {
  const int w = vec.w, h = vec.h;
  double xPos = -0., yPos = -1, max = -1, phase = 0;
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      double rad = std::sqrt((double)(((x < w / 2) ? (x * x) : ((x - w) * (x - w))) +
                                      ((y < h / 2) ? (y * y) : ((y - h) * (y - h)))));
      C<T> v = vec.get(x, y);
      double a = (double)cabs_f(v);
      if ((rad > kMin) && (a > max)) {
        max = a;
        xPos = x;
        yPos = y;
        phase = (double)(T)std::atan2((double)v.im, (double)v.re);
      }
    }
  if (xPos > w / 2) xPos = xPos - w;
  if (yPos > h / 2)
    yPos = h - yPos;
  else
    yPos *= -1;
  out[0] = xPos;
  out[1] = yPos;
  out[2] = max;
  out[3] = phase;
}

// fitPeak: 3 iterations of a 10x10 grid search (S/Correlation.java:43-136).
// grid_out (optional) receives 3*100*2 doubles: corr[iter][yi][xi] (re,im).
template <class T>
inline void fit_peak(const CVec<T>& band0, const CVec<T>& band1, int bn0, int bn1, const Otf<T>& otf, double kx,
                     double ky, double weightLimit, double search, double out[4], double* grid_out = nullptr) {
  double resPhase = 0, resMag = 0;
  for (int iter = 0; iter < 3; iter++) {
    CVec<T> b0 = band0, b1 = band1;
    common_region(b0, b1, bn0, bn1, otf, kx, ky, 0.15, weightLimit, true);
    fft2d(b0, true);
    fft2d(b1, true);
    C<double> corr[10][10];
    const double scal = 1. / v_norm2(b0);
    const double tkx = kx, tky = ky, ts = search;
    for (int p = 0; p < 100; p++) {
      int xi = p % 10, yi = p / 10;
      double xpos = tkx + ((xi - 4.5) / 4.5) * ts;
      double ypos = tky + ((yi - 4.5) / 4.5) * ts;
      CVec<T> b1s = b1;
      fourier_shift(b1s, xpos, -ypos);
      v_times(b1s, b0, true);
      C<double> s = v_sum(b1s);
      corr[xi][yi] = cmul(s, C<double>{scal, 0});
      if (grid_out) {
        grid_out[(iter * 100 + yi * 10 + xi) * 2] = corr[xi][yi].re;
        grid_out[(iter * 100 + yi * 10 + xi) * 2 + 1] = corr[xi][yi].im;
      }
    }
    double max = 0, newKx = 0, newKy = 0;
    for (int yi = 0; yi < 10; yi++)
      for (int xi = 0; xi < 10; xi++) {
        double hv = std::hypot(corr[xi][yi].re, corr[xi][yi].im);
        if (hv > max) {
          max = hv;
          newKx = tkx + ((xi - 4.5) / 4.5) * ts;
          newKy = tky + ((yi - 4.5) / 4.5) * ts;
          resPhase = std::atan2(corr[xi][yi].im, corr[xi][yi].re);
          resMag = hv;
        }
      }
    kx = newKx;
    ky = newKy;
    search /= 5;
  }
  out[0] = kx;
  out[1] = ky;
  out[2] = resPhase;
  out[3] = resMag;
}

// getPeak (S/Correlation.java:183-209)
template <class T>
inline C<double> get_peak(const CVec<T>& band0, const CVec<T>& band1, int bn0, int bn1, const Otf<T>& otf, double kx,
                          double ky, double weightLimit) {
  CVec<T> b0 = band0, b1 = band1;
  common_region(b0, b1, bn0, bn1, otf, kx, ky, 0.15, weightLimit, true);
  fft2d(b0, true);
  fft2d(b1, true);
  fourier_shift(b1, kx, -ky);
  v_times(b1, b0, true);
  const double scal = 1. / v_norm2(b0);
  return cmul(v_sum(b1), C<double>{scal, 0});
}

// ---------------------------------------------------------------------------
// SimAlgorithm.estimateParameters, 2- and 3-band forms (S/SimAlgorithm.java:37-159)
// Writes px,py (via setPxPy), phaOff and modulations into param. peaks_out (optional,
// nrDirs*4 doubles) receives the fitted [kx,ky,phase,mag] of each direction and
// coarse_out (optional, nrDirs*2) the integer locatePeak result.
// ---------------------------------------------------------------------------
template <class T>
inline void estimate_parameters(SimParam<T>& param, const std::vector<std::vector<CVec<T>>>& inFFT, int fitBand,
                                double fitExclude, double* peaks_out = nullptr, double* coarse_out = nullptr) {
  const int w = inFFT[0][0].w, h = inFFT[0][0].h;
  const Otf<T>& otfPr = param.otf;
  if (fitBand != 1 && fitBand != 2) throw std::runtime_error("Fitband neither 1 nor 2");
  RVec<T> otfAtt(w, h);
  otfPr.writeAttenuationVector(otfAtt, .99, 0.15 * otfPr.cutOff, 0, 0);
  for (int a = 0; a < param.nrDirs; a++) {
    Dir& dir = param.dirs[a];
    const int lb = 1;
    const int hb = (dir.nrBands == 3) ? 3 : 1;
    const int fb = (fitBand == 1) ? lb : hb;
    int nc = dir.nrBands * 2 - 1;
    std::vector<CVec<T>> sep(nc, CVec<T>(w, h));
    separate_bands_eq(inFFT[a], sep, 0, dir.nrBands, {});
    CVec<T> c0 = sep[0], c1 = sep[lb], c2 = sep[hb];
    v_times_real(c0, otfAtt);
    v_times_real(c1, otfAtt);
    v_times_real(c2, otfAtt);
    fft2d(c0, true);
    fft2d(c1, true);
    fft2d(c2, true);
    v_times(c1, c0, true);
    v_times(c2, c0, true);
    fft2d(c1, false);
    fft2d(c2, false);
    double minDist = fitExclude * otfPr.cutOff / param.cyclesPerMicron;
    double peak[4];
    locate_peak((fitBand == 1) ? c1 : c2, minDist, peak);
    if (coarse_out) {
      coarse_out[2 * a] = peak[0];
      coarse_out[2 * a + 1] = peak[1];
    }
    double fit[4];
    fit_peak(sep[0], sep[fb], 0, fitBand, otfPr, -peak[0], -peak[1], 0.05, 2.5, fit);
    if (lb != hb) {
      if (fitBand == 1) {
        fit[0] *= 2;
        fit[1] *= 2;
      }
      C<double> p1 = get_peak(sep[0], sep[lb], 0, 1, otfPr, fit[0] / 2, fit[1] / 2, 0.05);
      C<double> p2 = get_peak(sep[0], sep[hb], 0, 2, otfPr, fit[0], fit[1], 0.05);
      dir.setPxPy(-fit[0], -fit[1]);
      dir.phaOff = std::atan2(p1.im, p1.re);
      dir.modul[1] = std::hypot(p1.re, p1.im);
      dir.modul[2] = std::hypot(p2.re, p2.im);
    } else {
      C<double> p1 = get_peak(sep[0], sep[1], 0, 1, otfPr, fit[0], fit[1], 0.05);
      dir.setPxPy(-fit[0], -fit[1]);
      dir.phaOff = std::atan2(p1.im, p1.re);
      dir.modul[1] = std::hypot(p1.re, p1.im);
    }
    if (peaks_out) {
      peaks_out[4 * a + 0] = fit[0];
      peaks_out[4 * a + 1] = fit[1];
      peaks_out[4 * a + 2] = fit[2];
      peaks_out[4 * a + 3] = fit[3];
    }
  }
}

// ---------------------------------------------------------------------------
// Live path: ReconstructionThread.run for one channel and one stack
// (LM/ReconstructionRunner.java:434-542) with setupFilters (:773-813).
// raw: nrDirs*nrPhases frames of w*w unsigned 16-bit pixels, angle-major.
// ---------------------------------------------------------------------------
template <class T>
struct LiveFilters {
  RVec<T> damp, wien, apo;
  CVec<T> otfV;
};
template <class T>
inline LiveFilters<T> live_setup_filters(SimParam<T>& sp, bool useAtt, double attStr, double attFWHM,
                                         double wienParam) {
  const int w = sp.imgSize;
  LiveFilters<T> f;
  f.damp = RVec<T>(w, w);
  for (auto& v : f.damp.d) v += T(1);
  fade_border_cos(f.damp, 10);
  f.otfV = CVec<T>(w, w);
  sp.otf.setAttenuation(attStr, attFWHM);
  sp.otf.useAtt = useAtt;
  sp.otf.writeOtfWithAttVector(f.otfV, 0, 0, 0);
  f.wien = wiener_denominator(sp, wienParam);
  f.apo = RVec<T>(2 * w, 2 * w);
  sp.otf.writeApoVector(f.apo, 1, 2);
  return f;
}
template <class T>
inline void live_reconstruct(const SimParam<T>& sp, const LiveFilters<T>& f, const uint16_t* raw, T* out_recon,
                             T* out_widefield) {
  const int w = sp.imgSize;
  const int nA = sp.nrDirs, nP = sp.nrPhases;
  std::vector<std::vector<CVec<T>>> inFFT(nA, std::vector<CVec<T>>(nP, CVec<T>(w, w)));
  CVec<T> widefield(w, w), fullResult(2 * w, 2 * w);
  int count = 0;
  for (int a = 0; a < nA; a++)
    for (int p = 0; p < nP; p++) {
      const uint16_t* img = raw + (size_t)(count++) * w * w;
      CVec<T>& v = inFFT[a][p];
      for (size_t i = 0; i < v.n(); i++) {
        v.d[2 * i] = (T)(img[i] & 0xFFFF);
        v.d[2 * i + 1] = 0;
      }
      v_times_real(v, f.damp);
      v_add(widefield, v);
      fft2d(v, false);
    }
  v_scal(widefield, (T)(1.f / (nA * nP)));
  for (int a = 0; a < nA; a++) {
    const Dir& par = sp.dirs[a];
    int nc = par.nrBands * 2 - 1;
    std::vector<CVec<T>> sep(nc, CVec<T>(w, w));
    separate_bands(inFFT[a], sep, par.getPhases(), par.nrBands, par.getModulations());
    for (int i = 0; i < nc; i++) v_times(sep[i], f.otfV, true);
    std::vector<CVec<T>> shifted(nc, CVec<T>(2 * w, 2 * w));
    paste_freq(shifted[0], sep[0], 0, 0);
    for (int b = 1; b < par.nrBands; b++) {
      int pos = b * 2, neg = b * 2 - 1;
      paste_and_fourier_shift(sep[pos], shifted[pos], par.px(b), par.py(b), true);
      paste_and_fourier_shift(sep[neg], shifted[neg], -par.px(b), -par.py(b), true);
    }
    for (int i = 0; i < nc; i++) v_add(fullResult, shifted[i]);
  }
  v_times_real(fullResult, f.wien);
  v_times_real(fullResult, f.apo);
  fft2d(fullResult, true);
  if (out_recon)
    for (size_t i = 0; i < fullResult.n(); i++) out_recon[i] = fullResult.d[2 * i];
  if (out_widefield)
    for (size_t i = 0; i < widefield.n(); i++) out_widefield[i] = widefield.d[2 * i];
}

// ParameterRefitThread.doRefit (LM/ReconstructionRunner.java:642-746) on one stack.
template <class T>
inline void live_refit(SimParam<T>& sp, const uint16_t* raw, double* peaks_out = nullptr) {
  const int w = sp.imgSize, nA = sp.nrDirs, nP = sp.nrPhases;
  RVec<T> damp(w, w);
  for (auto& v : damp.d) v += T(1);
  fade_border_cos(damp, 10);
  std::vector<std::vector<CVec<T>>> inFFT(nA, std::vector<CVec<T>>(nP, CVec<T>(w, w)));
  int count = 0;
  for (int a = 0; a < nA; a++)
    for (int p = 0; p < nP; p++) {
      const uint16_t* img = raw + (size_t)(count++) * w * w;
      CVec<T>& v = inFFT[a][p];
      for (size_t i = 0; i < v.n(); i++) {
        v.d[2 * i] = (T)(img[i] & 0xFFFF);
        v.d[2 * i + 1] = 0;
      }
      v_times_real(v, damp);
      fft2d(v, false);
    }
  const Otf<T>& otfPr = sp.otf;
  for (int a = 0; a < sp.nrDirs; a++) {
    Dir& par = sp.dirs[a];
    int nc = par.nrBands * 2 - 1;
    std::vector<CVec<T>> sep(nc, CVec<T>(w, w));
    separate_bands_eq(inFFT[a], sep, 0, par.nrBands, {});
    const int lb = 1, hb = (par.nrBands == 3) ? 3 : 1;
    const int nBand = par.nrBands - 1;
    RVec<T> otfAtt(w, w);
    otfPr.writeAttenuationVector(otfAtt, .99, 0.15 * otfPr.cutOff, 0, 0);
    CVec<T> c0 = sep[0], c1 = sep[hb];
    v_times_real(c0, otfAtt);
    v_times_real(c1, otfAtt);
    fft2d(c0, true);
    fft2d(c1, true);
    v_times(c1, c0, true);
    fft2d(c1, false);
    double minDist = .8 * otfPr.cutOff / sp.cyclesPerMicron;
    double peak[4];
    locate_peak(c1, minDist, peak);
    double fit[4];
    fit_peak(sep[0], sep[hb], 0, 1, otfPr, -peak[0], -peak[1], 0.05, 2.5, fit);
    C<double> p1 = get_peak(sep[0], sep[lb], 0, 1, otfPr, fit[0] / nBand, fit[1] / nBand, 0.05);
    par.setPxPy(-fit[0], -fit[1]);
    par.phaOff = std::atan2(p1.im, p1.re);
    par.modul[1] = std::hypot(p1.re, p1.im);
    if (peaks_out) {
      for (int i = 0; i < 4; i++) peaks_out[4 * a + i] = fit[i];
    }
  }
}

}  // namespace ref
