// OTF table and per-pixel lookups with the reference's exact arithmetic
// (org/fairsim/sim_algorithm/OtfProvider.java:74-559, WienerFilter.java:46-122).
//
// Radii are computed in double with explicitly rounded operations (no FMA contraction,
// as Java evaluates them) so that the floor-indexed sample of every pixel is the one the
// reference picks; the sample arithmetic v*(1-f) + v*f is done in float the same way.
#pragma once

#include <cmath>

#include "common.cuh"

namespace fsim {

constexpr int OTF_SAMPLES = 512;          // OtfProvider.samplesLateral for estimates
constexpr int OTF_MAX_MEASURED = 1024;    // samples per band of a measured OTF

struct OtfTable {
  double cutoff;          // cycles/micron, 1000/(lambda/na/2)
  double cycles_per_sample;  // OtfProvider.cyclesPerMicron (estimates: cutoff/512)
  double vec_cpm;         // vector pixel size (SimParam cyclesPerMicron = 1/(w*pxl))
  // the same constants as float hi + lo: vec_cpm, vec_cpm / cycles_per_sample, cutoff
  float ff_cpm[2], ff_pos[2], ff_cut[2];
  float vals[OTF_SAMPLES];   // estimate: one real band
  float vals_att[OTF_SAMPLES];
  float only_att[OTF_SAMPLES];
  // measured OTF (OtfProvider.loadFromConfig with band data): complex bands
  int measured, multi_band, n_bands, n_samples;
  float2 mvals[FSIM_MAX_BANDS][OTF_MAX_MEASURED];
  float2 mvals_att[FSIM_MAX_BANDS][OTF_MAX_MEASURED];
  float monly_att[FSIM_MAX_BANDS][OTF_MAX_MEASURED];
};

// host: OtfProvider.fromEstimate or the measured bands, + setAttenuation
// (OtfProvider.java:96-127, 588-621, 276-287)
void build_otf_table(const fsim_sim_param* p, OtfTable* t);
inline bool otf_measured(const fsim_sim_param* p) { return p->otf_data && p->otf_samples > 0; }
double ideal_otf_host(double d);

__device__ __forceinline__ double d_hypot_java(double x, double y) {  // MTool.fhypot
  return __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
}

// OtfProvider.getOtfVal (floor-indexed; java:189-222)
__device__ __forceinline__ float otf_val(const OtfTable& t, double cycl, bool att) {
  if (cycl >= t.cutoff) return 0.f;
  const double pos = cycl / t.cycles_per_sample;
  if (ceil(pos) >= (double)OTF_SAMPLES) return 0.f;
  const int l = (int)floor(pos);
  const float f = (float)(pos - (double)l);
  const float v = att ? t.vals_att[l] : t.vals[l];
  return __fadd_rn(__fmul_rn(v, __fsub_rn(1.f, f)), __fmul_rn(v, f));
}
// OtfProvider.getAttVal (java:246-269)
__device__ __forceinline__ float att_val(const OtfTable& t, double cycl) {
  if (cycl >= t.cutoff) return 1.f;
  const double pos = cycl / t.cycles_per_sample;
  const int l = (int)floor(pos);
  const float f = (float)(pos - (double)l);
  const float v = t.only_att[l];
  return __fadd_rn(__fmul_rn(v, f), __fmul_rn(v, __fsub_rn(1.f, f)));
}
// Band-aware complex lookups (measured OTFs; estimates give (otf_val, 0)): getOtfVal with
// the band index (bands collapse to 0 unless the OTF is multi-band) and the floor-indexed
// v*(1-f) + v*f per component (Cplx.add(v.mult(1-f), v.mult(f)))
__device__ __forceinline__ float2 otf_val_c(const OtfTable& t, int band, double cycl, bool att) {
  if (!t.measured) return make_float2(otf_val(t, cycl, att), 0.f);
  if (!t.multi_band) band = 0;
  if (cycl >= t.cutoff) return make_float2(0.f, 0.f);
  const double pos = cycl / t.cycles_per_sample;
  if (ceil(pos) >= (double)t.n_samples) return make_float2(0.f, 0.f);
  const int l = (int)floor(pos);
  const float f = (float)(pos - (double)l), g = __fsub_rn(1.f, f);
  const float2 v = att ? t.mvals_att[band][l] : t.mvals[band][l];
  return make_float2(__fadd_rn(__fmul_rn(v.x, g), __fmul_rn(v.x, f)), __fadd_rn(__fmul_rn(v.y, g), __fmul_rn(v.y, f)));
}
// getAttVal with the band index; a position beyond a measured table (the reference indexes
// outside its arrays there) reads as no attenuation
__device__ __forceinline__ float att_val_b(const OtfTable& t, int band, double cycl) {
  if (!t.measured) return att_val(t, cycl);
  if (!t.multi_band) band = 0;
  if (cycl >= t.cutoff) return 1.f;
  const double pos = cycl / t.cycles_per_sample;
  const int l = (int)floor(pos);
  if (l >= t.n_samples) return 1.f;
  const float f = (float)(pos - (double)l);
  const float v = t.monly_att[band][l];
  return __fadd_rn(__fmul_rn(v, f), __fmul_rn(v, __fsub_rn(1.f, f)));
}
__device__ __forceinline__ float abs_sq(float2 v) { return __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y)); }

// otfToVector's per-pixel value at frequency (xh, yh) for an OTF centred at (kx, ky);
// returns false where the reference writes zero (cycl > cutOff).
__device__ __forceinline__ bool otf_at(const OtfTable& t, double xh, double yh, double kx, double ky, bool att,
                                       float* val) {
  const double rad = d_hypot_java(__dsub_rn(xh, kx), __dsub_rn(yh, ky));
  const double cycl = __dmul_rn(rad, t.vec_cpm);
  if (cycl > t.cutoff) return false;
  *val = otf_val(t, cycl, att);
  return true;
}

__device__ __forceinline__ bool otf_at_c(const OtfTable& t, int band, double xh, double yh, double kx, double ky,
                                         bool att, float2* val) {
  const double rad = d_hypot_java(__dsub_rn(xh, kx), __dsub_rn(yh, ky));
  const double cycl = __dmul_rn(rad, t.vec_cpm);
  if (cycl > t.cutoff) return false;
  *val = otf_val_c(t, band, cycl, att);
  return true;
}

// ---- table positions in float-float arithmetic -----------------------------------------------
// The reference evaluates cycl = hypot(xh - kx, yh - ky) * vec_cpm and pos = cycl /
// cycles_per_sample in double and then branches on cycl >= cutoff and floor(pos). GB300 runs
// FP64 at a small fraction of its FP32 rate, so the plan builders and the fit's common region
// evaluate the same
// quantities as unevaluated sums of two floats (hi + lo, ~44 significant bits; error-free
// sum and FMA product steps, Dekker / Knuth): the absolute error of pos stays below 1e-9
// samples for |kx|, |ky| <= 4096 pixels, so every test the reference makes comes out the
// same unless its operand lies within 1e-8 of the test's boundary (pos within 1e-8 of an
// integer, cycl within 1e-8 relative of the cutoff). There `exact` is false and the caller
// takes the double-precision lookup. The interpolation weight f is the float rounding of
// pos - l from the float-float value; it can differ from the reference's in its last bit,
// which v*(1-f) + v*f (one sample, twice) absorbs except for a rare last-bit difference.
struct FShift {  // a shift as float hi + lo (hi = (float)k, lo = (float)(k - hi))
  float xh, xl, yh, yl;
};
__host__ __device__ inline FShift fshift_host(double kx, double ky) {
  FShift s;
  s.xh = (float)kx;
  s.xl = (float)(kx - (double)s.xh);
  s.yh = (float)ky;
  s.yl = (float)(ky - (double)s.yh);
  return s;
}
__device__ __forceinline__ FShift fshift_neg(FShift s) { return FShift{-s.xh, -s.xl, -s.yh, -s.yl}; }
__device__ __forceinline__ void ff_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// (h, l) * (ch, cl) for a positive constant; result renormalised
__device__ __forceinline__ void ff_mul(float h, float l, float ch, float cl, float& ph, float& pl) {
  const float p = __fmul_rn(h, ch);
  const float e = __fadd_rn(__fmaf_rn(h, ch, -p), __fadd_rn(__fmul_rn(h, cl), __fmul_rn(l, ch)));
  ff_two_sum(p, e, ph, pl);
}
struct OtfPos {
  int l;       // floor(pos)
  float f;     // (float)(pos - l)
  bool beyond; // cycl beyond the cutoff
  bool exact;  // false: within 1e-8 of a boundary, take the double-precision path
};
__device__ __forceinline__ OtfPos otf_pos_ff(const OtfTable& t, int xh, int yh, FShift k) {
  float s, e, dxh, dxl, dyh, dyl;
  ff_two_sum((float)xh, -k.xh, s, e);
  ff_two_sum(s, __fsub_rn(e, k.xl), dxh, dxl);
  ff_two_sum((float)yh, -k.yh, s, e);
  ff_two_sum(s, __fsub_rn(e, k.yl), dyh, dyl);
  // squared radius: dx^2 + dy^2 (the lo^2 terms are below the precision kept)
  const float px = __fmul_rn(dxh, dxh), py = __fmul_rn(dyh, dyh);
  const float ex = __fadd_rn(__fmaf_rn(dxh, dxh, -px), __fmul_rn(2.f * dxh, dxl));
  const float ey = __fadd_rn(__fmaf_rn(dyh, dyh, -py), __fmul_rn(2.f * dyh, dyl));
  float qh, ql;
  ff_two_sum(px, py, qh, ql);
  ff_two_sum(qh, __fadd_rn(ql, __fadd_rn(ex, ey)), qh, ql);
  // radius: one Newton correction of the correctly rounded sqrtf
  float rh = 0.f, rl = 0.f;
  if (qh > 0.f) {
    rh = __fsqrt_rn(qh);
    rl = __fdiv_rn(__fadd_rn(__fmaf_rn(-rh, rh, qh), ql), __fmul_rn(2.f, rh));
  }
  OtfPos o;
  float ch, cl, ph, pl;
  ff_mul(rh, rl, t.ff_cpm[0], t.ff_cpm[1], ch, cl);  // cycl
  const float cg = __fadd_rn(__fsub_rn(ch, t.ff_cut[0]), __fsub_rn(cl, t.ff_cut[1]));  // cycl - cutoff
  o.beyond = cg > 0.f;
  o.exact = fabsf(cg) > 1e-8f * t.ff_cut[0];
  ff_mul(rh, rl, t.ff_pos[0], t.ff_pos[1], ph, pl);  // pos
  float lf = floorf(ph);
  if (ph == lf && pl < 0.f) lf = __fsub_rn(lf, 1.f);
  const float lo = __fadd_rn(__fsub_rn(ph, lf), pl);                   // pos - l
  const float hi = __fsub_rn(__fsub_rn(__fadd_rn(lf, 1.f), ph), pl);   // l + 1 - pos
  o.exact = o.exact && (o.beyond || (lo > 1e-8f && hi > 1e-8f));
  o.l = (int)lf;
  o.f = lo;
  return o;
}
// getOtfVal / getAttVal (estimated table) from a position; exact positions only
__device__ __forceinline__ float otf_val_pos(const OtfTable& t, const OtfPos& o, bool att) {
  if (o.beyond || o.l + 1 >= OTF_SAMPLES) return 0.f;  // cycl >= cutoff, ceil(pos) >= samples
  const float v = att ? t.vals_att[o.l] : t.vals[o.l];
  return __fadd_rn(__fmul_rn(v, __fsub_rn(1.f, o.f)), __fmul_rn(v, o.f));
}
__device__ __forceinline__ float att_val_pos(const OtfTable& t, const OtfPos& o) {
  if (o.beyond) return 1.f;
  const float v = t.only_att[o.l];
  return __fadd_rn(__fmul_rn(v, o.f), __fmul_rn(v, __fsub_rn(1.f, o.f)));
}
// band-aware complex value and attenuation (measured tables), as otf_val_c / att_val_b
__device__ __forceinline__ float2 otf_val_c_pos(const OtfTable& t, int band, const OtfPos& o, bool att) {
  if (!t.measured) return make_float2(otf_val_pos(t, o, att), 0.f);
  if (!t.multi_band) band = 0;
  if (o.beyond || o.l + 1 >= t.n_samples) return make_float2(0.f, 0.f);
  const float f = o.f, g = __fsub_rn(1.f, f);
  const float2 v = att ? t.mvals_att[band][o.l] : t.mvals[band][o.l];
  return make_float2(__fadd_rn(__fmul_rn(v.x, g), __fmul_rn(v.x, f)), __fadd_rn(__fmul_rn(v.y, g), __fmul_rn(v.y, f)));
}
__device__ __forceinline__ float att_val_b_pos(const OtfTable& t, int band, const OtfPos& o) {
  if (!t.measured) return att_val_pos(t, o);
  if (!t.multi_band) band = 0;
  if (o.beyond || o.l >= t.n_samples) return 1.f;
  const float v = t.monly_att[band][o.l];
  return __fadd_rn(__fmul_rn(v, o.f), __fmul_rn(v, __fsub_rn(1.f, o.f)));
}
// |OTF_band|^2 (times the attenuation) at (xh - k) for the Wiener denominator: float-float
// position, double precision within 1e-8 of a boundary (WienerFilter.java:46-122)
__device__ __forceinline__ float wiener_term(const OtfTable& t, int band, int xh, int yh, FShift kf, double kx,
                                             double ky, bool use_att) {
  const OtfPos o = otf_pos_ff(t, xh, yh, kf);
  if (o.exact) {
    float v = abs_sq(otf_val_c_pos(t, band, o, false));
    return use_att ? __fmul_rn(v, att_val_b_pos(t, band, o)) : v;
  }
  const double r = __dmul_rn(d_hypot_java(__dsub_rn((double)xh, kx), __dsub_rn((double)yh, ky)), t.vec_cpm);
  float v = abs_sq(otf_val_c(t, band, r, false));
  return use_att ? __fmul_rn(v, att_val_b(t, band, r)) : v;
}
// otf_at / otf_at_c through the float-float position (false: zero is written)
__device__ __forceinline__ bool otf_at_fast(const OtfTable& t, int band, int xh, int yh, FShift kf, double kx, double ky,
                                            bool att, float2* val) {
  const OtfPos o = otf_pos_ff(t, xh, yh, kf);
  if (o.exact) {
    if (o.beyond) return false;
    *val = otf_val_c_pos(t, band, o, att);
    return true;
  }
  return otf_at_c(t, band, (double)xh, (double)yh, kx, ky, att, val);
}

// OtfProvider.valIdealOTF with Java's separately rounded operations: near d = 1 the two
// terms cancel to ~(1-d)^1.5, so an FMA-contracted 1 - d*d (the compiler's default in
// device code) moves the result by up to 1e-4 relative
__device__ __forceinline__ double ideal_otf_dev(double d) {
  if (d < 0 || d > 1) return 0;
  const double s = __dsqrt_rn(__dsub_rn(1.0, __dmul_rn(d, d)));
  return __dmul_rn(2 / M_PI, __dsub_rn(acos(d), __dmul_rn(d, s)));
}

}  // namespace fsim
