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

__device__ __forceinline__ double ideal_otf_dev(double d) {
  if (d < 0 || d > 1) return 0;
  return (2 / M_PI) * (acos(d) - d * sqrt(1 - d * d));
}

}  // namespace fsim
