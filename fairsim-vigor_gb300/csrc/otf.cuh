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

constexpr int OTF_SAMPLES = 512;  // OtfProvider.samplesLateral for estimates

struct OtfTable {
  double cutoff;          // cycles/micron, 1000/(lambda/na/2)
  double cycles_per_sample;  // OtfProvider.cyclesPerMicron = cutoff/512
  double vec_cpm;         // vector pixel size (SimParam cyclesPerMicron = 1/(w*pxl))
  float vals[OTF_SAMPLES];
  float vals_att[OTF_SAMPLES];
  float only_att[OTF_SAMPLES];
};

// host: OtfProvider.fromEstimate + setAttenuation (OtfProvider.java:96-127, 276-287)
void build_otf_table(const fsim_sim_param* p, OtfTable* t);
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

__device__ __forceinline__ double ideal_otf_dev(double d) {
  if (d < 0 || d > 1) return 0;
  return (2 / M_PI) * (acos(d) - d * sqrt(1 - d * d));
}

}  // namespace fsim
