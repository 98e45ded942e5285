// Internal interface of the filter builders (filters.cu).
#pragma once

#include <mutex>

#include "common.cuh"
#include "otf.cuh"

namespace fsim {

struct ShiftSet {  // per-direction band-1 shifts
  int n_dirs, n_bands;
  double px[FSIM_MAX_DIRS], py[FSIM_MAX_DIRS];
};
ShiftSet shift_set(const fsim_sim_param* p);
// the band shifts (px[d] * b, py[d] * b) of a ShiftSet as float hi + lo (otf_pos_ff)
struct FShiftSet {
  FShift k[FSIM_MAX_DIRS][FSIM_MAX_BANDS];
};
FShiftSet fshift_set(const ShiftSet& s);
// The apodization (float)pow(valIdealOTF(hypot(x, y) * vec_cpm / cutoff_abs), bend) of
// OtfProvider.writeApoVector depends on |x| and |y| only, and symmetrically: it is
// evaluated in double once per point 0 <= j <= i <= n of one octant into q[i * (n + 1) + j]
// (bit-equal to the per-pixel evaluation; callers read q[max * (n + 1) + min]).
int apo_octant_device(float* q, int n, double vec_cpm, double cutoff_abs, double bend, cudaStream_t st);

constexpr int SEP_MAX_OUT = 2 * FSIM_MAX_BANDS - 1;
struct SepArgs {
  int n_in, n_out;
  const float2* in[FSIM_MAX_PHASES];
  float2* out[SEP_MAX_OUT];
  float2 coef[SEP_MAX_OUT * FSIM_MAX_PHASES];
};

// Stream-ordered upload of a SimParam's OTF table into the shared staging buffer; the
// caller holds otf_table_mutex() until the kernels that read the table are enqueued.
std::mutex& otf_table_mutex();
int upload_otf_table(const fsim_sim_param* p, OtfTable** dev, cudaStream_t st);
int wiener_denominator_device(float* out, const fsim_sim_param* p, double wiener, const OtfTable* t, bool reciprocal,
                              cudaStream_t st);
int apo_device(float* out, int cplx, int W, int H, double vec_cpm, double cutoff_abs, double bend, cudaStream_t st);
int att_device(float* out, int w, int h, double vec_cpm, double str, double fwhm, double kx, double ky, cudaStream_t st);
// otfToVector of band `band` (measured multi-band OTFs; estimates have one band)
int otf_vector_device(float2* v, int w, int h, const OtfTable* t, int band, double kx, double ky, bool att, bool write,
                      cudaStream_t st);
int separate_device(const SepArgs& a, size_t n, cudaStream_t st);

}  // namespace fsim
