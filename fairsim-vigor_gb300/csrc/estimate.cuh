// Internal interface of the device parameter estimation (estimate.cu, algo.cu).
#pragma once

#include <complex>
#include <vector>

#include "common.cuh"
#include "otf.cuh"

namespace fsim {

// Device scratch of one estimation (allocated stream-ordered; reused across calls).
struct FitState;  // fitPeak's iteration state on the device (estimate.cu)
constexpr int EST_PEAK_BLOCKS = 512;  // blocks of locatePeak's partial argmax
struct EstScratch {
  int n = 0;
  float2 *b0 = nullptr, *b1 = nullptr, *tx = nullptr, *ty = nullptr;
  double2 *Q = nullptr, *corr = nullptr;
  double* kbuf = nullptr;
  float* pmag = nullptr;
  int* pidx = nullptr;
  double* red = nullptr;  // reduction scratch (RED_SLOTS doubles): norms left on the device
  FitState* fit = nullptr;
  double* results = nullptr;  // per direction: fitPeak's kx, ky, phase, magnitude; getPeak's p1, p2
  int alloc(int N, cudaStream_t st);
  void free(cudaStream_t st);
};

// bn0 / bn1: the OTF bands of the two spectra (measured multi-band OTFs)
int common_region_device(float2* b0, float2* b1, int w, int h, const OtfTable* t, double kx, double ky, double dist,
                         double wl, bool divide, cudaStream_t st, int bn0 = 0, int bn1 = 1);
int locate_peak_device(const float2* v, int w, int h, double kmin, EstScratch& s, cudaStream_t st, double out4[4]);
// scal: the normaliser, or taken as 1 / *n2 when n2 (device) is not null
int corr_grid_device(const float2* b0, const float2* b1, int N, const double* kxs, int nx, const double* kys, int ny,
                     double scal, EstScratch& s, cudaStream_t st, std::vector<std::complex<double>>& out,
                     const double* n2 = nullptr);
int fit_peak_device(const float2* band0, const float2* band1, int N, const OtfTable* t, double kx, double ky, double wl,
                    double search, EstScratch& s, cudaStream_t st, double out4[4], double* grid_out, int bn0 = 0,
                    int bn1 = 1);
int get_peak_device(const float2* band0, const float2* band1, int N, const OtfTable* t, double kx, double ky, double wl,
                    EstScratch& s, cudaStream_t st, std::complex<double>* out, int bn0 = 0, int bn1 = 1);
// The same three steps without host round trips, chained through the device fit state:
// locatePeak leaves fitPeak's start (-peak) in it, fitPeak's result is stored at res[0..3],
// getPeak at (res[0], res[1]) * scale writes its correlation to out2 (two doubles).
int locate_peak_to_fit(const float2* v, int w, int h, double kmin, EstScratch& s, cudaStream_t st);
int fit_peak_iterate(const float2* band0, const float2* band1, int N, const OtfTable* t, double wl, EstScratch& s,
                     cudaStream_t st, double* res, int bn0 = 0, int bn1 = 1);
int get_peak_at_fit(const float2* band0, const float2* band1, int N, const OtfTable* t, double wl, EstScratch& s,
                    cudaStream_t st, const double* res, double scale, double* out2, int bn0 = 0, int bn1 = 1);

// SimAlgorithm.estimateParameters (live=false) or ParameterRefitThread.doRefit (live=true)
// on device spectra spec[a*nP + p] (N x N complex); updates p's shifts/phases/modulations.
int estimate_core(fsim_sim_param* p, const float2* const* spec, int fit_band, double fit_exclude, bool live,
                  double* peaks_out, cudaStream_t st);

}  // namespace fsim
