// Host-side SimParam logic (C++): phases, clamped modulations, band shifts and the
// band-separation matrix, as SimParam.Dir / BandSeparation / MatrixComplex define them.
#pragma once

#include <complex>
#include <vector>

#include "../../include/fairsim_gb300.h"

namespace fsim {

using cd = std::complex<double>;

// SimParam.Dir.getPhases (SimParam.java:472-477): explicit or 2*pi*i/nP, plus phaOff
std::vector<double> dir_phases(const fsim_sim_param* p, int d);
// SimParam.Dir.getModulations (SimParam.java:598-607): clamped to [0.3, 1.1]
std::vector<double> dir_modulations(const fsim_sim_param* p, int d);
inline double band_px(const fsim_sim_param* p, int d, int b) { return p->px[d] * b; }
inline double band_py(const fsim_sim_param* p, int d, int b) { return p->py[d] * b; }

// BandSeparation.createSeparationMatrix + separateBands' phase expansion
// (BandSeparation.java:40-114, 142-149). phases: band-1 phases; fac empty -> [1,.5,.5..].
// Returns the nC x nP inverse matrix (row-major), entries as doubles.
std::vector<cd> separation_matrix(const std::vector<double>& phases, int bands, std::vector<double> fac);

// separation coefficients of direction d in float (Cplx.Double.toFlt()), nC*nP entries
std::vector<std::complex<float>> separation_coeffs(const fsim_sim_param* p, int d, bool estimation);

int validate_param(const fsim_sim_param* p);

}  // namespace fsim
