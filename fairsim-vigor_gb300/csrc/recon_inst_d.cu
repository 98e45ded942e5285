// Instantiations of the fused offline passes for sizes 2048 (one translation unit per
// group so the library builds in parallel).
#include "recon_kernels.cuh"

namespace fsim {
template int launch_offline<2048>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
}  // namespace fsim
