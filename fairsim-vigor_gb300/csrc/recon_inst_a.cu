// Instantiations of the fused offline passes for sizes 64, 128, 192, 256, 384 (one translation unit per
// group so the library builds in parallel).
#include "recon_kernels.cuh"

namespace fsim {
template int launch_offline<64>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
template int launch_offline<128>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
template int launch_offline<192>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
template int launch_offline<256>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
template int launch_offline<384>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
}  // namespace fsim
