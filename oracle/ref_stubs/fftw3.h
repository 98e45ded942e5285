/* Declarations of the few FFTW single-precision names that the reference's standard-C
 * vector backend refers to (its header includes fftw3.h; FFTW itself is not installed).
 * Defined in fftw_stub.c: allocation by malloc, and a transform that aborts (the oracle
 * pinning never calls the FFT natives). */
#ifndef FSIM_REF_STUB_FFTW3_H
#define FSIM_REF_STUB_FFTW3_H
#include <stddef.h>
typedef float fftwf_complex[2];
typedef struct fsim_fftwf_plan_s* fftwf_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
void* fftwf_malloc(size_t n);
void fftwf_free(void* p);
void* fftwf_alloc_complex(size_t n);
void fftwf_execute_dft(const fftwf_plan p, void* in, void* out);
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, void* in, void* out, int sign, unsigned flags);
#endif
