/* Stand-ins for the FFTW names the reference's standard-C backend links against (see
 * fftw3.h beside this file). Only allocation works; any transform aborts. */
#include <stdio.h>
#include <stdlib.h>
#include "fftw3.h"

void* fftwf_malloc(size_t n) { return malloc(n); }
void fftwf_free(void* p) { free(p); }
void* fftwf_alloc_complex(size_t n) { return malloc(n * sizeof(fftwf_complex)); }
void fftwf_execute_dft(const fftwf_plan p, void* in, void* out) {
  (void)p, (void)in, (void)out;
  fprintf(stderr, "fftw stub: transforms are not available\n");
  abort();
}
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, void* in, void* out, int sign, unsigned flags) {
  (void)n0, (void)n1, (void)in, (void)out, (void)sign, (void)flags;
  fprintf(stderr, "fftw stub: plans are not available\n");
  abort();
}
