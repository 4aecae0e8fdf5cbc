/* Stand-in for the FFTW3 interface used by MG-PICOLA (reference test build only);
 * transforms are the oracle's FFTW-convention FFTs (oracle/orc_fft.c). */
#ifndef REF_SHIM_FFTW3_H
#define REF_SHIM_FFTW3_H
#include <stddef.h>
typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct ref_fftw_plan_s *fftw_plan;
typedef struct ref_fftw_plan_s *fftwf_plan;
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_MEASURE 0U
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#endif
