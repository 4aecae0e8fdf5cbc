#ifndef REF_SHIM_FFTW3_MPI_H
#define REF_SHIM_FFTW3_MPI_H
#include "fftw3.h"
#include "mpi.h"
void fftw_mpi_init(void);
void fftw_mpi_cleanup(void);
ptrdiff_t fftw_mpi_local_size_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, MPI_Comm c, ptrdiff_t *local_n0,
                                 ptrdiff_t *local_0_start);
fftw_plan fftw_mpi_plan_dft_r2c_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, double *in, fftw_complex *out,
                                   MPI_Comm c, unsigned flags);
fftw_plan fftw_mpi_plan_dft_c2r_3d(ptrdiff_t n0, ptrdiff_t n1, ptrdiff_t n2, fftw_complex *in, double *out,
                                   MPI_Comm c, unsigned flags);
#endif
