/*
 * TEST INFRASTRUCTURE ONLY (oracle recipe).
 *
 * The subset of the FFTW3 API that the reference calls (main.cpp:70-73,
 * field.cpp:41-46, 441, 451, 461), declared from FFTW3's public
 * documentation and implemented by fftw_shim.c on top of the oracle's own
 * C2C transform.  FFTW3 is an external dependency of the reference
 * (makefile:4, version not pinned there) and is not installed here.
 */
#ifndef FIPI_ORACLE_FFTW3_SHIM_H
#define FIPI_ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fipi_shim_plan* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

void* fftw_malloc(size_t n);
void fftw_free(void* p);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out, int sign,
                           unsigned flags);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_destroy_plan(fftw_plan p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);

#ifdef __cplusplus
}
#endif
#endif
