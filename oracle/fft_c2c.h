/*
 * TEST INFRASTRUCTURE ONLY (oracle).  Nothing in the product links this.
 *
 * In-place complex-to-complex 3-D DFT with FFTW3's documented conventions:
 * row-major dims (n0 slowest ... n2 fastest), forward sign -1, backward
 * sign +1, unnormalised.  The reference executes exactly this transform
 * through fftw_plan_dft_3d(Nz, Ny, Nx, ...) / fftw_execute_dft
 * (main.cpp:70-73, field.cpp:441,451).  Power-of-two sizes only.
 */
#ifndef ORACLE_FFT_C2C_H
#define ORACLE_FFT_C2C_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct offt_plan offt_plan;

offt_plan* offt_create(int n0, int n1, int n2);
void offt_destroy(offt_plan* p);
/* data: n0*n1*n2 interleaved (re, im) doubles. sign = -1 or +1. */
void offt_execute(const offt_plan* p, double* data, int sign);
/* Threads used by offt_execute (OpenMP); <= 0 means 1. */
void offt_set_threads(int n);
int offt_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
