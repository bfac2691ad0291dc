/*
 * TEST INFRASTRUCTURE ONLY (oracle recipe).
 *
 * FFTW3-API shim over the oracle's C2C transform (oracle/fft_c2c.c):
 * FFTW's conventions (row-major dims, sign -1 forward, unnormalised,
 * new-array execute with in == out) as its manual defines them.
 */
#include <stdlib.h>
#include <string.h>

#include "../fft_c2c.h"
#include "fftw3.h"

struct fipi_shim_plan {
    offt_plan* p;
    int sign;
    long n;
};

void* fftw_malloc(size_t n) {
    void* p = NULL;
    if (posix_memalign(&p, 64, n ? n : 1) != 0) return NULL;
    return p;
}

void fftw_free(void* p) { free(p); }

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out, int sign,
                           unsigned flags) {
    (void)in;
    (void)out;
    (void)flags;
    fftw_plan pl = (fftw_plan)calloc(1, sizeof(struct fipi_shim_plan));
    pl->p = offt_create(n0, n1, n2);
    pl->sign = sign;
    pl->n = (long)n0 * n1 * n2;
    return pl;
}

void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) {
    if (in != out) memcpy(out, in, sizeof(fftw_complex) * (size_t)p->n);
    offt_execute(p->p, (double*)out, p->sign);
}

void fftw_destroy_plan(fftw_plan p) {
    if (!p) return;
    offt_destroy(p->p);
    free(p);
}

int fftw_init_threads(void) { return 1; }

void fftw_plan_with_nthreads(int nthreads) { offt_set_threads(nthreads); }
