/*
 * TEST INFRASTRUCTURE ONLY (oracle).  Nothing in the product links this.
 *
 * C2C 3-D DFT from the definition X[k] = sum_n x[n] exp(sign 2 pi i k n / N)
 * per axis, computed as an iterative radix-2 decimation-in-time FFT with
 * twiddles taken from libm cos/sin of the exact angle (no recurrences), so
 * the error grows like log2(N) ulps.  It stands in for FFTW3, which the
 * reference links (makefile:4) but which is not vendored with it.  Its
 * output is pinned against numpy.fft in the oracle's own tests.
 */
#include "fft_c2c.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define COLS 16 /* columns gathered per strided batch */

typedef struct {
    int n, log2n;
    int* rev;    /* bit reversal permutation */
    double* tw;  /* n/2 twiddles exp(-2 pi i k / n), interleaved */
} axis_plan;

struct offt_plan {
    int n[3];
    axis_plan ax[3];
};

static int g_threads = 1;

void offt_set_threads(int n) { g_threads = n > 0 ? n : 1; }
int offt_get_threads(void) { return g_threads; }

static int ilog2_exact(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return ((1 << l) == n) ? l : -1;
}

static int axis_init(axis_plan* a, int n) {
    a->n = n;
    a->log2n = ilog2_exact(n);
    if (a->log2n < 0) return -1;
    a->rev = (int*)malloc(sizeof(int) * (size_t)n);
    a->tw = (double*)malloc(sizeof(double) * (size_t)(n > 1 ? n : 2));
    for (int i = 0; i < n; ++i) {
        int r = 0;
        for (int b = 0; b < a->log2n; ++b)
            if (i & (1 << b)) r |= 1 << (a->log2n - 1 - b);
        a->rev[i] = r;
    }
    const double two_pi = 6.283185307179586476925286766559;
    for (int k = 0; k < n / 2; ++k) {
        double ang = two_pi * (double)k / (double)n;
        a->tw[2 * k] = cos(ang);
        a->tw[2 * k + 1] = -sin(ang);
    }
    return 0;
}

offt_plan* offt_create(int n0, int n1, int n2) {
    offt_plan* p = (offt_plan*)calloc(1, sizeof(offt_plan));
    p->n[0] = n0;
    p->n[1] = n1;
    p->n[2] = n2;
    for (int d = 0; d < 3; ++d) {
        if (axis_init(&p->ax[d], p->n[d]) != 0) {
            offt_destroy(p);
            return NULL;
        }
    }
    return p;
}

void offt_destroy(offt_plan* p) {
    if (!p) return;
    for (int d = 0; d < 3; ++d) {
        free(p->ax[d].rev);
        free(p->ax[d].tw);
    }
    free(p);
}

/* One contiguous 1-D transform of length a->n, in place. */
static void fft1d(const axis_plan* a, double* x, int sign) {
    const int n = a->n;
    for (int i = 0; i < n; ++i) {
        int j = a->rev[i];
        if (i < j) {
            double tr = x[2 * i], ti = x[2 * i + 1];
            x[2 * i] = x[2 * j];
            x[2 * i + 1] = x[2 * j + 1];
            x[2 * j] = tr;
            x[2 * j + 1] = ti;
        }
    }
    const double s = (sign < 0) ? 1.0 : -1.0; /* conjugate twiddles for sign +1 */
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1;
        const int step = n / len;
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < half; ++k) {
                const double wr = a->tw[2 * k * step];
                const double wi = s * a->tw[2 * k * step + 1];
                double* u = x + 2 * (i + k);
                double* v = x + 2 * (i + k + half);
                const double vr = v[0] * wr - v[1] * wi;
                const double vi = v[0] * wi + v[1] * wr;
                v[0] = u[0] - vr;
                v[1] = u[1] - vi;
                u[0] = u[0] + vr;
                u[1] = u[1] + vi;
            }
        }
    }
}

/* Transform along axis d of the row-major n0 x n1 x n2 array. */
static void axis_pass(const offt_plan* p, double* data, int d, int sign) {
    const int n0 = p->n[0], n1 = p->n[1], n2 = p->n[2];
    const axis_plan* a = &p->ax[d];
    if (a->n == 1) return;
    if (d == 2) {
        const long rows = (long)n0 * n1;
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (long r = 0; r < rows; ++r) fft1d(a, data + 2 * r * n2, sign);
        return;
    }
    /* strided axis: stride between successive elements along d */
    const long stride = (d == 1) ? (long)n2 : (long)n1 * n2;
    const long outer = (d == 1) ? (long)n0 : 1;          /* blocks above d   */
    const long inner = stride;                             /* columns below d  */
    const long outer_stride = (long)a->n * stride;
    const long nbatch = outer * ((inner + COLS - 1) / COLS);
#pragma omp parallel num_threads(g_threads)
    {
        double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)a->n * COLS);
#pragma omp for schedule(static)
        for (long b = 0; b < nbatch; ++b) {
            const long o = b / ((inner + COLS - 1) / COLS);
            const long c0 = (b % ((inner + COLS - 1) / COLS)) * COLS;
            const int nc = (int)((inner - c0) < COLS ? (inner - c0) : COLS);
            double* base = data + 2 * (o * outer_stride + c0);
            for (int e = 0; e < a->n; ++e)
                for (int c = 0; c < nc; ++c) {
                    buf[2 * ((long)c * a->n + e)] = base[2 * (e * stride + c)];
                    buf[2 * ((long)c * a->n + e) + 1] = base[2 * (e * stride + c) + 1];
                }
            for (int c = 0; c < nc; ++c) fft1d(a, buf + 2 * (long)c * a->n, sign);
            for (int e = 0; e < a->n; ++e)
                for (int c = 0; c < nc; ++c) {
                    base[2 * (e * stride + c)] = buf[2 * ((long)c * a->n + e)];
                    base[2 * (e * stride + c) + 1] = buf[2 * ((long)c * a->n + e) + 1];
                }
        }
        free(buf);
    }
}

void offt_execute(const offt_plan* p, double* data, int sign) {
    axis_pass(p, data, 2, sign);
    axis_pass(p, data, 1, sign);
    axis_pass(p, data, 0, sign);
}
