/*
 * TEST INFRASTRUCTURE ONLY (oracle).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load this; the product never does.
 *
 * Plain-C FP64 restatement of the reference FIPI step.  Fields are full
 * complex C2C arrays (field.cpp:41-46) so the reference's imaginary-part
 * bookkeeping, its Nyquist handling and its x/0 -> 0 division survive.
 * Each block cites the reference statement it restates and keeps that
 * statement's evaluation order; the file is compiled with
 * -ffp-contract=off so no multiply-add is fused on any host (the reference
 * build has no FMA on x86-64).
 *
 * Where the reference is undefined or random, the oracle picks a defined
 * behaviour and the GPU library picks the same one:
 *  - grid index floor(x/dx) == N (x within an ulp of L) wraps to 0
 *    (field.cpp:229-245 and cluster.cpp:360-403 read out of bounds);
 *  - coincident particles (|d| == 0, cluster.cpp:234-242 draws rand())
 *    get the separation of coincident_d() below.
 */
#include "fipi_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fft_c2c.h"

struct oracle {
    fipi_params P;
    long V;
    offt_plan* plan;
    /* complex fields, interleaved (re, im) */
    double *c, *c_new, *c_old, *f, *f_old, *conv, *conv_old, *pch;
    double *grad[3], *u[3], *ftot[3], *fr[3];
    double *kx, *ky, *kz; /* wave numbers per axis (field.cpp:100-121) */
    /* particles (element.hpp:28-58), n x 3 particle-major */
    int n;
    double *p, *p_old, *up, *u_old, *f_pp, *f_pi, *f_ext, *c_loc, *dcdx, *r, *cth;
    int *keys, *sorted, *offsets;
    int it_mark;
    double tau;
    int t;
    /* extensions (off: the reference's particle model) */
    int couple;
    double kt;
    unsigned long long seed;
    double *uf, *f_rand; /* n x 3 */
    /* mass-conserving mode of the library (not in the reference): the k = 0
     * mode of the advection spectrum taken as 0 */
    int conserve;
};

void oracle_set_threads(int n) { offt_set_threads(n); }

static double* cfield(long V) { return (double*)calloc((size_t)(2 * V), sizeof(double)); }

/* field.cpp:100-121: k_i = i 2 pi / L for i <= N/2, else (i - N) 2 pi / L. */
static double* wave_numbers(int n, double L, double pi) {
    double* k = (double*)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) k[i] = (i <= n / 2) ? i * 2.0 * pi / L : (i - n) * 2.0 * pi / L;
    return k;
}

static int is_pow2(int n) { return n >= 2 && (n & (n - 1)) == 0; }

int oracle_params_ok(const fipi_params* P) {
    if (!is_pow2(P->nx) || !is_pow2(P->ny) || !is_pow2(P->nz)) return 0;
    if (P->n_p < 0) return 0;
    if (P->n_p > 0 && P->switch_particle) {
        int nc[3];
        double dc[3];
        oracle_cell_geometry(P, nc, dc);
        if (nc[0] < 3 || nc[1] < 3 || nc[2] < 3) return 0;
    }
    return 1;
}

oracle* oracle_create(const fipi_params* P) {
    if (!oracle_params_ok(P)) return NULL;
    oracle* o = (oracle*)calloc(1, sizeof(oracle));
    o->P = *P;
    o->V = (long)P->nx * P->ny * P->nz;
    o->plan = offt_create(P->nz, P->ny, P->nx); /* main.cpp:72-73 plan dims (Nz,Ny,Nx) */
    if (!o->plan) {
        free(o);
        return NULL;
    }
    const long V = o->V;
    o->c = cfield(V);
    o->c_new = cfield(V);
    o->c_old = cfield(V);
    o->f = cfield(V);
    o->f_old = cfield(V);
    o->conv = cfield(V);
    o->conv_old = cfield(V);
    o->pch = cfield(V);
    for (int d = 0; d < 3; ++d) {
        o->grad[d] = cfield(V);
        o->u[d] = cfield(V);
        o->ftot[d] = cfield(V);
        o->fr[d] = cfield(V);
    }
    o->kx = wave_numbers(P->nx, P->lx, P->pi);
    o->ky = wave_numbers(P->ny, P->ly, P->pi);
    o->kz = wave_numbers(P->nz, P->lz, P->pi);
    const int n = P->n_p;
    o->n = n;
    size_t n3 = (size_t)(n > 0 ? n : 1) * 3;
    o->p = (double*)calloc(n3, sizeof(double));
    o->p_old = (double*)calloc(n3, sizeof(double));
    o->up = (double*)calloc(n3, sizeof(double));
    o->u_old = (double*)calloc(n3, sizeof(double));
    o->uf = (double*)calloc(n3, sizeof(double));
    o->f_rand = (double*)calloc(n3, sizeof(double));
    o->f_pp = (double*)calloc(n3, sizeof(double));
    o->f_pi = (double*)calloc(n3, sizeof(double));
    o->f_ext = (double*)calloc(n3, sizeof(double));
    o->dcdx = (double*)calloc(n3, sizeof(double));
    o->c_loc = (double*)calloc(n3 / 3, sizeof(double));
    o->r = (double*)calloc(n3 / 3, sizeof(double));
    o->cth = (double*)calloc(n3 / 3, sizeof(double));
    for (int i = 0; i < n; ++i) {
        o->r[i] = P->r_p;  /* element.cpp:25 */
        o->c_loc[i] = 1.0; /* element.cpp:34 */
    }
    int nc[3];
    double dc[3];
    oracle_cell_geometry(P, nc, dc);
    o->keys = (int*)calloc(n3 / 3, sizeof(int));
    o->sorted = (int*)calloc(n3 / 3, sizeof(int));
    o->offsets = (int*)calloc((size_t)nc[0] * nc[1] * nc[2] + 1, sizeof(int));
    o->it_mark = -1; /* cluster.cpp:39 */
    o->tau = 0.0;
    o->t = 0;
    return o;
}

void oracle_destroy(oracle* o) {
    if (!o) return;
    offt_destroy(o->plan);
    double* all[] = {o->c, o->c_new, o->c_old, o->f, o->f_old, o->conv, o->conv_old, o->pch,
                     o->kx, o->ky, o->kz, o->p, o->p_old, o->up, o->u_old, o->f_pp, o->f_pi,
                     o->f_ext, o->c_loc, o->dcdx, o->r, o->cth, o->uf, o->f_rand};
    for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); ++i) free(all[i]);
    for (int d = 0; d < 3; ++d) {
        free(o->grad[d]);
        free(o->u[d]);
        free(o->ftot[d]);
        free(o->fr[d]);
    }
    free(o->keys);
    free(o->sorted);
    free(o->offsets);
    free(o);
}

/* ------------------------------------------------------------ state I/O */
int oracle_set_phase(oracle* o, const double* c) {
    for (long it = 0; it < o->V; ++it) {
        o->c[2 * it] = c[it];
        o->c[2 * it + 1] = 0.0;
    }
    o->t = 0;
    return FIPI_OK;
}

int oracle_set_velocity(oracle* o, const double* u) {
    for (int d = 0; d < 3; ++d)
        for (long it = 0; it < o->V; ++it) {
            o->u[d][2 * it] = u[d * o->V + it];
            o->u[d][2 * it + 1] = 0.0;
        }
    return FIPI_OK;
}

int oracle_set_particles(oracle* o, const double* p, const double* r, const double* cth,
                         const double* f_pp) {
    for (int i = 0; i < o->n; ++i) {
        for (int a = 0; a < 3; ++a) {
            o->p[3 * i + a] = p[3 * i + a];
            o->p_old[3 * i + a] = p[3 * i + a]; /* cluster.cpp:88 */
            o->f_pp[3 * i + a] = f_pp ? f_pp[3 * i + a] : 0.0;
        }
        o->r[i] = r ? r[i] : o->P.r_p;
        o->cth[i] = cth ? cth[i] : 0.0;
    }
    return FIPI_OK;
}

void oracle_get_phase(const oracle* o, double* c) {
    for (long it = 0; it < o->V; ++it) c[it] = o->c[2 * it];
}
void oracle_get_phase_imag(const oracle* o, double* c) {
    for (long it = 0; it < o->V; ++it) c[it] = o->c[2 * it + 1];
}
void oracle_get_velocity(const oracle* o, double* u) {
    for (int d = 0; d < 3; ++d)
        for (long it = 0; it < o->V; ++it) u[d * o->V + it] = o->u[d][2 * it];
}
void oracle_get_grad(const oracle* o, double* g) {
    for (int d = 0; d < 3; ++d)
        for (long it = 0; it < o->V; ++it) g[d * o->V + it] = o->grad[d][2 * it];
}
void oracle_get_particles(const oracle* o, double* p, double* f_pp, double* f_pi) {
    size_t b = sizeof(double) * 3 * (size_t)o->n;
    if (p) memcpy(p, o->p, b);
    if (f_pp) memcpy(f_pp, o->f_pp, b);
    if (f_pi) memcpy(f_pi, o->f_pi, b);
}
double oracle_tau(const oracle* o) { return o->tau; }
int oracle_time(const oracle* o) { return o->t; }

/* ------------------------------------------------------------ transforms */
void oracle_fft3(const fipi_params* P, double* data, int sign) {
    offt_plan* pl = offt_create(P->nz, P->ny, P->nx);
    offt_execute(pl, data, sign);
    offt_destroy(pl);
}

/* field::fft (field.cpp:438-443) */
static void fft(oracle* o, double* a) { offt_execute(o->plan, a, -1); }

/* field::ifft + normalize (field.cpp:446-455, primitive.cpp:54-62) */
static void ifft(oracle* o, double* a) {
    offt_execute(o->plan, a, +1);
    const int nn = o->P.nx * o->P.ny * o->P.nz;
    for (long it = 0; it < o->V; ++it) {
        a[2 * it] /= nn;
        a[2 * it + 1] /= nn;
    }
}

/* field::power(b) (field.cpp:408-431) receives its exponent at run time, so
 * the reference calls libm pow() even for b = 2; calling through a volatile
 * pointer keeps the compiler from folding pow(x, 2.0) into x*x here. */
static double (*volatile field_pow)(double, double) = pow;

#define IDX_I(o, it) ((int)((it) % (o)->P.nx))
#define IDX_J(o, it) ((int)(((it) / (o)->P.nx) % (o)->P.ny))
#define IDX_K(o, it) ((int)((it) / ((long)(o)->P.nx * (o)->P.ny)))

/* kf2 = kf.power(2.0) (main.cpp:31, field.cpp:408-431): sum of squares
 * accumulated from 0.0 in component order. */
static inline double kf2_at(const oracle* o, long it) {
    double kx = o->kx[IDX_I(o, it)], ky = o->ky[IDX_J(o, it)], kz = o->kz[IDX_K(o, it)];
    double s = 0.0;
    s += field_pow(kx, 2.0);
    s += field_pow(ky, 2.0);
    s += field_pow(kz, 2.0);
    return s;
}

/* field::grad (field.cpp:288-328) of the spectral scalar a into g[3]:
 * component d is i k_d a, zeroed where the index along d equals N_d/2. */
static void grad_spectral(oracle* o, const double* a, double* g[3]) {
    const fipi_params* P = &o->P;
    for (long it = 0; it < o->V; ++it) {
        const int i = IDX_I(o, it), j = IDX_J(o, it), k = IDX_K(o, it);
        const double kv[3] = {o->kx[i], o->ky[j], o->kz[k]};
        const int nyq[3] = {i == P->nx / 2, j == P->ny / 2, k == P->nz / 2};
        for (int d = 0; d < 3; ++d) {
            if (nyq[d]) {
                g[d][2 * it] = 0.0;
                g[d][2 * it + 1] = 0.0;
            } else {
                g[d][2 * it] = -kv[d] * a[2 * it + 1];
                g[d][2 * it + 1] = kv[d] * a[2 * it];
            }
        }
    }
}

/* c.fft; grad_c = c.grad(kf); grad_c.ifft  (main.cpp:190-192) on a real c. */
void oracle_grad(const fipi_params* P, const double* c, double* out) {
    oracle* o = oracle_create(P);
    if (!o) return;
    oracle_set_phase(o, c);
    fft(o, o->c);
    grad_spectral(o, o->c, o->grad);
    for (int d = 0; d < 3; ++d) ifft(o, o->grad[d]);
    oracle_get_grad(o, out);
    oracle_destroy(o);
}

/* field::div (field.cpp:332-361) of a real vector field v (3 x V): every
 * component transformed (field::fft), -k_d Im + i k_d Re accumulated over d
 * with no Nyquist zeroing, field::ifft, real part. */
void oracle_div(const fipi_params* P, const double* v, double* out) {
    oracle* o = oracle_create(P);
    if (!o) return;
    const long V = o->V;
    double* acc = (double*)calloc((size_t)(2 * V), sizeof(double));
    double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)V);
    for (int d = 0; d < 3; ++d) {
        for (long it = 0; it < V; ++it) {
            tmp[2 * it] = v[d * V + it];
            tmp[2 * it + 1] = 0.0;
        }
        fft(o, tmp);
        for (long it = 0; it < V; ++it) {
            const double k = d == 0 ? o->kx[IDX_I(o, it)] : (d == 1 ? o->ky[IDX_J(o, it)] : o->kz[IDX_K(o, it)]);
            acc[2 * it] += -k * tmp[2 * it + 1];
            acc[2 * it + 1] += k * tmp[2 * it];
        }
    }
    ifft(o, acc);
    for (long it = 0; it < V; ++it) out[it] = acc[2 * it];
    free(tmp);
    free(acc);
    oracle_destroy(o);
}

/* f = (lambda/sqr(epsilon))*(c.power(3.0)-c)  (main.cpp:81, 153) */
static void bulk_potential(oracle* o) {
    const double s = o->P.lambda / (o->P.epsilon * o->P.epsilon);
    for (long it = 0; it < o->V; ++it) {
        const double cr = o->c[2 * it];
        double pw = 0.0;
        pw += field_pow(cr, 3.0);    /* field::power accumulates from 0.0 */
        o->f[2 * it] = (pw - cr) * s; /* operator-, then operator*(double) */
        o->f[2 * it + 1] = 0.0;
    }
}

/* ------------------------------------------------------------- particles */
void oracle_cell_geometry(const fipi_params* P, int nc[3], double dc[3]) {
    /* cluster.cpp:26-32 */
    const double L[3] = {P->lx, P->ly, P->lz};
    for (int a = 0; a < 3; ++a) {
        nc[a] = (int)floor(L[a] / P->r_c + 2 * P->margin / P->r_c);
        dc[a] = (nc[a] > 0) ? fmod(L[a] + 2 * P->margin, P->r_c) / nc[a] + P->r_c : 0.0;
    }
}

static inline int cell_coord(double x, double dcell, double margin) {
    return (int)floor(x / dcell + margin / dcell); /* cluster.cpp:140-142, 197-199 */
}

int oracle_sorting(const fipi_params* P, int n, const double* p, int* keys, int* sorted,
                   int* offsets, int* it_mark) {
    int nc[3];
    double dc[3];
    oracle_cell_geometry(P, nc, dc);
    const int ncells = nc[0] * nc[1] * nc[2];
    double y_max = 0.0; /* cluster.cpp:128 */
    int status = FIPI_OK;
    for (int it = 0; it < n; ++it) {
        if (p[3 * it + 1] > y_max) { /* cluster.cpp:134-138 */
            y_max = p[3 * it + 1];
            if (it_mark) *it_mark = it;
        }
        const int i = cell_coord(p[3 * it], dc[0], P->margin);
        const int j = cell_coord(p[3 * it + 1], dc[1], P->margin);
        const int k = cell_coord(p[3 * it + 2], dc[2], P->margin);
        if (i < 0 || i >= nc[0] || j < 0 || j >= nc[1] || k < 0 || k >= nc[2]) {
            status = FIPI_ERR_OUT_OF_RANGE; /* cluster.cpp:144-163 */
            keys[it] = -1;
            continue;
        }
        keys[it] = i + j * nc[0] + k * nc[0] * nc[1]; /* cluster.cpp:165 */
    }
    if (status != FIPI_OK) return status;
    /* Appending ids in ascending order to per-cell lists (linked_list.cpp:30-43)
     * is a stable counting sort by key. */
    for (int c = 0; c <= ncells; ++c) offsets[c] = 0;
    for (int it = 0; it < n; ++it) offsets[keys[it] + 1]++;
    for (int c = 0; c < ncells; ++c) offsets[c + 1] += offsets[c];
    int* fill = (int*)malloc(sizeof(int) * (size_t)(ncells > 0 ? ncells : 1));
    for (int c = 0; c < ncells; ++c) fill[c] = offsets[c];
    for (int it = 0; it < n; ++it) sorted[fill[keys[it]]++] = it;
    free(fill);
    return FIPI_OK;
}

/* primitive.cpp:122-129 */
static double ramp(double t, double thr) {
    if (t < 0) return 0.0;
    else if (t >= 0 && t < thr) return t / thr;
    return 1.0;
}

/* vector::norm (primitive.hpp:58): pow(pow(x,2)+pow(y,2)+pow(z,2), 0.5) */
static inline double vnorm(double x, double y, double z) {
    return pow(x * x + y * y + z * z, 0.5);
}

/* Separation used when two particles coincide exactly.  The reference
 * draws rand()%1000/1e3*2 r_p - r_p per component (cluster.cpp:234-242);
 * this draws the same 1e-3 lattice from a hash of the pair, so the
 * oracle and the GPU agree.  Not pinned to the reference (its rand()). */
void oracle_coincident_d(int a, int b, double r_p, double d[3]) {
    uint64_t h = ((uint64_t)(uint32_t)a << 32) ^ (uint64_t)(uint32_t)b;
    for (int k = 0; k < 3; ++k) {
        h += 0x9E3779B97F4A7C15ull;
        uint64_t z = h;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        d[k] = (double)(z % 1000) / 1e3 * 2.0 * r_p - r_p;
    }
}

typedef struct {
    int i, j;
} pair_t;

static int pair_cmp(const void* a, const void* b) {
    const pair_t* x = (const pair_t*)a;
    const pair_t* y = (const pair_t*)b;
    if (x->i != y->i) return x->i < y->i ? -1 : 1;
    if (x->j != y->j) return x->j < y->j ? -1 : 1;
    return 0;
}

int oracle_f_pp(const fipi_params* P, int n, const double* p, int t, const double* f_pi,
                double* f_pp, double* tau_out, int* pairs, int max_pairs, int* n_pairs) {
    int nc[3];
    double dc[3];
    oracle_cell_geometry(P, nc, dc);
    const int ncells = nc[0] * nc[1] * nc[2];
    int* keys = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* sorted = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* offsets = (int*)malloc(sizeof(int) * (size_t)(ncells + 1));
    int it_mark = -1;
    int st = oracle_sorting(P, n, p, keys, sorted, offsets, &it_mark);
    if (st != FIPI_OK) {
        free(keys);
        free(sorted);
        free(offsets);
        return st;
    }
    pair_t* plist = NULL;
    long np_cap = 0, np_cnt = 0;
    const double bx = P->lx, by = P->ly, bz = P->lz; /* bc_x, bc_y, bc_z (cluster.cpp:185-187) */
    const double rmp = ramp((double)t, 0.2 * P->t_end);
    double tau = 0.0;
    for (int it = 0; it < 3 * n; ++it) f_pp[it] = 0.0; /* cluster.cpp:191 */
    for (int it = 0; it < n; ++it) {
        const int o_ = cell_coord(p[3 * it], dc[0], P->margin);
        const int p_ = cell_coord(p[3 * it + 1], dc[1], P->margin);
        const int q_ = cell_coord(p[3 * it + 2], dc[2], P->margin);
        for (int k = q_ - 1; k <= q_ + 1; k++)
            for (int j = p_ - 1; j <= p_ + 1; j++)
                for (int i = o_ - 1; i <= o_ + 1; i++) {
                    int co = (i + nc[0]) % nc[0];
                    co += (j + nc[1]) % nc[1] * nc[0];
                    co += (k + nc[2]) % nc[2] * nc[0] * nc[1];
                    for (int s = offsets[co]; s < offsets[co + 1]; ++s) {
                        const int id = sorted[s];
                        if (!(id > it)) continue; /* cluster.cpp:220 */
                        double d[3] = {p[3 * it] - p[3 * id], p[3 * it + 1] - p[3 * id + 1],
                                       p[3 * it + 2] - p[3 * id + 2]};
                        /* cluster.cpp:225-232 */
                        if (d[0] > dc[0] * (nc[0] - 2)) d[0] = d[0] - bx;
                        else if (d[0] < -dc[0] * (nc[0] - 2)) d[0] = d[0] + bx;
                        if (d[1] > dc[1] * (nc[1] - 2)) d[1] = d[1] - by;
                        else if (d[1] < -dc[1] * (nc[1] - 2)) d[1] = d[1] + by;
                        if (d[2] > dc[2] * (nc[2] - 2)) d[2] = d[2] - bz;
                        else if (d[2] < -dc[2] * (nc[2] - 2)) d[2] = d[2] + bz;
                        if (vnorm(d[0], d[1], d[2]) == 0.0) oracle_coincident_d(it, id, P->r_p, d);
                        const double dn = vnorm(d[0], d[1], d[2]);
                        if (dn < P->r_eq) { /* cluster.cpp:246-262 */
                            const double s_ = (P->r_eq - dn) * rmp * P->k_n;
                            double fn[3];
                            for (int a = 0; a < 3; ++a) fn[a] = (d[a] / dn) * s_;
                            for (int a = 0; a < 3; ++a) {
                                f_pp[3 * it + a] = f_pp[3 * it + a] + fn[a];
                                f_pp[3 * id + a] = f_pp[3 * id + a] - fn[a];
                            }
                            if (f_pi && it_mark >= 0 &&
                                vnorm(f_pi[3 * it], f_pi[3 * it + 1], f_pi[3 * it + 2]) != 0.0 &&
                                vnorm(f_pi[3 * it_mark], f_pi[3 * it_mark + 1],
                                      f_pi[3 * it_mark + 2]) != 0.0) {
                                const double h0 = fn[0] * 0.5, h1 = fn[1] * 0.5, h2 = fn[2] * 0.5;
                                tau += h0 * d[0] + h1 * d[1] + h2 * d[2];
                            }
                            if (pairs || n_pairs) {
                                if (np_cnt == np_cap) {
                                    np_cap = np_cap ? 2 * np_cap : 1024;
                                    plist = (pair_t*)realloc(plist, sizeof(pair_t) * (size_t)np_cap);
                                }
                                plist[np_cnt].i = it;
                                plist[np_cnt].j = id;
                                np_cnt++;
                            }
                        }
                    }
                }
    }
    if (tau_out) *tau_out = tau;
    if (n_pairs) *n_pairs = (int)np_cnt;
    if (pairs && np_cnt) {
        qsort(plist, (size_t)np_cnt, sizeof(pair_t), pair_cmp);
        for (long q = 0; q < np_cnt && q < max_pairs; ++q) {
            pairs[2 * q] = plist[q].i;
            pairs[2 * q + 1] = plist[q].j;
        }
    }
    free(plist);
    free(keys);
    free(sorted);
    free(offsets);
    return FIPI_OK;
}

/* field::interpolate (field.cpp:223-248) of one real field at n positions. */
void oracle_interpolate(const fipi_params* P, const double* v, int n, const double* pos,
                        double* out) {
    const int Nx = P->nx, Ny = P->ny, Nz = P->nz;
    const double dx = P->lx / Nx, dy = P->ly / Ny, dz = P->lz / Nz;
    for (int q = 0; q < n; ++q) {
        const double x = pos[3 * q], y = pos[3 * q + 1], z = pos[3 * q + 2];
        int i = (int)floor(x / dx), j = (int)floor(y / dy), k = (int)floor(z / dz);
        const double m = x / dx - floor(x / dx);
        const double nn = y / dy - floor(y / dy);
        const double oo = z / dz - floor(z / dz);
        i %= Nx; /* defined wrap where the reference reads past the end */
        j %= Ny;
        k %= Nz;
        const int i1 = (i + 1) % Nx, j1 = (j + 1) % Ny, k1 = (k + 1) % Nz;
        double val;
        val = (1.0 - m) * (1.0 - nn) * (1.0 - oo) * v[i + j * Nx + k * Nx * Ny];
        val += (1.0 - m) * nn * (1.0 - oo) * v[i + j1 * Nx + k * Nx * Ny];
        val += m * (1.0 - nn) * (1.0 - oo) * v[i1 + j * Nx + k * Nx * Ny];
        val += m * nn * (1.0 - oo) * v[i1 + j1 * Nx + k * Nx * Ny];
        val += (1.0 - m) * (1.0 - nn) * oo * v[i + j * Nx + k1 * Nx * Ny];
        val += (1.0 - m) * nn * oo * v[i + j1 * Nx + k1 * Nx * Ny];
        val += m * (1.0 - nn) * oo * v[i1 + j * Nx + k1 * Nx * Ny];
        val += m * nn * oo * v[i1 + j1 * Nx + k1 * Nx * Ny];
        out[q] = val;
    }
}

/* field::interpolate2 (field.cpp:250-281): the same products as
 * field::interpolate on the fractions m/3 + 1/3 of the size-3 stencil whose
 * corners are the nodes i + 1 and i + 2 (indices as the reference forms
 * them, periodic). */
void oracle_interpolate2(const fipi_params* P, const double* v, int n, const double* pos, double* out) {
    const int Nx = P->nx, Ny = P->ny, Nz = P->nz;
    const double dx = P->lx / Nx, dy = P->ly / Ny, dz = P->lz / Nz;
    const int size = 3;
    for (int q = 0; q < n; ++q) {
        const double x = pos[3 * q], y = pos[3 * q + 1], z = pos[3 * q + 2];
        const int i = (int)floor(x / dx), j = (int)floor(y / dy), k = (int)floor(z / dz);
        double m = x / dx - floor(x / dx);
        double nn = y / dy - floor(y / dy);
        double o = z / dz - floor(z / dz);
        m = m / size + 1.0 / size;
        nn = nn / size + 1.0 / size;
        o = o / size + 1.0 / size;
        const int i0 = (i - (1 - size) / 2 + Nx) % Nx, i1 = (i + (1 + size) / 2) % Nx;
        const int j0 = (j - (1 - size) / 2 + Ny) % Ny, j1 = (j + (1 + size) / 2) % Ny;
        const int k0 = (k - (1 - size) / 2 + Nz) % Nz, k1 = (k + (1 + size) / 2) % Nz;
        const long sxy = (long)Nx * Ny;
        double val;
        val = (1.0 - m) * (1.0 - nn) * (1.0 - o) * v[i0 + j0 * Nx + k0 * sxy];
        val += (1.0 - m) * nn * (1.0 - o) * v[i0 + j1 * Nx + k0 * sxy];
        val += m * (1.0 - nn) * (1.0 - o) * v[i1 + j0 * Nx + k0 * sxy];
        val += m * nn * (1.0 - o) * v[i1 + j1 * Nx + k0 * sxy];
        val += (1.0 - m) * (1.0 - nn) * o * v[i0 + j0 * Nx + k1 * sxy];
        val += (1.0 - m) * nn * o * v[i0 + j1 * Nx + k1 * sxy];
        val += m * (1.0 - nn) * o * v[i1 + j0 * Nx + k1 * sxy];
        val += m * nn * o * v[i1 + j1 * Nx + k1 * sxy];
        out[q] = val;
    }
}

/* element::get_f_pi (element.cpp:75-97) with the contact-angle extension:
 * f_mag = -A pi (d - r cos_theta) sigma; cos_theta = 0 is the reference. */
void oracle_f_pi(const fipi_params* P, int n, const double* c_loc, const double* dcdx,
                 const double* r, const double* cth, double* f_pi) {
    const double thr = tanh(2.0);
    for (int q = 0; q < n; ++q) {
        double f_mag = 0.0, d = 0.0;
        const double phi = c_loc[q];
        const double gx = dcdx[3 * q], gy = dcdx[3 * q + 1], gz = dcdx[3 * q + 2];
        const double rq = r ? r[q] : P->r_p;
        const double ct = cth ? cth[q] : 0.0;
        if (fabs(phi) <= thr && vnorm(gx, gy, gz) != 0.0) {
            d = 0.5 * log((1.0 + phi) / (1.0 - phi)) * sqrt(2.0) * P->epsilon;
            if (fabs(d) < rq) f_mag = -P->A * P->pi * (d - rq * ct) * P->sigma;
            else f_mag = 0.0;
            const double gn = vnorm(gx, gy, gz);
            f_pi[3 * q] = gx / gn * f_mag;
            f_pi[3 * q + 1] = gy / gn * f_mag;
            f_pi[3 * q + 2] = gz / gn * f_mag;
        } else {
            f_pi[3 * q] = f_pi[3 * q + 1] = f_pi[3 * q + 2] = 0.0;
        }
    }
}

/* element::advect (element.cpp:156-173); f_ext = 0 (element.cpp:100-104)
 * and uf = 0 (get_local_u, element.cpp:38-52). */
void oracle_advect(const fipi_params* P, int n, int stage, const double* f_pi,
                   const double* f_pp, const double* r, double* p, double* p_old,
                   double* u_old) {
    for (int q = 0; q < n; ++q) {
        const double rq = r ? r[q] : P->r_p;
        double v[3];
        for (int a = 0; a < 3; ++a) {
            double F = f_pi[3 * q + a] + 0.0; /* f_pi + f_ext */
            F = F + f_pp[3 * q + a];
            v[a] = 0.0 + F / 6.0 / P->pi / P->mu / rq; /* uf + F/6/pi/mu/r */
        }
        if (stage == 1) {
            for (int a = 0; a < 3; ++a) {
                u_old[3 * q + a] = v[a];
                p_old[3 * q + a] = p[3 * q + a];
                p[3 * q + a] = p[3 * q + a] + v[a] * P->dt;
            }
        } else {
            const double hdt = 0.5 * P->dt;
            for (int a = 0; a < 3; ++a)
                p[3 * q + a] = p_old[3 * q + a] + (u_old[3 * q + a] + v[a]) * hdt;
        }
    }
}

/* element::enforce_bc (element.cpp:177-185) */
void oracle_enforce_bc(const fipi_params* P, int n, double* p) {
    for (int q = 0; q < n; ++q) {
        p[3 * q] = fmod(p[3 * q] + P->lx, P->lx);
        p[3 * q + 1] = fmod(p[3 * q + 1] + P->ly, P->ly);
        p[3 * q + 2] = fmod(p[3 * q + 2] + P->lz, P->lz);
    }
}

/* cluster::compute_f_r (cluster.cpp:344-410) into out (3 x V reals, zeroed here). */
void oracle_spread(const fipi_params* P, int n, const double* pos, const double* f_pp,
                   double* out) {
    const int Nx = P->nx, Ny = P->ny, Nz = P->nz;
    const long V = (long)Nx * Ny * Nz;
    const double dx = P->lx / Nx, dy = P->ly / Ny, dz = P->lz / Nz;
    for (long it = 0; it < 3 * V; ++it) out[it] = 0.0;
    for (int q = 0; q < n; ++q) {
        double f[3];
        for (int a = 0; a < 3; ++a) f[a] = (f_pp[3 * q + a] + 0.0) / dx / dy / dz;
        const double X = pos[3 * q], Y = pos[3 * q + 1], Z = pos[3 * q + 2];
        int x = (int)floor(X / dx), y = (int)floor(Y / dy), z = (int)floor(Z / dz);
        const double o = X / dx - floor(X / dx);
        const double pp = Y / dy - floor(Y / dy);
        const double qq = Z / dz - floor(Z / dz);
        x %= Nx;
        y %= Ny;
        z %= Nz;
        const int x1 = (x + 1) % Nx, y1 = (y + 1) % Ny, z1 = (z + 1) % Nz;
        /* corner order and weight products of cluster.cpp:368-406 */
        const long co[8] = {x + y * Nx + (long)z * Nx * Ny,    x1 + y * Nx + (long)z * Nx * Ny,
                            x1 + y1 * Nx + (long)z * Nx * Ny,  x1 + y * Nx + (long)z1 * Nx * Ny,
                            x1 + y1 * Nx + (long)z1 * Nx * Ny, x + y * Nx + (long)z1 * Nx * Ny,
                            x + y1 * Nx + (long)z * Nx * Ny,   x + y1 * Nx + (long)z1 * Nx * Ny};
        for (int a = 0; a < 3; ++a) {
            double* g = out + a * V;
            g[co[0]] += f[a] * (1 - o) * (1 - pp) * (1 - qq);
            g[co[1]] += f[a] * o * (1 - pp) * (1 - qq);
            g[co[2]] += f[a] * o * pp * (1 - qq);
            g[co[3]] += f[a] * o * (1 - pp) * qq;
            g[co[4]] += f[a] * o * pp * qq;
            g[co[5]] += f[a] * (1 - o) * (1 - pp) * qq;
            g[co[6]] += f[a] * (1 - o) * pp * (1 - qq);
            g[co[7]] += f[a] * (1 - o) * pp * qq;
        }
    }
}

/* ------------------------------------------------ particle-model extensions
 * Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC 2011). */
void oracle_philox4x32(const unsigned ctr_in[4], unsigned k0, unsigned k1, unsigned out[4]) {
    unsigned c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const unsigned long long p0 = 0xD2511F53ull * c0, p1 = 0xCD9E8D57ull * c2;
        const unsigned hi0 = (unsigned)(p0 >> 32), lo0 = (unsigned)p0;
        const unsigned hi1 = (unsigned)(p1 >> 32), lo1 = (unsigned)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* element::get_f_rand's draw (element.cpp:109-144) with the Philox stream of
 * (particle, step) in place of rand(): Box-Muller on (k mod 1000)/1000,
 * redrawn while |g| > 5, at most 64 draws per normal (then 0). */
void oracle_brownian_normals(unsigned long long seed, unsigned id, unsigned t, double pi, double g[3]) {
    unsigned buf[4];
    int used = 4;
    unsigned blk = 0;
    for (int a = 0; a < 3; ++a) {
        double v = 0.0;
        for (int k = 0; k < 64; ++k) {
            unsigned x[2];
            for (int q = 0; q < 2; ++q) {
                if (used == 4) {
                    const unsigned ctr[4] = {id, t, blk++, 0u};
                    oracle_philox4x32(ctr, (unsigned)seed, (unsigned)(seed >> 32), buf);
                    used = 0;
                }
                x[q] = buf[used++];
            }
            const double r1 = (double)(x[0] % 1000u) / 1000;
            const double r2 = (double)(x[1] % 1000u) / 1000;
            v = sqrt(-2 * log(r1)) * cos(2 * pi * r2);
            if (fabs(v) <= 5.0) break;
            v = 0.0;
        }
        g[a] = v;
    }
}

void oracle_set_mass_conserving(oracle* o, int on) { o->conserve = on ? 1 : 0; }

void oracle_set_extensions(oracle* o, int couple, double kt, unsigned long long seed) {
    o->couple = couple;
    o->kt = kt;
    o->seed = seed;
}

/* element::advect (element.cpp:156-173) with uf (fluid coupling) and the
 * Brownian force added to f_pi + f_ext + f_pp. */
static void advect_ext(const oracle* o, int stage) {
    const fipi_params* P = &o->P;
    for (int q = 0; q < o->n; ++q) {
        const double rq = o->r[q];
        double v[3];
        for (int a = 0; a < 3; ++a) {
            double F = o->f_pi[3 * q + a] + 0.0;
            F = F + o->f_pp[3 * q + a];
            if (o->kt > 0.0) F = F + o->f_rand[3 * q + a];
            v[a] = (o->couple ? o->uf[3 * q + a] : 0.0) + F / 6.0 / P->pi / P->mu / rq;
        }
        if (stage == 1) {
            for (int a = 0; a < 3; ++a) {
                o->u_old[3 * q + a] = v[a];
                o->p_old[3 * q + a] = o->p[3 * q + a];
                o->p[3 * q + a] = o->p[3 * q + a] + v[a] * P->dt;
            }
        } else {
            const double hdt = 0.5 * P->dt;
            for (int a = 0; a < 3; ++a)
                o->p[3 * q + a] = o->p_old[3 * q + a] + (o->u_old[3 * q + a] + v[a]) * hdt;
        }
    }
}

/* ------------------------------------------------------------------ step */
static void particle_stage(oracle* o, int stage) {
    const fipi_params* P = &o->P;
    const int n = o->n;
    const long V = o->V;
    /* interpolate_local_variables (cluster.cpp:307-323) */
    if (P->switch_ch) {
        double* tmp = (double*)malloc(sizeof(double) * (size_t)V);
        double* vals = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        for (long it = 0; it < V; ++it) tmp[it] = o->c[2 * it];
        oracle_interpolate(P, tmp, n, o->p, o->c_loc);
        for (int d = 0; d < 3; ++d) {
            for (long it = 0; it < V; ++it) tmp[it] = o->grad[d][2 * it];
            oracle_interpolate(P, tmp, n, o->p, vals);
            for (int q = 0; q < n; ++q) o->dcdx[3 * q + d] = vals[q];
        }
        free(tmp);
        free(vals);
    }
    if (o->couple) { /* get_local_u with its interpolation (element.cpp:38-52) */
        double* tmp = (double*)malloc(sizeof(double) * (size_t)V);
        double* vals = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        for (int d = 0; d < 3; ++d) {
            for (long it = 0; it < V; ++it) tmp[it] = o->u[d][2 * it];
            oracle_interpolate(P, tmp, n, o->p, vals);
            for (int q = 0; q < n; ++q) o->uf[3 * q + d] = vals[q];
        }
        free(tmp);
        free(vals);
    }
    if (o->kt > 0.0 && stage == 1) /* the step's Brownian force (element.cpp:138-143) */
        for (int q = 0; q < n; ++q) {
            double g[3];
            oracle_brownian_normals(o->seed, (unsigned)q, (unsigned)o->t, P->pi, g);
            const double s = sqrt(12.0 * P->pi * o->r[q] * P->mu * o->kt / P->dt);
            for (int a = 0; a < 3; ++a) o->f_rand[3 * q + a] = s * g[a];
        }
    /* sorting (cluster.cpp:116-169) */
    (void)oracle_sorting(P, n, o->p, o->keys, o->sorted, o->offsets, &o->it_mark);
    /* compute_f_pi (cluster.cpp:286-290) */
    oracle_f_pi(P, n, o->c_loc, o->dcdx, o->r, o->cth, o->f_pi);
    /* compute_f_pp(t+1) (main.cpp:202, 213) */
    oracle_f_pp(P, n, o->p, o->t + 1, o->f_pi, o->f_pp, &o->tau, NULL, 0, NULL);
    /* compute_f_ext: zero (element.cpp:100-104); advect; enforce_bc */
    if (o->couple || o->kt > 0.0) advect_ext(o, stage);
    else oracle_advect(P, n, stage, o->f_pi, o->f_pp, o->r, o->p, o->p_old, o->u_old);
    oracle_enforce_bc(P, n, o->p);
}

int oracle_step(oracle* o) {
    const fipi_params* P = &o->P;
    const long V = o->V;
    const int t = o->t;
    const double dt = P->dt, M = P->mobility, lam = P->lambda;

    if (P->n_p > 0 && P->switch_particle) {
        /* the reference exits inside sorting(); check the range up front so
         * the oracle's state stays untouched on error */
        int* keys = (int*)malloc(sizeof(int) * (size_t)o->n);
        int* srt = (int*)malloc(sizeof(int) * (size_t)o->n);
        int nc[3];
        double dc[3];
        oracle_cell_geometry(P, nc, dc);
        int* off = (int*)malloc(sizeof(int) * (size_t)(nc[0] * nc[1] * nc[2] + 1));
        int st = oracle_sorting(P, o->n, o->p, keys, srt, off, NULL);
        free(keys);
        free(srt);
        free(off);
        if (st != FIPI_OK) return st;
    }

    /* ------------------------------------------- Phase field (main.cpp:79-141) */
    if (P->switch_ch) {
        bulk_potential(o); /* main.cpp:81 */
        fft(o, o->f);      /* main.cpp:83 */
        fft(o, o->c);      /* main.cpp:84 */
        if (P->switch_ns) {
            grad_spectral(o, o->c, o->grad); /* main.cpp:88 */
            for (int d = 0; d < 3; ++d) ifft(o, o->grad[d]);
            for (long it = 0; it < V; ++it) { /* conv_c = u.dot(grad_c) (field.cpp:388-401) */
                double s = 0.0;
                for (int d = 0; d < 3; ++d) s += o->u[d][2 * it] * o->grad[d][2 * it];
                o->conv[2 * it] = s;
                o->conv[2 * it + 1] = 0.0;
            }
            fft(o, o->conv); /* main.cpp:92 */
            if (o->conserve) o->conv[0] = o->conv[1] = 0.0;
        }
        if (t == 0) { /* main.cpp:95-114 */
            memcpy(o->c_old, o->c, sizeof(double) * 2 * (size_t)V);
            memcpy(o->f_old, o->f, sizeof(double) * 2 * (size_t)V);
            if (P->switch_ns) memcpy(o->conv_old, o->conv, sizeof(double) * 2 * (size_t)V);
            const double s1 = dt * M, s2 = dt * M * lam;
            for (long it = 0; it < V; ++it) {
                const double k2 = kf2_at(o, it);
                const double a = k2 * s1;
                o->c[2 * it] -= a * o->f[2 * it];
                o->c[2 * it + 1] -= a * o->f[2 * it + 1];
                if (P->switch_ns) {
                    o->c[2 * it] -= o->conv[2 * it] * dt;
                    o->c[2 * it + 1] -= o->conv[2 * it + 1] * dt;
                }
                double k4 = 0.0;
                k4 += field_pow(k2, 2.0);
                const double den = k4 * s2 + 1.0;
                o->c[2 * it] /= den;
                o->c[2 * it + 1] /= den;
            }
        } else { /* main.cpp:115-138 */
            const double s4 = 4.0 * dt * M, s2m = 2.0 * dt * M;
            const double s4c = 4.0 * dt, s2c = 2.0 * dt, s3 = 2.0 * dt * M * lam;
            for (long it = 0; it < V; ++it) {
                const double k2 = kf2_at(o, it);
                double re = o->c[2 * it] * 4.0 - o->c_old[2 * it];
                double im = o->c[2 * it + 1] * 4.0 - o->c_old[2 * it + 1];
                const double a4 = k2 * s4, a2 = k2 * s2m;
                re -= a4 * o->f[2 * it];
                im -= a4 * o->f[2 * it + 1];
                re += a2 * o->f_old[2 * it];
                im += a2 * o->f_old[2 * it + 1];
                if (P->switch_ns) {
                    re -= o->conv[2 * it] * s4c;
                    im -= o->conv[2 * it + 1] * s4c;
                    re += o->conv_old[2 * it] * s2c;
                    im += o->conv_old[2 * it + 1] * s2c;
                }
                double k4 = 0.0;
                k4 += field_pow(k2, 2.0);
                const double den = k4 * s3 + 3.0;
                o->c_new[2 * it] = re / den;
                o->c_new[2 * it + 1] = im / den;
            }
            /* c_old = c; f_old = f; conv_c_old = conv_c; c = c_new (main.cpp:129-137) */
            double* tmp = o->c_old;
            o->c_old = o->c;
            o->c = o->c_new;
            o->c_new = tmp;
            tmp = o->f_old;
            o->f_old = o->f;
            o->f = tmp;
            if (P->switch_ns) {
                tmp = o->conv_old;
                o->conv_old = o->conv;
                o->conv = tmp;
            }
        }
        ifft(o, o->c); /* main.cpp:140 */
    }

    /* ------------------------------------------- Fluid velocity (main.cpp:146-181) */
    if (P->switch_ns) {
        for (int d = 0; d < 3; ++d) memset(o->ftot[d], 0, sizeof(double) * 2 * (size_t)V);
        if (P->switch_ch) {
            bulk_potential(o); /* main.cpp:153 */
            fft(o, o->f);
            fft(o, o->c);
            for (long it = 0; it < V; ++it) { /* pch = lambda*kf2*c + f (main.cpp:157) */
                const double a = kf2_at(o, it) * lam;
                o->pch[2 * it] = a * o->c[2 * it] + o->f[2 * it];
                o->pch[2 * it + 1] = a * o->c[2 * it + 1] + o->f[2 * it + 1];
            }
            ifft(o, o->pch);
            grad_spectral(o, o->c, o->grad); /* main.cpp:160-162 */
            for (int d = 0; d < 3; ++d) ifft(o, o->grad[d]);
            ifft(o, o->c);
            for (int d = 0; d < 3; ++d) /* f_total += pch*grad_c (main.cpp:164) */
                for (long it = 0; it < V; ++it) {
                    o->ftot[d][2 * it] += o->pch[2 * it] * o->grad[d][2 * it];
                    o->ftot[d][2 * it + 1] = 0.0;
                }
        }
        if (P->switch_particle && o->n > 0) { /* f_total += suspension.compute_f_r() */
            double* sp = (double*)malloc(sizeof(double) * 3 * (size_t)V);
            oracle_spread(P, o->n, o->p, o->f_pp, sp);
            for (int d = 0; d < 3; ++d)
                for (long it = 0; it < V; ++it) {
                    o->ftot[d][2 * it] += sp[d * V + it];
                    o->ftot[d][2 * it + 1] = 0.0;
                }
            free(sp);
        }
        for (long it = 0; it < V; ++it) { /* buoyancy (main.cpp:172) */
            const double cr = o->c[2 * it];
            double a = cr + 1.0;
            a = a / 2.0;
            a = a * P->rho1;
            double b = cr * (-1.0) + 1.0;
            b = b / 2.0;
            b = b * P->rho2;
            const double s = a + b;
            o->ftot[0][2 * it] += s * 0.0;
            o->ftot[1][2 * it] += s * 0.0;
            o->ftot[2][2 * it] += s * P->gravity;
            for (int d = 0; d < 3; ++d) o->ftot[d][2 * it + 1] = 0.0;
        }
        for (int d = 0; d < 3; ++d) fft(o, o->ftot[d]); /* main.cpp:175 */
        /* u = f_total - kf*(kf.dot(f_total))/kf2; u /= mu*kf2 (main.cpp:177-178) */
        for (long it = 0; it < V; ++it) {
            const double kv[3] = {o->kx[IDX_I(o, it)], o->ky[IDX_J(o, it)], o->kz[IDX_K(o, it)]};
            const double k2 = kf2_at(o, it);
            double dre = 0.0, dim = 0.0;
            for (int d = 0; d < 3; ++d) {
                dre += kv[d] * o->ftot[d][2 * it];
                dim += kv[d] * o->ftot[d][2 * it + 1];
            }
            const double m = k2 * P->mu;
            for (int d = 0; d < 3; ++d) {
                double qre = kv[d] * dre, qim = kv[d] * dim;
                if (k2 != 0.0) {
                    qre = qre / k2;
                    qim = qim / k2;
                } else {
                    qre = 0.0;
                    qim = 0.0;
                }
                double ure = o->ftot[d][2 * it] - qre;
                double uim = o->ftot[d][2 * it + 1] - qim;
                if (m != 0.0) {
                    ure /= m;
                    uim /= m;
                } else {
                    ure = 0.0;
                    uim = 0.0;
                }
                o->u[d][2 * it] = ure;
                o->u[d][2 * it + 1] = uim;
            }
        }
        for (int d = 0; d < 3; ++d) ifft(o, o->u[d]); /* main.cpp:179 */
    }

    /* ------------------------------------------- Particles (main.cpp:186-219) */
    if (P->switch_particle && o->n > 0) {
        if (P->switch_ch) {
            fft(o, o->c); /* main.cpp:190-193 */
            grad_spectral(o, o->c, o->grad);
            for (int d = 0; d < 3; ++d) ifft(o, o->grad[d]);
            ifft(o, o->c);
        }
        particle_stage(o, 1);
        particle_stage(o, 2);
    }
    o->t = t + 1;
    return FIPI_OK;
}

/* main.cpp:232 with field.cpp:507-516: sum of
 * lambda*(0.5 |grad c|^2 + 0.25/eps^2 (c^2-1)^2) * dx^3. */
double oracle_free_energy(const oracle* o) {
    const fipi_params* P = &o->P;
    const double dx = P->lx / P->nx;
    const double e2 = 0.25 / (P->epsilon * P->epsilon);
    double sum = 0.0;
    for (long it = 0; it < o->V; ++it) {
        double g2 = 0.0;
        for (int d = 0; d < 3; ++d) g2 += field_pow(o->grad[d][2 * it], 2.0);
        const double cr = o->c[2 * it];
        double c2 = 0.0;
        c2 += field_pow(cr, 2.0);
        const double w = c2 - 1.0;
        double w2 = 0.0;
        w2 += field_pow(w, 2.0);
        const double fe = (g2 * 0.5 + w2 * e2) * P->lambda;
        sum += fe * (dx * dx * dx);
    }
    return sum;
}

double oracle_mass(const oracle* o) {
    const fipi_params* P = &o->P;
    const double dv = (P->lx / P->nx) * (P->ly / P->ny) * (P->lz / P->nz);
    double s = 0.0;
    for (long it = 0; it < o->V; ++it) s += o->c[2 * it];
    return s * dv;
}

/* ------------------------------------------------ the reference's initial state
 * glibc's rand() (random() with the default TYPE_3 state of 31 words):
 * state r[0] = seed (1 if 0), r[i] = 16807 r[i-1] mod (2^31 - 1) for i < 31
 * (Schrage's decomposition), front index 3 and rear index 0, then 310
 * discarded outputs; each output adds the rear word into the front word
 * (mod 2^32) and returns it shifted right by one. */
typedef struct {
    int32_t r[31];
    int f, b;
} glibc_rand;

static int glibc_next(glibc_rand* g) {
    const uint32_t v = (uint32_t)g->r[g->f] + (uint32_t)g->r[g->b];
    g->r[g->f] = (int32_t)v;
    g->f = (g->f + 1) % 31;
    g->b = (g->b + 1) % 31;
    return (int)(v >> 1);
}

static void glibc_srand(glibc_rand* g, unsigned int seed) {
    int32_t word = (int32_t)(seed ? seed : 1u);
    g->r[0] = word;
    for (int i = 1; i < 31; ++i) {
        const int32_t hi = word / 127773, lo = word % 127773;
        word = 16807 * lo - 2836 * hi;
        if (word < 0) word += 2147483647;
        g->r[i] = word;
    }
    g->f = 3;
    g->b = 0;
    for (int i = 0; i < 310; ++i) glibc_next(g);
}

/* vector::norm (primitive.hpp:58) */
static double ref_norm3(double x, double y, double z) {
    return pow(pow(x, 2) + pow(y, 2) + pow(z, 2), 0.5);
}

int oracle_reference_initial_state(const fipi_params* P, unsigned int seed, double* c, double* pos,
                                   long max_candidates) {
    glibc_rand g;
    glibc_srand(&g, seed); /* srand (main.cpp:24) */
    const long V = (long)P->nx * P->ny * P->nz;
    for (long it = 0; it < V; ++it) { /* field("SCALARS","phase_field") (field.cpp:85-99) */
        const double v = (double)(glibc_next(&g) % 1000) / 1e3 * 0.2 - 0.1;
        if (c) c[it] = v;
    }
    if (!P->switch_particle || P->n_p <= 0) return FIPI_OK;
    const int n = P->n_p;
    double* p = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    for (int it = 0; it < n; ++it) { /* cluster::distribute (cluster.cpp:53-92) */
        long cand = 0;
        for (;;) {
            const double r1 = (double)(glibc_next(&g) % 1000) / 1e3;
            const double r2 = (double)(glibc_next(&g) % 1000) / 1e3;
            const double r3 = (double)(glibc_next(&g) % 1000) / 1e3;
            p[3 * it] = P->lx * r1;
            p[3 * it + 1] = P->ly * r2;
            p[3 * it + 2] = P->lz * r3;
            int overlap = 0; /* check_overlap (cluster.cpp:98-113) */
            for (int j = 0; j < it; ++j) {
                if (ref_norm3(p[3 * j] - p[3 * it], p[3 * j + 1] - p[3 * it + 1], p[3 * j + 2] - p[3 * it + 2]) <
                    2.0 * P->r_p) {
                    overlap = 1;
                    break;
                }
            }
            if (!overlap) break;
            if (++cand >= max_candidates) {
                free(p);
                return FIPI_ERR_BAD_PARAMS;
            }
        }
    }
    if (pos) memcpy(pos, p, sizeof(double) * 3 * (size_t)n);
    free(p);
    return FIPI_OK;
}

/* ------------------------------------------------ seeded synthetic inputs
 * Restatement of the library's own input generators fipi_seed_phase and
 * fipi_seed_particles (the reference draws from unseeded rand() instead,
 * field.cpp:96, cluster.cpp:59-89), so that the CPU baselines can build the
 * same inputs without loading the library.  splitmix64 (Steele, Lea, Flood
 * 2014) drives both: 53-bit uniforms in [0, 1).  Equal to the library's
 * draws bit for bit (tests/test_capi_cpu.py). */
static uint64_t sm64_next(uint64_t* s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double sm64_u01(uint64_t* s) { return (double)(sm64_next(s) >> 11) * 0x1.0p-53; }

void oracle_seed_phase(const fipi_params* P, unsigned long long seed, double mean, double amp, double* c) {
    uint64_t s = (uint64_t)seed * 0x2545F4914F6CDD1Dull + 1;
    const long V = (long)P->nx * P->ny * P->nz;
    for (long i = 0; i < V; ++i) c[i] = mean + amp * (2.0 * sm64_u01(&s) - 1.0);
}

static double seed_wrapd(double d, double l) {
    if (d > 0.5 * l) d -= l;
    else if (d < -0.5 * l) d += l;
    return d;
}

/* Random sequential addition with the periodic minimum-image test
 * |x_i - x_j| >= r_i + r_j over a hash grid of cells >= 2 r_max (every
 * particle closer than r_i + r_j lies in one of the 27 cells around the
 * candidate); candidates are drawn until one fits, at most 200000 times. */
int oracle_seed_particles(const fipi_params* P, unsigned long long seed, double r_min, double r_max,
                          double theta_min_deg, double theta_max_deg, int allow_overlap, double* pos, double* r,
                          double* cos_theta) {
    const int n = P->n_p;
    if (n <= 0) return FIPI_OK;
    uint64_t s = (uint64_t)seed * 0x9E3779B97F4A7C15ull + 7;
    const double L[3] = {P->lx, P->ly, P->lz};
    int gc[3];
    double gs[3];
    for (int a = 0; a < 3; ++a) {
        gc[a] = (int)floor(L[a] / (2.0 * r_max));
        if (gc[a] < 1) gc[a] = 1;
        gs[a] = L[a] / gc[a];
    }
    const long ncell = (long)gc[0] * gc[1] * gc[2];
    /* per-cell singly linked lists in insertion order (head, tail, next) */
    int* head = (int*)malloc(sizeof(int) * (size_t)ncell);
    int* tail = (int*)malloc(sizeof(int) * (size_t)ncell);
    int* next = (int*)malloc(sizeof(int) * (size_t)n);
    double* rr = (double*)malloc(sizeof(double) * (size_t)n);
    for (long q = 0; q < ncell; ++q) head[q] = tail[q] = -1;
    for (int i = 0; i < n; ++i) rr[i] = r_min + (r_max - r_min) * sm64_u01(&s);
    int status = FIPI_OK;
    for (int i = 0; i < n && status == FIPI_OK; ++i) {
        double x[3];
        int ok = 0;
        for (long tries = 0; tries < 200000 && !ok; ++tries) {
            for (int a = 0; a < 3; ++a) {
                x[a] = L[a] * sm64_u01(&s);
                if (x[a] >= L[a]) x[a] = 0.0;
            }
            if (allow_overlap) {
                ok = 1;
                break;
            }
            int ci[3];
            for (int a = 0; a < 3; ++a) {
                ci[a] = (int)(x[a] / gs[a]);
                if (ci[a] > gc[a] - 1) ci[a] = gc[a] - 1;
            }
            ok = 1;
            for (int dk = -1; dk <= 1 && ok; ++dk)
                for (int dj = -1; dj <= 1 && ok; ++dj)
                    for (int di = -1; di <= 1 && ok; ++di) {
                        const long c = (long)((ci[0] + di + gc[0]) % gc[0]) +
                                       (long)((ci[1] + dj + gc[1]) % gc[1]) * gc[0] +
                                       (long)((ci[2] + dk + gc[2]) % gc[2]) * gc[0] * gc[1];
                        for (int j = head[c]; j >= 0; j = next[j]) {
                            double d2 = 0.0;
                            for (int a = 0; a < 3; ++a) {
                                const double d = seed_wrapd(x[a] - pos[3 * j + a], L[a]);
                                d2 += d * d;
                            }
                            const double rs = rr[i] + rr[j];
                            if (d2 < rs * rs) {
                                ok = 0;
                                break;
                            }
                        }
                    }
        }
        if (!ok) {
            status = FIPI_ERR_BAD_PARAMS;
            break;
        }
        for (int a = 0; a < 3; ++a) pos[3 * i + a] = x[a];
        int ci[3];
        for (int a = 0; a < 3; ++a) {
            ci[a] = (int)(x[a] / gs[a]);
            if (ci[a] > gc[a] - 1) ci[a] = gc[a] - 1;
        }
        const long c = (long)ci[0] + (long)ci[1] * gc[0] + (long)ci[2] * gc[0] * gc[1];
        next[i] = -1;
        if (tail[c] < 0) head[c] = i;
        else next[tail[c]] = i;
        tail[c] = i;
    }
    if (status == FIPI_OK) {
        if (r)
            for (int i = 0; i < n; ++i) r[i] = rr[i];
        if (cos_theta)
            for (int i = 0; i < n; ++i) {
                const double th = theta_min_deg + (theta_max_deg - theta_min_deg) * sm64_u01(&s);
                cos_theta[i] = (th == 90.0) ? 0.0 : cos(th * 3.14159265358979323846 / 180.0);
            }
    }
    free(head);
    free(tail);
    free(next);
    free(rr);
    return status;
}
