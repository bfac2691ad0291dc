/*
 * TEST INFRASTRUCTURE ONLY (oracle).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load this; the product never does.
 *
 * A plain-C, FP64 restatement of the reference FIPI step (main.cpp:75-219)
 * and of the field / cluster / element calls it makes, using full complex
 * C2C fields exactly as the reference does (field.cpp:41-46), so that it
 * reproduces the reference's arithmetic, its Nyquist handling and its
 * imaginary-part bookkeeping.  Every function cites the reference lines it
 * follows.  Pinned against the reference itself (compiled in place by
 * oracle/ref/) and against committed golden vectors (tests/golden/).
 */
#ifndef FIPI_ORACLE_H
#define FIPI_ORACLE_H

#include "../include/fipi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle oracle;

/* NULL when the parameters are outside what the oracle restates
 * (non power-of-two grid, fewer than 3 cells per axis with particles on). */
oracle* oracle_create(const fipi_params* p);
int oracle_params_ok(const fipi_params* p);
/* cluster.cpp:26-32 */
void oracle_cell_geometry(const fipi_params* p, int nc[3], double dc[3]);
/* deterministic stand-in for the rand() separation of cluster.cpp:234-242 */
void oracle_coincident_d(int a, int b, double r_p, double d[3]);
void oracle_destroy(oracle* o);
void oracle_set_threads(int n);

/* state: c (V reals), u (3V reals), particles (n x 3), radii, cos_theta */
int oracle_set_phase(oracle* o, const double* c);
int oracle_set_velocity(oracle* o, const double* u);
int oracle_set_particles(oracle* o, const double* p, const double* r, const double* cos_theta,
                         const double* f_pp);
void oracle_get_phase(const oracle* o, double* c);
void oracle_get_phase_imag(const oracle* o, double* c_im);
void oracle_get_velocity(const oracle* o, double* u);
void oracle_get_grad(const oracle* o, double* g);
void oracle_get_particles(const oracle* o, double* p, double* f_pp, double* f_pi);
double oracle_tau(const oracle* o);
int oracle_time(const oracle* o);

/* One iteration of the main.cpp:75-219 loop body; returns FIPI_OK or
 * FIPI_ERR_OUT_OF_RANGE (the reference's cluster.cpp:144-163 exit). */
int oracle_step(oracle* o);

/* Fine-grained restatements (stateless w.r.t. the step). */
void oracle_fft3(const fipi_params* P, double* data, int sign); /* C2C, unnormalised */
void oracle_grad(const fipi_params* P, const double* c, double* out); /* 3 x V */
void oracle_div(const fipi_params* P, const double* v, double* out);  /* 3 x V -> V */
void oracle_interpolate2(const fipi_params* P, const double* field, int n, const double* p, double* out);
int oracle_sorting(const fipi_params* P, int n, const double* p, int* keys, int* sorted,
                   int* offsets, int* it_mark);
int oracle_f_pp(const fipi_params* P, int n, const double* p, int t, const double* f_pi,
                double* f_pp, double* tau, int* pairs, int max_pairs, int* n_pairs);
void oracle_interpolate(const fipi_params* P, const double* field, int n, const double* p,
                        double* out);
void oracle_f_pi(const fipi_params* P, int n, const double* c_loc, const double* dcdx,
                 const double* r, const double* cos_theta, double* f_pi);
void oracle_advect(const fipi_params* P, int n, int stage, const double* f_pi,
                   const double* f_pp, const double* r, double* p, double* p_old,
                   double* u_old);
void oracle_enforce_bc(const fipi_params* P, int n, double* p);
void oracle_spread(const fipi_params* P, int n, const double* p, const double* f_pp,
                   double* out);
/* Particle-model extensions (off by default): fluid coupling (uf = u
 * interpolated, element.cpp:38-52) and the Brownian force of
 * element.cpp:109-144 drawn from Philox-4x32-10. */
void oracle_set_extensions(oracle* o, int couple, double kt, unsigned long long seed);
/* The library's mass-conserving mode (fipi_set_mass_conserving): the k = 0
 * mode of the advection spectrum (main.cpp:92) taken as 0. */
void oracle_set_mass_conserving(oracle* o, int on);
void oracle_philox4x32(const unsigned ctr[4], unsigned k0, unsigned k1, unsigned out[4]);
void oracle_brownian_normals(unsigned long long seed, unsigned id, unsigned t, double pi, double g[3]);
/* srand(seed) (main.cpp:24), the phase field's draws (field.cpp:85-99) and
 * cluster::distribute (cluster.cpp:53-113) with glibc's rand(); returns
 * FIPI_ERR_BAD_PARAMS when a particle exceeds max_candidates draws. */
int oracle_reference_initial_state(const fipi_params* P, unsigned int seed, double* c, double* pos,
                                   long max_candidates);
double oracle_free_energy(const oracle* o);
double oracle_mass(const oracle* o);
/* The library's seeded input generators (fipi_seed_phase,
 * fipi_seed_particles of include/fipi.h) restated, same draws bit for bit. */
void oracle_seed_phase(const fipi_params* P, unsigned long long seed, double mean, double amp, double* c);
int oracle_seed_particles(const fipi_params* P, unsigned long long seed, double r_min, double r_max,
                          double theta_min_deg, double theta_max_deg, int allow_overlap, double* pos, double* r,
                          double* cos_theta);

#ifdef __cplusplus
}
#endif
#endif
