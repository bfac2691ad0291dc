/*
 * fipi.h — C ABI of the GB300-native FIPI step (sm_103a).
 *
 * This library replaces the per-step hot path of FIPI (Fast Interface
 * Particle Interaction): a pseudo-spectral Cahn–Hilliard phase field coupled
 * to a Stokes velocity by Leray projection, and overdamped spheres moved by
 * interface-attachment and pair-contact forces whose contact forces are
 * spread back onto the grid.
 *
 * The reference is host C++ (class `field`, `cluster`, `element`, `list`)
 * with no FFI; every entry point below names the reference call it replaces
 * (path:line inside the reference project).  All functions return a
 * `fipi_status` (0 = FIPI_OK); the reference printed a message and called
 * exit(0) instead.  The text of the last error of the calling thread is
 * returned by fipi_last_error_string().
 *
 * Conventions
 *  - Real grid fields are Nz*Ny*Nx doubles, x fastest: linear index
 *    it = i + j*Nx + k*Nx*Ny, grid node i sits at x = i*dx
 *    (field.cpp:88-92 of the reference).
 *  - Vector grid fields are 3 such arrays back to back (component-major),
 *    like field::v[d] (field.hpp:25).
 *  - Particle vectors are n_p x 3 doubles, particle-major (x,y,z per
 *    particle), like element::p (element.hpp:32).
 *  - A context owns all device buffers and one CUDA stream.  It is not
 *    thread-safe: use one host thread per context.
 *  - Host pointers are copied in/out synchronously with respect to the
 *    calling thread.
 */
#ifndef FIPI_H
#define FIPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FIPI_ABI_VERSION 1

typedef enum fipi_status {
    FIPI_OK = 0,
    FIPI_ERR_BAD_PARAMS = 1,    /* parameters rejected by fipi_create         */
    FIPI_ERR_BAD_ARG = 2,       /* NULL pointer, bad size or stage name       */
    FIPI_ERR_CUDA = 3,          /* a CUDA runtime call failed                 */
    FIPI_ERR_OUT_OF_RANGE = 4,  /* particle outside the sorting range:
                                   cluster.cpp:144-163 printed and exit(0)    */
    FIPI_ERR_NONFINITE = 5,     /* NaN/Inf detected in the state              */
    FIPI_ERR_NO_DEVICE = 6,     /* no CUDA device visible                     */
    FIPI_ERR_STATE = 7,         /* call out of order (e.g. step before state) */
    FIPI_ERR_UNSUPPORTED = 8,   /* configuration outside what is built        */
    FIPI_ERR_RANGE = 9,         /* a value outside what an accumulator holds
                                   (mixed-form fixed-point spreading)         */
    FIPI_ERR_TIMEOUT = 10       /* a bounded device wait gave up; the work of
                                   that call is incomplete, the context usable */
} fipi_status;

typedef enum fipi_precision {
    FIPI_FP64 = 0,   /* plain FP64 everywhere (parity form)                   */
    FIPI_MIXED = 1   /* FP32 grid/FFT/particle-force arithmetic; FP64 k=0
                        mode, compensated reductions, particle positions      */
} fipi_precision;

/*
 * Run-time replacement of the reference's compile-time constants
 * (head.hpp:27-74, parameter.hpp:18-20).  fipi_params_reference() fills the
 * values of the reference's head.hpp.
 */
typedef struct fipi_params {
    int nx, ny, nz;            /* grid points, powers of two in [8, 512]      head.hpp:29-31 */
    double lx, ly, lz;         /* periodic box lengths                         head.hpp:33-35 */
    double dt;                 /* time step                                    head.hpp:41    */
    int t_end;                 /* run length; enters ramp(t, 0.2 t_end) only   head.hpp:42    */
    double pi;                 /* the reference uses pi = 3.1415926            head.hpp:27    */
    double sigma;              /* surface tension                              head.hpp:45    */
    double epsilon;            /* interface width                              head.hpp:46    */
    double lambda;             /* gradient energy coefficient                  head.hpp:47    */
    double mobility;           /* Cahn-Hilliard mobility M                     head.hpp:58    */
    double mu;                 /* viscosity                                    head.hpp:54    */
    double rho1, rho2;         /* fluid densities (buoyancy)                   head.hpp:52-53 */
    double gravity;            /* z component of g                             head.hpp:51    */
    double A;                  /* attachment force constant                    head.hpp:57    */
    double k_n;                /* contact stiffness                            parameter.hpp:18 */
    double margin;             /* cell-grid margin                             parameter.hpp:20 */
    double r_p;                /* default particle radius                      head.hpp:59    */
    double r_eq;               /* contact range                                head.hpp:64    */
    double r_c;                /* cell-list cell size                          head.hpp:65    */
    int n_p;                   /* number of particles (0 allowed)              head.hpp:63    */
    int switch_particle;       /* head.hpp:72 */
    int switch_ch;             /* head.hpp:73 */
    int switch_ns;             /* head.hpp:74 */
} fipi_params;

typedef struct fipi_ctx fipi_ctx;

/* ---------------------------------------------------------------- basics */
int fipi_abi_version(void);
const char* fipi_last_error_string(void);
/* Values of the reference's head.hpp / parameter.hpp (64^3, Lx = 2 pi, ...). */
fipi_status fipi_params_reference(fipi_params* out);
/* Cell-grid geometry of cluster::cluster() (cluster.cpp:26-32):
 * n_cell = floor(L/r_c + 2 margin/r_c), d_cell = fmod(L + 2 margin, r_c)/n_cell + r_c. */
fipi_status fipi_cell_geometry(const fipi_params* p, int n_cell[3], double d_cell[3]);

/* ------------------------------------------------------------- lifecycle */
/* Allocates every device buffer of the step on `device`.  Replaces the field
 * constructors of main.cpp:29-58 and cluster::cluster (cluster.cpp:21-40). */
fipi_status fipi_create(const fipi_params* p, fipi_precision prec, int device, fipi_ctx** out);
fipi_status fipi_destroy(fipi_ctx* ctx);
/* Bytes of device memory held by the context. */
fipi_status fipi_device_bytes(const fipi_ctx* ctx, size_t* out);
/* Replaces the physical constants of a live context (the reference fixes
 * them at compile time, head.hpp:44-58, parameter.hpp:18): sigma, epsilon,
 * lambda, mobility, mu, rho1, rho2, gravity, A and k_n; they take effect at
 * the next step.  Everything else must equal the context's parameters
 * (FIPI_ERR_BAD_PARAMS otherwise).  The state is kept, so a sensitivity
 * study or a finite-difference check needs no new context. */
fipi_status fipi_set_params(fipi_ctx* ctx, const fipi_params* p);

/* ----------------------------------------------------------------- state */
/* Initial phase field (field.cpp:85-99 drew it from rand()); resets t = 0
 * and the SBDF2 history, like entering main.cpp:75 with t = 0. */
fipi_status fipi_set_phase(fipi_ctx* ctx, const double* c);
/* Velocity field u (3 x V).  The reference starts from u = 0 (main.cpp:49). */
fipi_status fipi_set_velocity(fipi_ctx* ctx, const double* u);
/* Particle state (cluster::distribute, cluster.cpp:53-92, drew p from rand()).
 * p: n_p x 3 positions in [0, L).  r: n_p radii or NULL (= r_p, element.cpp:25).
 * cos_theta: n_p wettabilities or NULL (= 0, the reference's 90 degree form).
 * f_pp: n_p x 3 contact forces of the previous step or NULL (= 0); they are
 * spread at the next step (cluster.cpp:358).  The arrays are consumed before
 * the call returns; the upload completes in stream order (nothing waits). */
fipi_status fipi_set_particles(fipi_ctx* ctx, const double* p, const double* r,
                               const double* cos_theta, const double* f_pp);
fipi_status fipi_get_phase(fipi_ctx* ctx, double* c);
fipi_status fipi_get_velocity(fipi_ctx* ctx, double* u);
/* Any output pointer may be NULL.  f_pi is the attachment force of the last
 * stage (element.cpp:75-97). */
fipi_status fipi_get_particles(fipi_ctx* ctx, double* p, double* f_pp, double* f_pi);
/* Device-pointer variants (zero host copies): the same FP64 layouts as the
 * host calls above, in device memory of the context's device (e.g. a torch
 * CUDA tensor's data pointer).  They return once the arrays have been read
 * or written (the context stream is synchronised). */
fipi_status fipi_set_phase_device(fipi_ctx* ctx, const double* d_c);
fipi_status fipi_set_velocity_device(fipi_ctx* ctx, const double* d_u);
fipi_status fipi_set_particles_device(fipi_ctx* ctx, const double* d_p, const double* d_r,
                                      const double* d_cos_theta, const double* d_f_pp);
fipi_status fipi_get_phase_device(fipi_ctx* ctx, double* d_c);
fipi_status fipi_get_velocity_device(fipi_ctx* ctx, double* d_u);
fipi_status fipi_get_particles_device(fipi_ctx* ctx, double* d_p, double* d_f_pp, double* d_f_pi);
fipi_status fipi_get_time(const fipi_ctx* ctx, int* t);

/* ------------------------------------------------------------------ step */
/* Advances `nsteps` iterations of the loop body of main.cpp:75-219
 * (Cahn-Hilliard, Stokes, two Heun particle stages). */
fipi_status fipi_step(fipi_ctx* ctx, int nsteps);
/* Enqueues the steps without waiting for them; errors raised on the device
 * (particle out of range, non-finite state) are reported by the next
 * fipi_sync, fipi_step or state read. */
fipi_status fipi_step_async(fipi_ctx* ctx, int nsteps);
fipi_status fipi_sync(fipi_ctx* ctx);
/* The three parts of one iteration, for callers that interleave their own
 * work between them: the Cahn-Hilliard update (main.cpp:79-141), the
 * spreading and Stokes solve (main.cpp:146-181), the two particle stages
 * (main.cpp:186-219, ending the iteration: t += 1).  In this order they give
 * the same results as fipi_step(ctx, 1); any other order is
 * FIPI_ERR_STATE, and so is fipi_step while an iteration is open. */
fipi_status fipi_step_ch(fipi_ctx* ctx);
fipi_status fipi_step_stokes(fipi_ctx* ctx);
fipi_status fipi_step_particles(fipi_ctx* ctx);
/* The CUDA stream the context runs on (as a void*: cudaStream_t). */
fipi_status fipi_stream(const fipi_ctx* ctx, void** stream);

/* ------------------------------------------------------------ diagnostics */
/* integral of phi: sum c dx dy dz.  FP64 form: compensated sum of the real
 * field; mixed form: the FP64 k = 0 mode.  Not in the reference. */
fipi_status fipi_mass(fipi_ctx* ctx, double* out);
/* Total free energy sum lambda (0.5|grad c|^2 + 0.25/eps^2 (c^2-1)^2) dx^3
 * (main.cpp:232 + field.cpp:507-516), compensated sum. */
fipi_status fipi_free_energy(fipi_ctx* ctx, double* out);
/* Packing energy tau of the last contact-force evaluation (cluster.cpp:189-259). */
fipi_status fipi_packing_tau(fipi_ctx* ctx, double* out);

/* -------------------------------------------------------- instrumentation
 * Not in the reference (its only timing is clock() around the whole run,
 * main.cpp:25-26, 248-249).  Every kernel launch of the library is
 * counted; with timing enabled each launch is bracketed by CUDA events on
 * the context stream and accumulated per kernel class together with the
 * kernel's algorithmic bytes per launch (arrays it must read and write). */
fipi_status fipi_set_kernel_timing(fipi_ctx* ctx, int enable); /* also resets the stats */
fipi_status fipi_kernel_stat_count(fipi_ctx* ctx, int* n);
fipi_status fipi_kernel_stats(fipi_ctx* ctx, int i, char* name, int name_cap, long long* launches,
                              double* total_ms, double* bytes_per_launch);
/* Kernels launched by this context since creation. */
fipi_status fipi_launch_count(const fipi_ctx* ctx, long long* n);
/* Fused multiply-add throughput of `device` in TFLOP/s (an FMA counted as
 * two FLOPs), FP64 (fp64 != 0) or FP32, measured with a kernel of
 * independent FMA chains on every SM (about 20 ms of device time).  The FP64
 * form of the step is bound by this rate, not by HBM, on GB300. */
fipi_status fipi_fma_peak(int device, int fp64, double* tflops);

/* ------------------------------------------ fine-grained parity entry points
 * One call per reference function, on host arrays; they use the context's
 * grid and particle count but do not touch its step state. */

/* 3-D real-to-half-spectrum DFT, sign -1, unnormalised (field::fft,
 * field.cpp:438-443, restricted to a real input).  Output layout:
 * out[((kz*(nx/2+1)) + kx)*ny + ky] as (re, im) pairs, i.e. the half
 * spectrum with kx in [0, nx/2], ky fastest. */
fipi_status fipi_fft_r2c(fipi_ctx* ctx, const double* in, double* out);
/* Inverse of the above, normalised by 1/V like field::ifft + normalize
 * (field.cpp:446-455, primitive.cpp:54-62): real part of the inverse DFT
 * of the Hermitian completion of the half spectrum. */
fipi_status fipi_fft_c2r(fipi_ctx* ctx, const double* in, double* out);
/* grad c = ifft(i k c_hat) with the Nyquist index of each component zeroed
 * (field::grad, field.cpp:288-328, then ifft).  c: V reals, out: 3 x V. */
fipi_status fipi_grad(fipi_ctx* ctx, const double* c, double* grad_out);
/* cluster::sorting (cluster.cpp:116-169): cell key of every particle,
 * particle ids sorted by (cell, id), cell offsets (n_cells + 1 entries).
 * Any output may be NULL.  Returns FIPI_ERR_OUT_OF_RANGE like the reference's
 * out-of-range exit. */
fipi_status fipi_cells_build(fipi_ctx* ctx, const double* p, int* keys, int* sorted_ids,
                             int* cell_offsets);
/* cluster::compute_f_pp(t) (cluster.cpp:174-275): contact forces, n_p x 3.
 * f_pi (n_p x 3, may be NULL = all zero) only feeds the packing energy tau. */
fipi_status fipi_f_pp(fipi_ctx* ctx, const double* p, int t, const double* f_pi,
                      double* f_pp, double* tau);
/* The set of interacting pairs found by compute_f_pp (|d| < r_eq), as
 * (i, j) with i < j, sorted; *n_pairs receives the count.  pairs may be
 * NULL to query the count; max_pairs bounds what is written. */
fipi_status fipi_pairs(fipi_ctx* ctx, const double* p, int* pairs, int max_pairs, int* n_pairs);
/* element::get_local_c / get_local_dcdx via field::interpolate
 * (element.cpp:55-71, field.cpp:223-248): trilinear values of `fields`
 * (nfields x V reals) at the particles -> out (n_p x nfields). */
fipi_status fipi_interpolate(fipi_ctx* ctx, const double* fields, int nfields, const double* p,
                             double* out);
/* element::get_f_pi (element.cpp:75-97) for every particle, with the
 * contact-angle extension f_mag = -A pi (d - r cos_theta) sigma
 * (cos_theta = 0 is the reference).  c_loc: n_p, dcdx: n_p x 3. */
fipi_status fipi_f_pi(fipi_ctx* ctx, const double* c_loc, const double* dcdx, const double* r,
                      const double* cos_theta, double* f_pi);
/* element::advect (element.cpp:156-173) + element::enforce_bc
 * (element.cpp:177-185).  stage 1: u_old = F/(6 pi mu r), p_old = p,
 * p += dt u_old; stage 2: u = F/(6 pi mu r), p = p_old + dt/2 (u_old + u).
 * p, p_old, u_old are updated in place (n_p x 3). */
fipi_status fipi_advect(fipi_ctx* ctx, int stage, const double* f_pi, const double* f_pp,
                        const double* r, double* p, double* p_old, double* u_old);
/* field::interpolate2 (field.cpp:250-281; not called by the reference's
 * loop): the size-3-stencil variant of fipi_interpolate, same layout. */
fipi_status fipi_interpolate2(fipi_ctx* ctx, const double* fields, int nfields, const double* p, double* out);
/* field::div (field.cpp:332-361) + field::ifft, real part (not called by the
 * reference's loop): divergence of a real vector field v (3 x V) -> out (V). */
fipi_status fipi_div(fipi_ctx* ctx, const double* v, double* out);
/* element::enforce_bc (element.cpp:177-185) / cluster::enforce_bc:
 * p = fmod(p + L, L) per axis, n_p x 3 in place. */
fipi_status fipi_wrap(fipi_ctx* ctx, double* p);
/* cluster::compute_f_r (cluster.cpp:344-410): trilinear spreading of
 * f_pp / (dx dy dz) onto the grid, out: 3 x V.  Deterministic: per grid
 * node the contributions are summed in ascending particle id. */
fipi_status fipi_spread(fipi_ctx* ctx, const double* p, const double* f_pp, double* out);

/* ---------------------------------------------- no-allocation cell list
 * No counterpart in the reference.  The cell-list build of
 * fipi_cells_build (cluster::sorting) for callers that cannot call
 * cudaMalloc: code inside a host framework that owns a fixed device pool,
 * real-time loops that forbid driver allocations, or callers that only
 * hand over buffers they already hold.  It needs no context and allocates
 * nothing; its scratch is a fixed array inside the library (about 2.4 MB
 * on every GPU that loads the library, held until the process exits),
 * sized for at most FIPI_NOALLOC_MAX_PARTICLES particles; larger n_p is
 * rejected with FIPI_ERR_UNSUPPORTED.
 *   p          grid/box/cell parameters and n_p
 *   d_pos      device, n_p x 3 doubles (particle-major)
 *   d_keys     device, n_p ints: cell key of each particle (by id)
 *   d_sorted   device, n_p ints: particle ids sorted by (cell, id)
 *   d_offsets  device, n_cells + 1 ints
 *   stream     cudaStream_t (as void*) the work is queued on; the call
 *              synchronises it before returning the status
 * The first call on a device looks up the scratch's device address (with
 * that device current); make that first call before any stream capture.
 * All calls share the one scratch array: calls whose work overlaps on the
 * GPU (other threads, other streams) race and must be serialised. */
#define FIPI_NOALLOC_MAX_PARTICLES 65536
fipi_status fipi_cells_build_noalloc(const fipi_params* p, const double* d_pos, int* d_keys,
                                     int* d_sorted, int* d_offsets, void* stream);

/* ------------------------------------------------------------- VTK output
 * The reference's output step (main.cpp:225-238): legacy ASCII VTK files
 * written by field::output_to_file (field.cpp:469-503) and cluster::output
 * (cluster.cpp:415-456).  The host writers below produce, for the same
 * values, the same bytes as the reference.  They need no device. */
/* Structured-points field: components 1 (SCALARS, V values) or 3 (VECTORS,
 * 3 x V values, component-major like field::v), named `name`. */
fipi_status fipi_vtk_write_field(const fipi_params* p, const char* path, const char* name, int components,
                                 const double* values);
/* Particles: positions / dx, radii / dx (r NULL = r_p) and
 * |f_pp| / A / pi / sigma / r_p; pos and f_pp are n x 3. */
fipi_status fipi_vtk_write_particles(const fipi_params* p, const char* path, int n, const double* pos,
                                     const double* r, const double* f_pp);
/* The free-energy density field lambda (0.5 |grad c|^2 + 0.25/eps^2 (c^2-1)^2)
 * of main.cpp:232 (c: V, grad_c: 3 x V, out: V). */
fipi_status fipi_free_energy_density(const fipi_params* p, const double* c, const double* grad_c, double* out);
/* The context's current state: the phase field ("phase"), the free-energy
 * density ("free_energy"), the velocity ("u") or the particles. */
#define FIPI_VTK_PHASE 0
#define FIPI_VTK_FREE_ENERGY 1
#define FIPI_VTK_VELOCITY 2
#define FIPI_VTK_PARTICLES 3
fipi_status fipi_write_vtk(fipi_ctx* ctx, int what, const char* path);

/* ------------------------------------------------------------ checkpoints
 * No counterpart in the reference (it has no checkpoint or restart).  A
 * checkpoint is a device-resident copy of everything one step reads from
 * the previous one: c, grad c, the spectra c_hat, f_hat and the SBDF2
 * histories c_hat_old, f_hat_old, C_hat_old, the velocity spectrum (kept
 * after its inverse z pass, the form the step starts from), positions,
 * radii, cos(theta) and f_pp (spread at the next step, cluster.cpp:358),
 * the step index t (the contact ramp depends on it) and, in the mixed form,
 * the FP64 k = 0 record.  Slots live in HBM so the sqrt(N) schedule of the
 * adjoint costs device copies only.  Resuming from a slot is bit-exact. */
/* Allocates `slots` checkpoint slots (frees the previous ones). */
fipi_status fipi_checkpoint_reserve(fipi_ctx* ctx, int slots);
/* Bytes of one slot's payload; the exported blob is this plus a 64-byte header. */
fipi_status fipi_checkpoint_bytes(const fipi_ctx* ctx, size_t* bytes);
fipi_status fipi_checkpoint_save(fipi_ctx* ctx, int slot);
fipi_status fipi_checkpoint_load(fipi_ctx* ctx, int slot);
/* Host copies of a slot: a header (magic "FIPICKP1", precision, grid, n_p,
 * t, payload size) followed by the payload.  Import checks the header
 * against the context. */
fipi_status fipi_checkpoint_export(fipi_ctx* ctx, int slot, void* blob, size_t blob_bytes);
fipi_status fipi_checkpoint_import(fipi_ctx* ctx, int slot, const void* blob, size_t blob_bytes);

/* ---------------------------------------------------------------- adjoint
 * No counterpart in the reference.  Reverse-mode derivative of the FP64
 * step (FIPI_FP64 contexts; FIPI_ERR_UNSUPPORTED otherwise).  The
 * cotangent lives in the context and refers to one state: its c (as a real
 * field; c_hat, f_hat and grad c of that state are functions of c), the
 * real-field equivalents of the three SBDF2 histories, u, the positions and
 * f_pp.  Branches of the step (floor of the interpolation cell, the
 * |phi| <= tanh 2 and |d| < r tests of element.cpp:84-89, the pair test
 * |d| < r_eq of cluster.cpp:246) are held fixed: the derivative is the one
 * of the branch the forward step took. */
/* Sets the cotangent of the context's current state (any pointer NULL =
 * zero): dc V reals, du 3 x V, dp and df_pp n_p x 3. */
fipi_status fipi_adjoint_seed(fipi_ctx* ctx, const double* dc, const double* du, const double* dp,
                              const double* df_pp);
/* Reverses one step.  `slot` holds the state at the start of the step
 * whose end state the cotangent refers to (its t must be one less); the
 * step is recomputed from it with its intermediates kept, then the
 * cotangent is carried back to that state.  The context's state is left
 * at the end of the recomputed step. */
fipi_status fipi_adjoint_step(fipi_ctx* ctx, int slot);
/* The cotangent (any pointer may be NULL): dc V, du 3 x V, dp, df_pp n_p x 3. */
fipi_status fipi_adjoint_get(fipi_ctx* ctx, double* dc, double* du, double* dp, double* df_pp);
/* Cotangents of the step's parameters, summed over every step reversed
 * since fipi_adjoint_seed (after fipi_trajectory_backward: the gradient of
 * the trajectory's loss with respect to parameters that are constant along
 * it).  The mobility enters the CH update (main.cpp:106-127), lambda the
 * bulk potential f = (lambda/eps^2)(c^3 - c) (main.cpp:81), mu_hat = lambda
 * k^2 c_hat + f_hat (main.cpp:153) and the CH denominators, k_n the contact
 * forces (cluster.cpp:246-255) and sigma the attachment force f_pi
 * (element.cpp:89).  `sigma` is the total derivative with lambda =
 * 3 sigma eps / (2 sqrt 2) (head.hpp:47) and k_n = sigma / 2
 * (parameter.hpp:18) following sigma; the partial derivatives are given
 * too.  dcos_theta (n_p, may be NULL): the cotangent of each particle's
 * wettability cos(theta) of the contact-angle extension of f_pi.  The
 * history terms of the trajectory's start state (its c_hat, f_hat and C_hat
 * histories) are held fixed, except f_hat, which is a function of c there.
 * Needs lambda != 0 (FIPI_ERR_UNSUPPORTED otherwise). */
typedef struct fipi_param_grads {
    double mobility;     /* dL/dM                                           */
    double sigma;        /* dL/dsigma (lambda and k_n following sigma)       */
    double lambda;       /* partial dL/dlambda                               */
    double k_n;          /* partial dL/dk_n                                  */
    double sigma_attach; /* partial dL/dsigma through f_pi alone              */
} fipi_param_grads;
fipi_status fipi_adjoint_get_params(fipi_ctx* ctx, fipi_param_grads* out, double* dcos_theta);
/* Cotangents of the SBDF2 histories as real fields (V each, NULL = skip). */
fipi_status fipi_adjoint_get_history(fipi_ctx* ctx, double* dc_old, double* df_old, double* dconv_old);
/* Whole-trajectory gradient with sqrt(N) checkpointing.
 * fipi_trajectory_forward advances nsteps from the current state, saving a
 * checkpoint every `stride` steps (stride <= 0: ceil(sqrt(nsteps))) into
 * slots it reserves (ceil(nsteps/stride) + stride + 1 of them).
 * fipi_trajectory_backward seeds the cotangent of the final state and
 * reverses every step: each segment is run once more from its checkpoint
 * with its states kept in slots and the velocity and chemical potential
 * each step forms kept in a per-segment tape (4 V doubles per step, stride
 * steps; allocated on the first call), then reversed step by step from
 * those without recomputing the steps again.  The gradient with respect to
 * the trajectory's first state is then read with fipi_adjoint_get, and with
 * respect to the parameters with fipi_adjoint_get_params. */
fipi_status fipi_trajectory_forward(fipi_ctx* ctx, int nsteps, int stride);
fipi_status fipi_trajectory_backward(fipi_ctx* ctx, const double* dc, const double* du, const double* dp,
                                     const double* df_pp);

/* ------------------------------------------------ seeded synthetic inputs
 * Host-only helpers (no device needed).  The reference draws its initial
 * state from unseeded rand() (field.cpp:96, cluster.cpp:59-89); these draw
 * from a splitmix64 stream so runs are reproducible. */
/* c[i] = mean + amp * U(-1, 1), V values. */
fipi_status fipi_seed_phase(const fipi_params* p, uint64_t seed, double mean, double amp, double* c);
/* n_p positions uniform in the box (n_p x 3), radii U[r_min, r_max],
 * contact angles U[theta_min, theta_max] degrees returned as cos(theta).
 * Without allow_overlap the spheres are placed by random sequential
 * addition with the periodic minimum-image distance >= r_i + r_j
 * (the reference's check_overlap, cluster.cpp:98-113, ignores periodic
 * images).  r and cos_theta may be NULL. */
fipi_status fipi_seed_particles(const fipi_params* p, uint64_t seed, double r_min, double r_max,
                                double theta_min_deg, double theta_max_deg, int allow_overlap,
                                double* pos, double* r, double* cos_theta);

/* ------------------------------------------------ particle-model extensions
 * The reference carries a fluid-to-particle coupling and a Brownian force
 * that its step never uses: get_local_u sets uf = 0 with the interpolation
 * commented out (element.cpp:38-52), and get_f_rand / get_f_drag
 * (element.cpp:109-150) are never called.  Both are off by default (the
 * step is then the reference's); the adjoint rejects contexts with either on.
 *
 * fipi_set_fluid_coupling(ctx, 1): every stage interpolates the fluid
 * velocity u^{n+1} at the particle (field::interpolate per component, the
 * commented-out body of get_local_u) and advects with
 * uf + (f_pi + f_ext + f_pp)/(6 pi mu r) (element.cpp:163, 170).  The drag
 * f_drag = -6 pi r mu (u - uf) of element.cpp:147-150 then balances the
 * other forces exactly and is not stored.
 *
 * fipi_set_brownian(ctx, kt, seed): kt > 0 adds to both stages of step t
 * f_rand = sqrt(12 pi r mu kt / dt) g (element.cpp:138-143, with the
 * particle's radius), g three standard normals drawn as get_f_rand draws
 * them -- Box-Muller on uniforms (k mod 1000)/1000, redrawn while |g| > 5 --
 * from Philox-4x32-10 keyed by seed with counter (particle, t, block, 0)
 * instead of rand().  kt = 0 switches it off. */
fipi_status fipi_set_fluid_coupling(fipi_ctx* ctx, int on);
fipi_status fipi_set_brownian(fipi_ctx* ctx, double kt, uint64_t seed);

/* Mass-conserving mode (off by default: the step is then the reference's).
 * The reference's wave vector takes +N/2 at the Nyquist index for a mode and
 * its mirror alike (field.cpp:108-115), so the projected velocity is not
 * exactly divergence-free against the Nyquist-zeroed gradient and the k = 0
 * mode of the advection term u . grad c (main.cpp:88-92) is not zero: the
 * integral of phi drifts (about 4e-11 of sum |phi| dV over 1000 steps at
 * 256^3).  With on != 0 that mode is taken as 0 in the Cahn-Hilliard update
 * of both forms (and in the adjoint), so the integral of phi stays constant
 * to rounding; every other mode is unchanged. */
fipi_status fipi_set_mass_conserving(fipi_ctx* ctx, int on);

/* Test hooks of the bounded device waits (not for production runs).
 * FIPI_DEBUG_FFT_FIRST_WAIT_POLLS: the number of polls the first bulk-copy
 * wait of every Y-pass block makes before it gives up (-1 restores the
 * normal bound of 2^22 polls; 0 gives up at once).  A block that gives up
 * sets the device error word, waits (with the normal bound) for its copies
 * in flight and returns, so the call reports FIPI_ERR_TIMEOUT and the
 * context stays usable.  Later waits of the block keep the normal bound. */
#define FIPI_DEBUG_FFT_FIRST_WAIT_POLLS 1
fipi_status fipi_set_debug(fipi_ctx* ctx, int what, long long value);

/* The reference's own initial state for a given seed (host only): srand(seed)
 * (main.cpp:24 seeds from the clock), then the phase field's V draws
 * c = (rand()%1000)/1e3*0.2 - 0.1 in index order (field.cpp:85-99) and,
 * when switch_particle, cluster::distribute (cluster.cpp:53-113): per
 * particle, candidates p = L (rand()%1000)/1e3 (3 draws) until none of the
 * earlier particles lies closer than 2 r_p (check_overlap, cluster.cpp:98-113,
 * no periodic images).  rand() is glibc's generator, restated so every host
 * draws the same values.  c: V values or NULL (drawn either way); pos:
 * n_p x 3 or NULL.  FIPI_ERR_BAD_PARAMS when a particle finds no place in
 * 1e7 candidates (the reference would loop forever). */
fipi_status fipi_reference_initial_state(const fipi_params* p, unsigned int seed, double* c, double* pos);

#ifdef __cplusplus
}
#endif
#endif /* FIPI_H */
