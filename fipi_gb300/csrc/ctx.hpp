// Internal context of the FIPI GB300 library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/fipi.h"
#include "fft.cuh"

namespace fipi {

// Device buffers of one precision form.  T = float (mixed) or double.
struct FieldBufs {
    void* twx = nullptr;  // exp(-2 pi i q / nx), q < nx     (cplx<T>)
    void* twy = nullptr;  // exp(-2 pi i q / ny)
    void* twz = nullptr;  // exp(-2 pi i q / nz)
    void* kx = nullptr;   // wave numbers (T): kx[0..M], ky[0..ny), kz[0..nz)
    void* ky = nullptr;
    void* kz = nullptr;
    // real fields (T, V each)
    void* c = nullptr;       // phase field c^n
    void* g[3] = {};         // grad c^n
    void* fsp[3] = {};       // spread particle force density (cluster::compute_f_r)
    void* ureal = nullptr;   // 3V, velocity materialised on demand
    // spectral fields (cplx<T>, SH each)
    void* chat = nullptr;
    void* chat_old = nullptr;
    void* fhat = nullptr;
    void* fhat_old = nullptr;
    void* Chat_old = nullptr;
    void* upre[3] = {};  // velocity state: Z^-1 u_hat (the first pass of u = C2R(u_hat))
    void* S[4] = {};  // scratch
};

// Cell-list / sort scratch of the particle side.
struct ParticleBufs {
    int n = 0;
    int ncell[3] = {0, 0, 0};
    double dcell[3] = {0, 0, 0};
    int ncells = 0;
    // state, SoA, FP64
    double* p = nullptr;      // 3 x n (x[n], y[n], z[n])
    double* p_old = nullptr;  // 3 x n
    double* u_old = nullptr;  // 3 x n
    double* f_pp = nullptr;   // 3 x n
    double* f_pi = nullptr;   // 3 x n
    double* r = nullptr;      // n
    double* cth = nullptr;    // n
    // cell list
    unsigned* keys = nullptr;      // n
    unsigned* keys_alt = nullptr;  // n
    unsigned* ids = nullptr;       // n (sorted particle ids)
    unsigned* ids_alt = nullptr;   // n
    int* cell_off = nullptr;       // ncells + 1
    int* cell_cnt = nullptr;       // ncells
    // spreading records (8 per particle)
    unsigned* sp_keys = nullptr;      // 8n node index
    unsigned* sp_keys_alt = nullptr;  // 8n
    unsigned* sp_vals = nullptr;      // 8n record id = particle*8 + corner
    unsigned* sp_vals_alt = nullptr;  // 8n
    unsigned* sp_prev = nullptr;      // 8n nodes written by the previous spread
    // mixed form: per node 32 bytes, the three fixed-point spread sums and,
    // in the low half of the fourth word, the FP32 sum of |contribution|
    // (the range bound): one 32-byte sector per touched node
    unsigned long long* sp_acc = nullptr;
    int sp_prev_valid = 0;
    // radix sort scratch
    unsigned* hist = nullptr;  // 256 * max_blocks
    int hist_cap = 0;
    // diagnostics
    double* tau_part = nullptr;  // n, per-particle packing-energy terms
    float4* spos = nullptr;      // n, sorted cell-relative FP32 positions + id (mixed form)
    void* sp_fw = nullptr;       // 6 x n (TA): spread force density (3) and trilinear fractions (3)
    unsigned long long* ymax = nullptr;  // [max p_y bits, first index] for it_mark
    bool tau_valid = false;
    int* it_mark = nullptr;      // 1
    double* tau = nullptr;       // 1
    // extensions (off by default): fluid velocity at the particle and the
    // Brownian force of the current step
    double* uf = nullptr;      // 3 x n
    double* f_rand = nullptr;  // 3 x n
};

// Device-resident checkpoints of the step state (one allocation, `slots`
// payloads of `bytes` each).
struct CheckpointStore {
    int slots = 0;
    size_t bytes = 0;
    unsigned char* base = nullptr;
    std::vector<int> t;  // step index held by each slot, -1 = empty
    // the last fipi_trajectory_forward: first step, steps, stride, segments
    struct Traj {
        int t0 = -1, n = 0, s = 0, K = 0;
    } traj;
};

// Reverse-mode state of the FP64 step.  Cotangents of spectral state are
// kept as half spectra of the real-field cotangent (la = R2C(lambda)), so
// every Fourier multiplier of the step is its own adjoint.
struct AdjBufs {
    bool ready = false;
    int t = -1;  // step index of the state the cotangent refers to
    // spectral (cplx<double>, SH each)
    void* la_c = nullptr;   // c of the state (c_hat, f_hat, grad c folded in)
    void* la_co = nullptr;  // SBDF2 histories c_hat_old, f_hat_old, C_hat_old
    void* la_fo = nullptr;
    void* la_Co = nullptr;
    void* AS[5] = {};       // transform scratch
    // real fields (double)
    double* la_u = nullptr;  // 3V
    double* lamF = nullptr;  // 3V cotangent of the force density F of the Stokes solve
    double* part = nullptr;  // 4V particle cotangents on c^{n+1}, grad c^{n+1}
    double* tc0 = nullptr;   // V   tape: c^n
    double* tg0 = nullptr;   // 3V  tape: grad c^n
    double* tu = nullptr;    // 3V  tape: u^n
    double* tmu = nullptr;   // V   tape: mu^{n+1}
    // particles (SoA, 3n unless noted)
    double* la_p = nullptr;
    double* la_fpp = nullptr;
    double* tp0 = nullptr;     // positions at the step start
    double* tfpp0 = nullptr;   // f_pp at the step start (spread in the step)
    double* p1 = nullptr;      // stage-1 positions
    double* fpi1 = nullptr;
    double* fpp1 = nullptr;
    double* loc = nullptr;     // 8n: c, grad c interpolated at p^n (4n) and p1 (4n)
    double* lamF1 = nullptr;   // cotangent of the stage-1 contact forces
    double* lamF2 = nullptr;   // cotangent of the stage-2 contact forces
    double* lam_p1 = nullptr;  // cotangent of p1
    double* lamloc = nullptr;  // 8n cotangents of `loc`
    unsigned* rk = nullptr;    // 16n spreading records (node, record) + ping-pong
    unsigned* rv = nullptr;
    unsigned* rk2 = nullptr;
    unsigned* rv2 = nullptr;
    double* rw = nullptr;      // 14n: fractions (3) and cotangents (4) of 2n interpolations
    double* rmp = nullptr;     // 1: ramp factor of the reversed step
    // parameter cotangents, summed from fipi_adjoint_seed over every reversed step
    double* pg = nullptr;       // kParamGrads doubles: mobility, lambda, k_n, sigma through f_pi
    double* pg_part = nullptr;  // per-block partial sums of one reduction
    int pg_nparts = 0;
    void* tfo = nullptr;        // SH tape: f_hat^{n-1} (the start state's f_hat history)
    double* dct = nullptr;      // n: cotangent of each particle's cos(theta)
    double* pp_sig = nullptr;   // n: per-particle terms of the sigma (f_pi) cotangent of one step
    double* pp_kn = nullptr;    // n: per-particle terms of the k_n cotangent of one step
    // per-step tapes of a trajectory segment (u^n, mu^{n+1}: 4V doubles each)
    double* seg_tape = nullptr;
    int seg_tape_steps = 0;
};
// Slots of AdjBufs::pg.
enum : int { kPgMobility = 0, kPgLambda = 1, kPgKn = 2, kPgSigmaAttach = 3, kParamGrads = 4 };

}  // namespace fipi

namespace fipi {
// Per-kernel-class instrumentation: launch counts always, CUDA-event
// durations on the context stream when enabled.
struct KernelStat {
    std::string name;
    long long launches = 0;
    double ms = 0.0;
    double bytes = 0.0;      // algorithmic bytes per launch (mean over the timed launches)
    double bytes_sum = 0.0;  // algorithmic bytes of all timed launches
};
struct PendingLaunch {
    int idx;
    double bytes;
    std::pair<cudaEvent_t, cudaEvent_t> ev;
};
struct KTimer {
    bool enabled = false;
    long long launches = 0;
    std::vector<KernelStat> stats;
    std::vector<PendingLaunch> pending;
    std::vector<cudaEvent_t> pool;
};
}  // namespace fipi

struct fipi_ctx {
    fipi_params P{};
    fipi_precision prec = FIPI_FP64;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    fipi::Geom g{};
    fipi::FieldBufs fb;
    fipi::ParticleBufs pb;
    double* k0 = nullptr;        // mixed form FP64 k=0 mode: [c0, c0_old, C0_old, C0_cur, (float) c0/V]
    double* partials = nullptr;  // per-block FP64 partial sums
    int n_partials = 0;
    int* status = nullptr;       // device error word
    double* scratch_d = nullptr; // small FP64 device scratch (reductions)
    int t = 0;
    int* d_t = nullptr;          // device copy of t (advanced by step_tick or the last advection)
    double* d_rmp = nullptr;     // ramp(t + 1, 0.2 t_end) for the next step
    // CUDA graphs of one step (t >= 1) for each of the two states of the
    // ping-pong buffers; `after` is the host-side buffer state the step leaves
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        void* key = nullptr;     // fb.chat when captured (identifies the state)
        fipi::FieldBufs fb_after;
        fipi::ParticleBufs pb_after;
        long long launches = 0;
    } graphs[2];
    bool use_graphs = true;
    int substep = 0;           // 1 after fipi_step_ch, 2 after fipi_step_stokes
    double* pin = nullptr;     // pinned host staging of the particle state, 12 n doubles
    double* pin_dev = nullptr; // the same buffer as a device pointer (mapped pinned memory)
    bool have_phase = false;
    int couple_u = 0;          // fluid coupling: uf = u interpolated at the particle
    int conserve_mass = 0;     // the k = 0 mode of u . grad c taken as 0 (exact mass conservation)
    int debug_first_wait = -1; // test hook: polls of each Y-pass block's first copy wait (-1: normal)
    double brown_kt = 0.0;     // Brownian force strength kT (0: off)
    uint64_t noise_seed = 0;   // Philox key of the Brownian force
    bool track_tau = true;     // packing energy during the step (cluster.cpp:256-259)
    size_t device_bytes = 0;
    std::string last_error;
    fipi::KTimer kt;
    fipi::CheckpointStore ck;
    fipi::AdjBufs ad;
    // forward-step tape (non-NULL only while the adjoint recomputes a step):
    // u^n from the conv pass, mu^{n+1} from the force pass
    void* tape_u[3] = {};
    void* tape_mu = nullptr;
};

namespace fipi {

// fields.cu
fipi_status fields_alloc(fipi_ctx* ctx);
void fields_free(fipi_ctx* ctx);
// Set c^0 (host doubles) and derive c_hat, f_hat, grad c (t = 0 state).
// State I/O from / to host memory, or with `dev` device memory (no host copy).
fipi_status fields_set_phase(fipi_ctx* ctx, const double* c, bool dev = false);
fipi_status fields_set_velocity(fipi_ctx* ctx, const double* u, bool dev = false);
fipi_status fields_get_phase(fipi_ctx* ctx, double* c, bool dev = false);
fipi_status fields_get_velocity(fipi_ctx* ctx, double* u, bool dev = false);
// The three grid sub-steps of one iteration (enqueue only).
void fields_step_ch(fipi_ctx* ctx, int t);        // conv, CH update, c, f
void fields_step_stokes(fipi_ctx* ctx);           // mu, grad c, force, projection
fipi_status fields_get_grad(fipi_ctx* ctx, double* g_host);  // grad c of the state, 3 x V
fipi_status fields_mass(fipi_ctx* ctx, double* out);
fipi_status fields_free_energy(fipi_ctx* ctx, double* out);
// Fine-grained transforms on host arrays.
fipi_status fields_fft_r2c(fipi_ctx* ctx, const double* in, double* out);
fipi_status fields_fft_c2r(fipi_ctx* ctx, const double* in, double* out);
fipi_status fields_grad(fipi_ctx* ctx, const double* c, double* out);
fipi_status fields_div(fipi_ctx* ctx, const double* v, double* out);
// Device pointers of the real fields used by the particle side (T-typed).
const void* fields_real_c(fipi_ctx* ctx);
const void* fields_real_grad(fipi_ctx* ctx, int d);

// particles.cu
fipi_status particles_alloc(fipi_ctx* ctx);
void particles_free(fipi_ctx* ctx);
// Spread f_pp at p onto the dense spread grid (enqueue).
void particles_spread(fipi_ctx* ctx);
// Two Heun stages (enqueue); the ramp factor is read from ctx->d_rmp.
// Returns true when its last kernel also ended the step (step_tick's
// update); otherwise the caller enqueues step_tick.
bool particles_step(fipi_ctx* ctx);
fipi_status particles_ext_alloc(fipi_ctx* ctx);
void fields_velocity_real(fipi_ctx* ctx);  // fb.ureal = u (the fluid-coupling extension)
// t += 1 on the device and the next step's ramp factor.
void step_tick(fipi_ctx* ctx);
// Fine-grained parity entry points (synchronous, host arrays).
fipi_status particles_cells_build(fipi_ctx* ctx, const double* p, int* keys, int* sorted,
                                  int* offsets);
fipi_status particles_f_pp(fipi_ctx* ctx, const double* p, int t, const double* f_pi,
                           double* f_pp, double* tau);
fipi_status particles_pairs(fipi_ctx* ctx, const double* p, int* pairs, int max_pairs,
                            int* n_pairs);
fipi_status particles_interpolate(fipi_ctx* ctx, const double* fields, int nfields,
                                  const double* p, double* out);
fipi_status particles_interpolate2(fipi_ctx* ctx, const double* fields, int nfields,
                                   const double* p, double* out);
fipi_status particles_f_pi(fipi_ctx* ctx, const double* c_loc, const double* dcdx,
                           const double* r, const double* cth, double* f_pi);
fipi_status particles_advect(fipi_ctx* ctx, int stage, const double* f_pi, const double* f_pp,
                             const double* r, double* p, double* p_old, double* u_old);
fipi_status particles_spread_host(fipi_ctx* ctx, const double* p, const double* f_pp,
                                  double* out);
// Packing energy of the last contact-force evaluation.
fipi_status particles_packing_tau(fipi_ctx* ctx, double* out);
fipi_status particles_get_radii(fipi_ctx* ctx, double* r_host);
fipi_status particles_wrap(fipi_ctx* ctx, double* p_host);

// Reverse mode (adjoint.cu / particles.cu).
void enqueue_step(fipi_ctx* ctx);  // one forward step, direct launches
// Sets the device step index and the ramp factor of step t (particles.cu).
void set_tick(fipi_ctx* ctx, int t);
// Particle stages of the step reversed (after the taped forward step):
// la_p, la_fpp of the end state -> la_p of the start state (stage part) and
// the particle cotangents `part` on c^{n+1}, grad c^{n+1}.
fipi_status particles_adjoint(fipi_ctx* ctx);
// Adjoint of the spreading of f_pp^n at p^n, given lamF: la_fpp = I(p) lamF / dV,
// la_p += (f_pp / dV) grad_p I(p) lamF.
void particles_adjoint_spread(fipi_ctx* ctx);
fipi_status particles_adjoint_alloc(fipi_ctx* ctx);
void particles_adjoint_free(fipi_ctx* ctx);

// Brackets one kernel launch: counts it and, when timing is on, records
// events around it on the context stream (capi.cu).
struct LaunchScope {
    fipi_ctx* ctx;
    double bytes;
    int idx = -1;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    LaunchScope(fipi_ctx* c, const char* name, double bytes);
    ~LaunchScope();
};

// capi.cu helpers
fipi_status set_error(fipi_ctx* ctx, fipi_status st, const std::string& msg);
fipi_status cuda_check(fipi_ctx* ctx, cudaError_t e, const char* what);
// Synchronises the stream and turns the device error word into a status.
fipi_status check_status(fipi_ctx* ctx);
// Host n x 3 (particle-major) <-> device 3 x n (SoA), synchronous.
fipi_status upload_soa(fipi_ctx* ctx, const double* h, double* d, int n);
fipi_status download_soa(fipi_ctx* ctx, const double* d, double* h, int n);
void graphs_reset(fipi_ctx* ctx);
// adjoint.cu: frees checkpoint slots and adjoint buffers.
void adjoint_free(fipi_ctx* ctx);
// *dst += scale * (sum of part[0..np)), one block in a fixed order (deterministic).
void param_acc(fipi_ctx* ctx, const double* part, int np, double scale, double* dst);

}  // namespace fipi

// Stream-ordered synchronous copies: the context stream is non-blocking, so
// plain cudaMemcpy on the legacy stream would not order with its kernels.
inline cudaError_t h2d(fipi_ctx* ctx, void* d, const void* h, size_t n) {
    cudaError_t e = cudaMemcpyAsync(d, h, n, cudaMemcpyHostToDevice, ctx->stream);
    return e != cudaSuccess ? e : cudaStreamSynchronize(ctx->stream);
}
inline cudaError_t d2h(fipi_ctx* ctx, void* h, const void* d, size_t n) {
    cudaError_t e = cudaMemcpyAsync(h, d, n, cudaMemcpyDeviceToHost, ctx->stream);
    return e != cudaSuccess ? e : cudaStreamSynchronize(ctx->stream);
}
// Raises a kernel's dynamic shared-memory limit to `bytes` when needed and,
// on first use, asks for the largest shared-memory carveout so several
// blocks fit per SM (per kernel instantiation; `cur` remembers the grant and
// starts at a 48 KiB sentinel).  Without the attribute a kernel may only take
// 48 KiB minus its static shared memory, so the attribute is set on first
// use whatever the size.
template <class K> inline cudaError_t ensure_smem(K kern, size_t bytes, size_t& cur) {
    if (cur == 48 * 1024) {
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cur = 0;
    }
    if (bytes <= cur) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

#define FIPI_CUDA(ctx, call)                                                   \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) return fipi::cuda_check((ctx), e_, #call);      \
    } while (0)
