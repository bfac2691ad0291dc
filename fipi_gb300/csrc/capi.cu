// C ABI of the FIPI GB300 library: context lifecycle, state I/O, the step
// driver (main.cpp:75-219 of the reference) and the fine-grained parity
// entry points.  Errors are returned as fipi_status codes; the reference
// printed a message and called exit(0).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.hpp"

namespace {
thread_local std::string g_last_error;
}

namespace fipi {

fipi_status set_error(fipi_ctx* ctx, fipi_status st, const std::string& msg) {
    g_last_error = msg;
    if (ctx) ctx->last_error = msg;
    return st;
}

fipi_status cuda_check(fipi_ctx* ctx, cudaError_t e, const char* what) {
    return set_error(ctx, FIPI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

static cudaEvent_t take_event(fipi_ctx* ctx) {
    if (!ctx->kt.pool.empty()) {
        cudaEvent_t e = ctx->kt.pool.back();
        ctx->kt.pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

LaunchScope::LaunchScope(fipi_ctx* c, const char* name, double b) : ctx(c), bytes(b) {
    ctx->kt.launches++;
    if (!ctx->kt.enabled) return;
    auto& st = ctx->kt.stats;
    for (size_t i = 0; i < st.size(); ++i)
        if (st[i].name == name) idx = (int)i;
    if (idx < 0) {
        st.push_back(KernelStat{name, 0, 0.0, 0.0, 0.0});
        idx = (int)st.size() - 1;
    }
    e0 = take_event(ctx);
    e1 = take_event(ctx);
    cudaEventRecord(e0, ctx->stream);
}

LaunchScope::~LaunchScope() {
    if (idx < 0) return;
    cudaEventRecord(e1, ctx->stream);
    ctx->kt.pending.push_back({idx, bytes, {e0, e1}});
}

// Folds finished event pairs into the per-kernel totals.
static void drain_timer(fipi_ctx* ctx) {
    cudaStreamSynchronize(ctx->stream);
    for (auto& p : ctx->kt.pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.ev.first, p.ev.second);
        KernelStat& s = ctx->kt.stats[p.idx];
        s.launches++;
        s.ms += ms;
        s.bytes_sum += p.bytes;
        s.bytes = s.bytes_sum / (double)s.launches;
        ctx->kt.pool.push_back(p.ev.first);
        ctx->kt.pool.push_back(p.ev.second);
    }
    ctx->kt.pending.clear();
}

}  // namespace fipi

using namespace fipi;

static bool pow2_in(int n, int lo, int hi) { return n >= lo && n <= hi && (n & (n - 1)) == 0; }

static fipi_status validate(const fipi_params* P, fipi_precision prec) {
    if (!P) return set_error(nullptr, FIPI_ERR_BAD_ARG, "params is NULL");
    if (prec != FIPI_FP64 && prec != FIPI_MIXED) return set_error(nullptr, FIPI_ERR_BAD_PARAMS, "unknown precision");
    if (!pow2_in(P->nx, 8, 512) || !pow2_in(P->ny, 8, 512) || !pow2_in(P->nz, 8, 512))
        return set_error(nullptr, FIPI_ERR_UNSUPPORTED, "grid sizes must be powers of two in [8, 512]");
    if (prec == FIPI_MIXED && P->ny < 16)
        return set_error(nullptr, FIPI_ERR_UNSUPPORTED, "the mixed form needs ny >= 16");
    if (!(P->lx > 0 && P->ly > 0 && P->lz > 0 && P->dt > 0 && P->mu > 0 && P->epsilon > 0))
        return set_error(nullptr, FIPI_ERR_BAD_PARAMS, "box lengths, dt, mu and epsilon must be positive");
    if (!P->switch_ch || !P->switch_ns)
        return set_error(nullptr, FIPI_ERR_UNSUPPORTED,
                         "switch_ch = 0 or switch_ns = 0 is not built (use n_p = 0 or switch_particle = 0 "
                         "to drop the particles)");
    if (P->n_p < 0) return set_error(nullptr, FIPI_ERR_BAD_PARAMS, "n_p < 0");
    if (P->n_p > (1 << 28)) return set_error(nullptr, FIPI_ERR_UNSUPPORTED, "n_p too large");
    if (P->n_p > 0 && P->switch_particle) {
        if (!(P->r_eq > 0 && P->r_c > 0)) return set_error(nullptr, FIPI_ERR_BAD_PARAMS, "r_eq, r_c must be positive");
        int nc[3];
        double dc[3];
        const fipi_status gs = fipi_cell_geometry(P, nc, dc);
        if (gs != FIPI_OK) return gs;
        if (nc[0] < 3 || nc[1] < 3 || nc[2] < 3)
            return set_error(nullptr, FIPI_ERR_UNSUPPORTED,
                             "the cell grid needs at least 3 cells per axis (L/r_c >= 3); with fewer the "
                             "reference visits neighbour cells twice");
        if (!(P->r_eq > 0 && P->r_c > 0)) return set_error(nullptr, FIPI_ERR_BAD_PARAMS, "r_eq, r_c must be positive");
    }
    return FIPI_OK;
}

extern "C" {

int fipi_abi_version(void) { return FIPI_ABI_VERSION; }

const char* fipi_last_error_string(void) { return g_last_error.c_str(); }

fipi_status fipi_params_reference(fipi_params* o) {
    if (!o) return set_error(nullptr, FIPI_ERR_BAD_ARG, "out is NULL");
    // head.hpp:27-74, parameter.hpp:18-20
    const double pi = 3.1415926;
    std::memset(o, 0, sizeof(*o));
    o->nx = o->ny = o->nz = 64;
    o->lx = o->ly = o->lz = 2 * pi;
    o->pi = pi;
    o->dt = 1e-3;
    o->t_end = 20000;
    const double dx = o->lx / o->nx;
    o->sigma = 0.07;
    o->epsilon = 3.0 * dx / std::pow(2, 0.5) / 2.0;
    o->lambda = o->sigma * o->epsilon * 3.0 / 2.0 / std::pow(2, 0.5);
    const double r_drop = 0.4 * o->lx;
    o->gravity = -1e1;
    o->rho1 = 1e-3;
    o->rho2 = o->rho1 - 0.0 * o->sigma / o->gravity / r_drop / r_drop;
    o->mu = 1e-3;
    o->A = 2;
    o->mobility = std::pow(0.2 * o->epsilon, 2) / o->mu;
    o->r_p = 0.03 * r_drop;
    o->n_p = 20000;
    o->r_eq = 5 * o->r_p;
    o->r_c = 5 * o->r_p;
    o->k_n = 0.5 * o->sigma;
    o->margin = 0.0;
    o->switch_particle = o->switch_ch = o->switch_ns = 1;
    return FIPI_OK;
}

fipi_status fipi_cell_geometry(const fipi_params* P, int n_cell[3], double d_cell[3]) {
    if (!P || !n_cell || !d_cell) return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    const double L[3] = {P->lx, P->ly, P->lz};
    // the cell counts are converted to int below: r_c must be finite and
    // positive and every L / r_c within the int range first
    if (!(P->r_c > 0) || !std::isfinite(P->r_c) || !std::isfinite(P->margin))
        return set_error(nullptr, FIPI_ERR_BAD_PARAMS, "r_c must be finite and positive (and margin finite)");
    for (int a = 0; a < 3; ++a) {
        const double q = std::floor(L[a] / P->r_c + 2 * P->margin / P->r_c);
        if (!(q >= 0.0 && q <= 1073741824.0))
            return set_error(nullptr, FIPI_ERR_BAD_PARAMS, "cell count L / r_c outside [0, 2^30]");
    }
    for (int a = 0; a < 3; ++a) {
        n_cell[a] = (int)std::floor(L[a] / P->r_c + 2 * P->margin / P->r_c);  // cluster.cpp:26-28
        d_cell[a] = n_cell[a] > 0 ? std::fmod(L[a] + 2 * P->margin, P->r_c) / n_cell[a] + P->r_c : 0.0;
    }
    return FIPI_OK;
}

fipi_status fipi_create(const fipi_params* P, fipi_precision prec, int device, fipi_ctx** out) {
    if (!out) return set_error(nullptr, FIPI_ERR_BAD_ARG, "out is NULL");
    *out = nullptr;
    fipi_status st = validate(P, prec);
    if (st != FIPI_OK) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return set_error(nullptr, FIPI_ERR_NO_DEVICE, "no CUDA device visible");
    if (device < 0 || device >= ndev) return set_error(nullptr, FIPI_ERR_BAD_ARG, "device index out of range");
    fipi_ctx* ctx = new fipi_ctx();
    ctx->P = *P;
    ctx->prec = prec;
    ctx->device = device;
    auto fail = [&](fipi_status s) {
        std::string msg = ctx->last_error;
        fipi_destroy(ctx);
        set_error(nullptr, s, msg);
        return s;
    };
    if (cudaSetDevice(device) != cudaSuccess) return fail(cuda_check(ctx, cudaGetLastError(), "cudaSetDevice"));
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (ctx->num_sms < 1) ctx->num_sms = 1;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(cuda_check(ctx, e, "cudaStreamCreate"));
    e = cudaMalloc(&ctx->status, sizeof(int));
    if (e != cudaSuccess) return fail(cuda_check(ctx, e, "cudaMalloc(status)"));
    e = cudaMalloc(&ctx->d_t, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_rmp, sizeof(double));
    if (e != cudaSuccess) return fail(cuda_check(ctx, e, "cudaMalloc(step counter)"));
    cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->stream);
    st = fields_alloc(ctx);
    if (st != FIPI_OK) return fail(st);
    st = particles_alloc(ctx);
    if (st != FIPI_OK) return fail(st);
    if (ctx->pb.n > 0) {
        e = cudaMallocHost((void**)&ctx->pin, sizeof(double) * 12 * (size_t)ctx->pb.n);
        if (e != cudaSuccess) return fail(cuda_check(ctx, e, "cudaMallocHost(particle staging)"));
        e = cudaHostGetDevicePointer((void**)&ctx->pin_dev, ctx->pin, 0);
        if (e != cudaSuccess) return fail(cuda_check(ctx, e, "cudaHostGetDevicePointer(particle staging)"));
    }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(cuda_check(ctx, e, "init"));
    // default particle radii r_p (element.cpp:25)
    if (ctx->pb.n > 0) {
        std::vector<double> r(ctx->pb.n, P->r_p);
        e = h2d(ctx, ctx->pb.r, r.data(), sizeof(double) * r.size());
        if (e != cudaSuccess) return fail(cuda_check(ctx, e, "radii"));
    }
    *out = ctx;
    return FIPI_OK;
}


fipi_status fipi_destroy(fipi_ctx* ctx) {
    if (!ctx) return FIPI_OK;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    graphs_reset(ctx);
    if (ctx->d_t) cudaFree(ctx->d_t);
    if (ctx->d_rmp) cudaFree(ctx->d_rmp);
    drain_timer(ctx);
    for (cudaEvent_t e : ctx->kt.pool) cudaEventDestroy(e);
    adjoint_free(ctx);
    if (ctx->pin) cudaFreeHost(ctx->pin);
    fields_free(ctx);
    particles_free(ctx);
    if (ctx->status) cudaFree(ctx->status);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return FIPI_OK;
}

fipi_status fipi_device_bytes(const fipi_ctx* ctx, size_t* out) {
    if (!ctx || !out) return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    *out = ctx->device_bytes;
    return FIPI_OK;
}

}  // extern "C"

fipi_status fipi::check_status(fipi_ctx* ctx) {
    // the copy of the error word is ordered after all enqueued work, so one
    // synchronisation covers both
    int st = 0;
    FIPI_CUDA(ctx, d2h(ctx, &st, ctx->status, sizeof(int)));
    FIPI_CUDA(ctx, cudaGetLastError());
    if (st) {
        FIPI_CUDA(ctx, cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->stream));
        if (st & ERR_TMA_TIMEOUT) return set_error(ctx, FIPI_ERR_TIMEOUT, "a bulk-copy wait timed out in an FFT pass");
        if (st & ERR_NONFINITE) return set_error(ctx, FIPI_ERR_NONFINITE, "non-finite particle position");
        if (st & ERR_SPREAD_RANGE)
            return set_error(ctx, FIPI_ERR_RANGE, "a spread force density left the range of the fixed-point "
                                                  "accumulators (|sum| >= 2^31 per node)");
        return set_error(ctx, FIPI_ERR_OUT_OF_RANGE, "particle out of sorting range (cluster.cpp:144-163)");
    }
    return FIPI_OK;
}

extern "C" {

static fipi_status set_phase_impl(fipi_ctx* ctx, const double* c, bool dev) {
    if (!ctx || !c) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    graphs_reset(ctx);
    fipi_status st = fields_set_phase(ctx, c, dev);
    if (st != FIPI_OK) return st;
    ctx->t = 0;
    // device step counter and ramp(t + 1, 0.2 t_end) for t = 0
    const int t0 = 0;
    const double thr = 0.2 * ctx->P.t_end;
    const double rmp = (1.0 < thr) ? 1.0 / thr : 1.0;
    FIPI_CUDA(ctx, h2d(ctx, ctx->d_t, &t0, sizeof(int)));
    FIPI_CUDA(ctx, h2d(ctx, ctx->d_rmp, &rmp, sizeof(double)));
    ctx->have_phase = true;
    return check_status(ctx);
}

fipi_status fipi_set_phase(fipi_ctx* ctx, const double* c) { return set_phase_impl(ctx, c, false); }
fipi_status fipi_set_phase_device(fipi_ctx* ctx, const double* d_c) { return set_phase_impl(ctx, d_c, true); }

static fipi_status set_velocity_impl(fipi_ctx* ctx, const double* u, bool dev) {
    if (!ctx || !u) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = fields_set_velocity(ctx, u, dev);
    if (st != FIPI_OK) return st;
    return check_status(ctx);
}
fipi_status fipi_set_velocity(fipi_ctx* ctx, const double* u) { return set_velocity_impl(ctx, u, false); }
fipi_status fipi_set_velocity_device(fipi_ctx* ctx, const double* d_u) { return set_velocity_impl(ctx, d_u, true); }

}  // extern "C"

fipi_status fipi::upload_soa(fipi_ctx* ctx, const double* h, double* d, int n) {
    std::vector<double> s((size_t)3 * n);
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) s[(size_t)a * n + i] = h[3 * i + a];
    FIPI_CUDA(ctx, cudaMemcpyAsync(d, s.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return FIPI_OK;
}

fipi_status fipi::download_soa(fipi_ctx* ctx, const double* d, double* h, int n) {
    std::vector<double> s((size_t)3 * n);
    FIPI_CUDA(ctx, cudaMemcpyAsync(s.data(), d, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) h[3 * i + a] = s[(size_t)a * n + i];
    return FIPI_OK;
}

extern "C" {

// Particle state in and out through the pinned staging buffer: the host
// side is plain copies into and out of it; the AoS (n x 3, the reference's
// particle[i].p) <-> SoA (3 x n) transposes run on the device and read or
// write the mapped staging buffer directly (no separate copy); a call
// synchronises at most once.
}  // extern "C"

namespace {
// The whole particle state from AoS sources (p, f_pp: n x 3; r, cos theta:
// n; NULL f_pp / r / cos theta: 0 / r_default / 0) into the SoA state
// arrays; p_old = p (cluster.cpp:88), f_pi = u_old = 0.
__global__ void k_state_in(const double* __restrict__ ap, const double* __restrict__ afpp,
                           const double* __restrict__ ar, const double* __restrict__ acth, double r_default, int n,
                           double* p, double* p_old, double* f_pp, double* r, double* cth, double* f_pi,
                           double* u_old) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < 3 * n; j += gridDim.x * blockDim.x) {
        const int i = j / 3, a = j - 3 * i;
        const size_t s = (size_t)a * n + i;
        const double x = ap[j];
        p[s] = x;
        p_old[s] = x;
        f_pp[s] = afpp ? afpp[j] : 0.0;
        f_pi[s] = 0.0;
        u_old[s] = 0.0;
        if (j < n) {
            r[j] = ar ? ar[j] : r_default;
            cth[j] = acth ? acth[j] : 0.0;
        }
    }
}
// SoA arrays into AoS destinations (NULL pairs are skipped).
__global__ void k_state_out(const double* __restrict__ a0, const double* __restrict__ a1,
                            const double* __restrict__ a2, int n, double* o0, double* o1, double* o2) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < 3 * n; j += gridDim.x * blockDim.x) {
        const int i = j / 3, a = j - 3 * i;
        const size_t s = (size_t)a * n + i;
        if (o0) o0[j] = a0[s];
        if (o1) o1[j] = a1[s];
        if (o2) o2[j] = a2[s];
    }
}
inline int state_blocks(int n) { return (3 * n + 255) / 256 < 1024 ? (3 * n + 255) / 256 : 1024; }
}  // namespace

extern "C" {

// The copies are enqueued on the context stream (nothing is waited for at
// the end: the next call that reads results synchronises); the caller's
// arrays are consumed before the call returns.
fipi_status fipi_set_particles(fipi_ctx* ctx, const double* p, const double* r, const double* cos_theta,
                               const double* f_pp) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    const int n = ctx->pb.n;
    if (n == 0) return FIPI_OK;
    if (!p) return set_error(ctx, FIPI_ERR_BAD_ARG, "p is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the staging buffer is free
    double* pin = ctx->pin;
    const size_t b3 = sizeof(double) * 3 * n, b1 = sizeof(double) * n;
    std::memcpy(pin, p, b3);
    if (f_pp) std::memcpy(pin + 3 * (size_t)n, f_pp, b3);
    double* pr = pin + 6 * (size_t)n;
    double* pc = pr + n;
    if (r) std::memcpy(pr, r, b1);
    else
        for (int i = 0; i < n; ++i) pr[i] = ctx->P.r_p;
    if (cos_theta) std::memcpy(pc, cos_theta, b1);
    else std::memset(pc, 0, b1);
    {  // one kernel reads the pinned staging buffer directly (mapped host memory)
        const double* st = ctx->pin_dev;
        LaunchScope ls(ctx, "particle state in", 0.0);
        k_state_in<<<state_blocks(n), 256, 0, ctx->stream>>>(
            st, f_pp ? st + 3 * (size_t)n : nullptr, st + 6 * (size_t)n, st + 7 * (size_t)n, ctx->P.r_p, n,
            ctx->pb.p, ctx->pb.p_old, ctx->pb.f_pp, ctx->pb.r, ctx->pb.cth, ctx->pb.f_pi, ctx->pb.u_old);
    }
    FIPI_CUDA(ctx, cudaGetLastError());
    return FIPI_OK;
}

fipi_status fipi_set_particles_device(fipi_ctx* ctx, const double* d_p, const double* d_r,
                                      const double* d_cos_theta, const double* d_f_pp) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    const int n = ctx->pb.n;
    if (n == 0) return FIPI_OK;
    if (!d_p) return set_error(ctx, FIPI_ERR_BAD_ARG, "p is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    {
        LaunchScope ls(ctx, "particle state in", 0.0);
        k_state_in<<<state_blocks(n), 256, 0, ctx->stream>>>(d_p, d_f_pp, d_r, d_cos_theta, ctx->P.r_p, n,
                                                                  ctx->pb.p, ctx->pb.p_old, ctx->pb.f_pp,
                                                                  ctx->pb.r, ctx->pb.cth, ctx->pb.f_pi,
                                                                  ctx->pb.u_old);
    }
    return check_status(ctx);  // the caller's arrays may be reused on return
}

fipi_status fipi_get_phase(fipi_ctx* ctx, double* c) {
    if (!ctx || !c) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = check_status(ctx);
    if (st != FIPI_OK) return st;
    return fields_get_phase(ctx, c);
}

fipi_status fipi_get_velocity(fipi_ctx* ctx, double* u) {
    if (!ctx || !u) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = check_status(ctx);
    if (st != FIPI_OK) return st;
    return fields_get_velocity(ctx, u);
}

fipi_status fipi_get_particles(fipi_ctx* ctx, double* p, double* f_pp, double* f_pi) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    const int n = ctx->pb.n;
    if (n == 0) return check_status(ctx);
    const size_t b3 = sizeof(double) * 3 * n;
    double* dst[3] = {p, f_pp, f_pi};
    const double* src[3] = {ctx->pb.p, ctx->pb.f_pp, ctx->pb.f_pi};
    if (p || f_pp || f_pi) {
        double* st = ctx->pin_dev;
        LaunchScope ls(ctx, "particle state out", 0.0);
        k_state_out<<<state_blocks(n), 256, 0, ctx->stream>>>(
            src[0], src[1], src[2], n, p ? st : nullptr, f_pp ? st + 3 * (size_t)n : nullptr,
            f_pi ? st + 6 * (size_t)n : nullptr);
    }
    fipi_status st = check_status(ctx);  // the one synchronisation of the call
    if (st != FIPI_OK) return st;
    for (int k = 0; k < 3; ++k)
        if (dst[k]) std::memcpy(dst[k], ctx->pin + 3 * (size_t)n * k, b3);
    return FIPI_OK;
}

fipi_status fipi_get_particles_device(fipi_ctx* ctx, double* d_p, double* d_f_pp, double* d_f_pi) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    const int n = ctx->pb.n;
    if (n > 0 && (d_p || d_f_pp || d_f_pi)) {
        LaunchScope ls(ctx, "particle state out", 0.0);
        k_state_out<<<state_blocks(n), 256, 0, ctx->stream>>>(ctx->pb.p, ctx->pb.f_pp, ctx->pb.f_pi, n, d_p,
                                                                   d_f_pp, d_f_pi);
    }
    return check_status(ctx);
}

fipi_status fipi_get_phase_device(fipi_ctx* ctx, double* d_c) {
    if (!ctx || !d_c) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = fields_get_phase(ctx, d_c, true);
    if (st != FIPI_OK) return st;
    return check_status(ctx);
}

fipi_status fipi_get_velocity_device(fipi_ctx* ctx, double* d_u) {
    if (!ctx || !d_u) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = fields_get_velocity(ctx, d_u, true);
    if (st != FIPI_OK) return st;
    return check_status(ctx);
}

fipi_status fipi_get_time(const fipi_ctx* ctx, int* t) {
    if (!ctx || !t) return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    *t = ctx->t;
    return FIPI_OK;
}

}  // extern "C"

void fipi::graphs_reset(fipi_ctx* ctx) {
    for (auto& g : ctx->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = fipi_ctx::StepGraph{};
    }
}


// One iteration of main.cpp:75-219, enqueued on the context stream.
void fipi::enqueue_step(fipi_ctx* ctx) {
    const int t = ctx->t;
    fields_step_ch(ctx, t);      // main.cpp:79-141
    particles_spread(ctx);       // main.cpp:169 (compute_f_r of the previous step's state)
    fields_step_stokes(ctx);     // main.cpp:146-181
    if (!particles_step(ctx))    // main.cpp:186-219
        step_tick(ctx);
    ctx->t = t + 1;
}

extern "C" {

// Steps with t >= 1 are replayed from a CUDA graph of one step.  The step
// swaps ping-pong buffers, so the buffer assignment alternates between two
// states; each state gets its own graph, keyed by the current c_hat buffer,
// together with the host-side assignment the step leaves behind.
static fipi_status graph_step(fipi_ctx* ctx, bool* done) {
    *done = false;
    void* key = ctx->fb.chat;
    fipi_ctx::StepGraph* g = nullptr;
    for (auto& x : ctx->graphs)
        if (x.exec && x.key == key) g = &x;
    if (!g) {
        for (auto& x : ctx->graphs)
            if (!x.exec) g = &x;
        if (!g) return FIPI_OK;
        const fipi::FieldBufs fb0 = ctx->fb;
        const fipi::ParticleBufs pb0 = ctx->pb;
        const int t0 = ctx->t;
        const long long l0 = ctx->kt.launches;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            enqueue_step(ctx);
            e = cudaStreamEndCapture(ctx->stream, &graph);
        }
        cudaGraphExec_t exec = nullptr;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        const fipi::FieldBufs fb1 = ctx->fb;
        const fipi::ParticleBufs pb1 = ctx->pb;
        const long long launches = ctx->kt.launches - l0;
        ctx->fb = fb0;  // the capture did not run anything
        ctx->pb = pb0;
        ctx->t = t0;
        ctx->kt.launches = l0;
        if (e != cudaSuccess) {  // fall back to direct launches for this context
            cudaGetLastError();
            ctx->use_graphs = false;
            return FIPI_OK;
        }
        g->exec = exec;
        g->key = key;
        g->fb_after = fb1;
        g->pb_after = pb1;
        g->launches = launches;
    }
    FIPI_CUDA(ctx, cudaGraphLaunch(g->exec, ctx->stream));
    ctx->fb = g->fb_after;
    ctx->pb = g->pb_after;
    ctx->t += 1;
    ctx->kt.launches += g->launches;
    *done = true;
    return FIPI_OK;
}

fipi_status fipi_step_async(fipi_ctx* ctx, int nsteps) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    if (nsteps < 0) return set_error(ctx, FIPI_ERR_BAD_ARG, "nsteps < 0");
    if (!ctx->have_phase) return set_error(ctx, FIPI_ERR_STATE, "fipi_set_phase must come before fipi_step");
    if (ctx->substep != 0)
        return set_error(ctx, FIPI_ERR_STATE, "an iteration begun with fipi_step_ch is not finished");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    for (int s = 0; s < nsteps; ++s) {
        const bool spread_ready = ctx->pb.sp_prev_valid || ctx->pb.n == 0 || !ctx->P.switch_particle;
        if (ctx->use_graphs && ctx->t > 0 && !ctx->kt.enabled && spread_ready) {
            bool done = false;
            fipi_status st = graph_step(ctx, &done);
            if (st != FIPI_OK) return st;
            if (done) continue;
        }
        enqueue_step(ctx);
    }
    FIPI_CUDA(ctx, cudaGetLastError());
    return FIPI_OK;
}

fipi_status fipi_sync(fipi_ctx* ctx) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return check_status(ctx);
}

fipi_status fipi_step(fipi_ctx* ctx, int nsteps) {
    fipi_status st = fipi_step_async(ctx, nsteps);
    if (st != FIPI_OK) return st;
    return check_status(ctx);
}

// The three parts of one iteration (direct launches), in the order of
// enqueue_step; fipi_step_particles ends the iteration.
fipi_status fipi_step_ch(fipi_ctx* ctx) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    if (!ctx->have_phase) return set_error(ctx, FIPI_ERR_STATE, "fipi_set_phase must come first");
    if (ctx->substep != 0) return set_error(ctx, FIPI_ERR_STATE, "fipi_step_ch must start an iteration");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fields_step_ch(ctx, ctx->t);  // main.cpp:79-141
    ctx->substep = 1;
    return check_status(ctx);
}

fipi_status fipi_step_stokes(fipi_ctx* ctx) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    if (ctx->substep != 1) return set_error(ctx, FIPI_ERR_STATE, "fipi_step_stokes must follow fipi_step_ch");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    particles_spread(ctx);      // main.cpp:169
    fields_step_stokes(ctx);    // main.cpp:146-181
    ctx->substep = 2;
    return check_status(ctx);
}

fipi_status fipi_step_particles(fipi_ctx* ctx) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    if (ctx->substep != 2) return set_error(ctx, FIPI_ERR_STATE, "fipi_step_particles must follow fipi_step_stokes");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!particles_step(ctx))   // main.cpp:186-219
        step_tick(ctx);
    ctx->t += 1;
    ctx->substep = 0;
    return check_status(ctx);
}

fipi_status fipi_stream(const fipi_ctx* ctx, void** stream) {
    if (!ctx || !stream) return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    *stream = (void*)ctx->stream;
    return FIPI_OK;
}

fipi_status fipi_mass(fipi_ctx* ctx, double* out) {
    if (!ctx || !out) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return fields_mass(ctx, out);
}

fipi_status fipi_free_energy(fipi_ctx* ctx, double* out) {
    if (!ctx || !out) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return fields_free_energy(ctx, out);
}

fipi_status fipi_packing_tau(fipi_ctx* ctx, double* out) {
    if (!ctx || !out) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return particles_packing_tau(ctx, out);
}

// ---------------------------------------------------------------- instrumentation
fipi_status fipi_set_kernel_timing(fipi_ctx* ctx, int enable) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    drain_timer(ctx);
    ctx->kt.stats.clear();
    ctx->kt.enabled = enable != 0;
    return FIPI_OK;
}

fipi_status fipi_kernel_stats(fipi_ctx* ctx, int i, char* name, int name_cap, long long* launches, double* total_ms,
                              double* bytes_per_launch) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    drain_timer(ctx);
    if (i < 0 || i >= (int)ctx->kt.stats.size()) return set_error(ctx, FIPI_ERR_BAD_ARG, "no such kernel index");
    const KernelStat& s = ctx->kt.stats[i];
    if (name && name_cap > 0) {
        std::strncpy(name, s.name.c_str(), (size_t)name_cap - 1);
        name[name_cap - 1] = 0;
    }
    if (launches) *launches = s.launches;
    if (total_ms) *total_ms = s.ms;
    if (bytes_per_launch) *bytes_per_launch = s.bytes;
    return FIPI_OK;
}

fipi_status fipi_kernel_stat_count(fipi_ctx* ctx, int* n) {
    if (!ctx || !n) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    *n = (int)ctx->kt.stats.size();
    return FIPI_OK;
}

fipi_status fipi_launch_count(const fipi_ctx* ctx, long long* n) {
    if (!ctx || !n) return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    *n = ctx->kt.launches;
    return FIPI_OK;
}

// ---------------------------------------------------------------- fine-grained
#define NEED(x) \
    if (!(x)) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument: " #x)

// ---------------------------------------------------------------- extensions
fipi_status fipi_set_fluid_coupling(fipi_ctx* ctx, int on) {
    NEED(ctx);
    if (ctx->substep != 0) return set_error(ctx, FIPI_ERR_STATE, "extensions change between iterations only");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->couple_u = on ? 1 : 0;
    graphs_reset(ctx);
    return particles_ext_alloc(ctx);
}

fipi_status fipi_set_brownian(fipi_ctx* ctx, double kt, uint64_t seed) {
    NEED(ctx);
    if (!(kt >= 0.0) || !std::isfinite(kt)) return set_error(ctx, FIPI_ERR_BAD_ARG, "kt must be finite and >= 0");
    if (ctx->substep != 0) return set_error(ctx, FIPI_ERR_STATE, "extensions change between iterations only");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->brown_kt = kt;
    ctx->noise_seed = seed;
    graphs_reset(ctx);
    return particles_ext_alloc(ctx);
}

fipi_status fipi_set_params(fipi_ctx* ctx, const fipi_params* P) {
    NEED(ctx);
    NEED(P);
    if (ctx->substep != 0) return set_error(ctx, FIPI_ERR_STATE, "parameters change between iterations only");
    const fipi_params& Q = ctx->P;
    // the grid, box, time step, particle geometry and switches the context's
    // buffers, wave-number tables and cell grid were built for stay fixed
    const bool same = P->nx == Q.nx && P->ny == Q.ny && P->nz == Q.nz && P->lx == Q.lx && P->ly == Q.ly &&
                      P->lz == Q.lz && P->dt == Q.dt && P->t_end == Q.t_end && P->pi == Q.pi &&
                      P->margin == Q.margin && P->r_p == Q.r_p && P->r_eq == Q.r_eq && P->r_c == Q.r_c &&
                      P->n_p == Q.n_p && P->switch_particle == Q.switch_particle && P->switch_ch == Q.switch_ch &&
                      P->switch_ns == Q.switch_ns;
    if (!same)
        return set_error(ctx, FIPI_ERR_BAD_PARAMS,
                         "only sigma, epsilon, lambda, mobility, mu, rho1, rho2, gravity, A and k_n can change "
                         "on a live context");
    fipi_status st = validate(P, ctx->prec);
    if (st != FIPI_OK) return st;
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->P = *P;
    graphs_reset(ctx);
    return FIPI_OK;
}

fipi_status fipi_set_mass_conserving(fipi_ctx* ctx, int on) {
    NEED(ctx);
    if (ctx->substep != 0) return set_error(ctx, FIPI_ERR_STATE, "the mode changes between iterations only");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->conserve_mass = on ? 1 : 0;
    graphs_reset(ctx);
    return FIPI_OK;
}

fipi_status fipi_set_debug(fipi_ctx* ctx, int what, long long value) {
    NEED(ctx);
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    switch (what) {
        case FIPI_DEBUG_FFT_FIRST_WAIT_POLLS:
            if (value < -1 || value > (1 << 22)) return set_error(ctx, FIPI_ERR_BAD_ARG, "polls must be -1 or in [0, 2^22]");
            ctx->debug_first_wait = (int)value;
            break;
        default:
            return set_error(ctx, FIPI_ERR_BAD_ARG, "unknown debug setting");
    }
    graphs_reset(ctx);
    return FIPI_OK;
}

fipi_status fipi_fft_r2c(fipi_ctx* ctx, const double* in, double* out) {
    NEED(ctx);
    NEED(in);
    NEED(out);
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    const fipi_status st = fields_fft_r2c(ctx, in, out);
    return st != FIPI_OK ? st : check_status(ctx);  // the transforms' device error word (bounded copy waits)
}

fipi_status fipi_fft_c2r(fipi_ctx* ctx, const double* in, double* out) {
    NEED(ctx);
    NEED(in);
    NEED(out);
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    const fipi_status st = fields_fft_c2r(ctx, in, out);
    return st != FIPI_OK ? st : check_status(ctx);  // the transforms' device error word (bounded copy waits)
}

fipi_status fipi_grad(fipi_ctx* ctx, const double* c, double* g) {
    NEED(ctx);
    NEED(c);
    NEED(g);
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    const fipi_status st = fields_grad(ctx, c, g);
    return st != FIPI_OK ? st : check_status(ctx);  // the transforms' device error word (bounded copy waits)
}

fipi_status fipi_cells_build(fipi_ctx* ctx, const double* p, int* keys, int* sorted_ids, int* cell_offsets) {
    NEED(ctx);
    NEED(p);
    if (ctx->pb.n == 0) return FIPI_OK;
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return particles_cells_build(ctx, p, keys, sorted_ids, cell_offsets);
}

fipi_status fipi_f_pp(fipi_ctx* ctx, const double* p, int t, const double* f_pi, double* f_pp, double* tau) {
    NEED(ctx);
    NEED(p);
    if (ctx->pb.n == 0) {
        if (tau) *tau = 0.0;
        return FIPI_OK;
    }
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return particles_f_pp(ctx, p, t, f_pi, f_pp, tau);
}

fipi_status fipi_pairs(fipi_ctx* ctx, const double* p, int* pairs, int max_pairs, int* n_pairs) {
    NEED(ctx);
    NEED(p);
    NEED(n_pairs);
    *n_pairs = 0;
    if (ctx->pb.n == 0) return FIPI_OK;
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return particles_pairs(ctx, p, pairs, max_pairs, n_pairs);
}

fipi_status fipi_interpolate(fipi_ctx* ctx, const double* fields, int nfields, const double* p, double* out) {
    NEED(ctx);
    NEED(fields);
    NEED(p);
    NEED(out);
    if (nfields < 1 || nfields > 16) return set_error(ctx, FIPI_ERR_BAD_ARG, "nfields must be in [1, 16]");
    if (ctx->pb.n == 0) return FIPI_OK;
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return particles_interpolate(ctx, fields, nfields, p, out);
}

fipi_status fipi_f_pi(fipi_ctx* ctx, const double* c_loc, const double* dcdx, const double* r,
                      const double* cos_theta, double* f_pi) {
    NEED(ctx);
    NEED(c_loc);
    NEED(dcdx);
    NEED(f_pi);
    if (ctx->pb.n == 0) return FIPI_OK;
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return particles_f_pi(ctx, c_loc, dcdx, r, cos_theta, f_pi);
}

fipi_status fipi_advect(fipi_ctx* ctx, int stage, const double* f_pi, const double* f_pp, const double* r, double* p,
                        double* p_old, double* u_old) {
    NEED(ctx);
    NEED(f_pi);
    NEED(f_pp);
    NEED(p);
    NEED(p_old);
    NEED(u_old);
    if (stage != 1 && stage != 2) return set_error(ctx, FIPI_ERR_BAD_ARG, "stage must be 1 or 2");
    if (ctx->pb.n == 0) return FIPI_OK;
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return particles_advect(ctx, stage, f_pi, f_pp, r, p, p_old, u_old);
}

fipi_status fipi_interpolate2(fipi_ctx* ctx, const double* fields, int nfields, const double* p, double* out) {
    if (!ctx || !fields || !out || nfields < 1 || (!p && ctx->pb.n > 0))
        return set_error(ctx, FIPI_ERR_BAD_ARG, "bad argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    if (ctx->pb.n == 0) return FIPI_OK;
    return particles_interpolate2(ctx, fields, nfields, p, out);
}

fipi_status fipi_div(fipi_ctx* ctx, const double* v, double* out) {
    if (!ctx || !v || !out) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    const fipi_status st = fields_div(ctx, v, out);
    return st != FIPI_OK ? st : check_status(ctx);  // the transforms' device error word (bounded copy waits)
}

fipi_status fipi_wrap(fipi_ctx* ctx, double* p) {
    if (!ctx || (!p && ctx->pb.n > 0)) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return particles_wrap(ctx, p);
}

fipi_status fipi_spread(fipi_ctx* ctx, const double* p, const double* f_pp, double* out) {
    NEED(ctx);
    NEED(p);
    NEED(f_pp);
    NEED(out);
    if (ctx->pb.n == 0) {
        std::memset(out, 0, sizeof(double) * 3 * (size_t)ctx->g.V);
        return FIPI_OK;
    }
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return particles_spread_host(ctx, p, f_pp, out);
}

// ---------------------------------------------------------------- seeded inputs
// splitmix64 (Steele, Lea, Flood 2014) -> 53-bit uniforms in [0, 1).
static inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline double uniform01(uint64_t& s) { return (double)(splitmix64(s) >> 11) * 0x1.0p-53; }

fipi_status fipi_seed_phase(const fipi_params* P, uint64_t seed, double mean, double amp, double* c) {
    if (!P || !c) return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    uint64_t s = seed * 0x2545F4914F6CDD1Dull + 1;
    const size_t V = (size_t)P->nx * P->ny * P->nz;
    for (size_t i = 0; i < V; ++i) c[i] = mean + amp * (2.0 * uniform01(s) - 1.0);
    return FIPI_OK;
}

fipi_status fipi_seed_particles(const fipi_params* P, uint64_t seed, double r_min, double r_max,
                                double theta_min_deg, double theta_max_deg, int allow_overlap, double* pos, double* r,
                                double* cos_theta) {
    if (!P || !pos) return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    const int n = P->n_p;
    if (n <= 0) return FIPI_OK;
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 7;
    const double L[3] = {P->lx, P->ly, P->lz};
    // hash grid of cell size >= 2 r_max for the periodic overlap test
    int gc[3];
    double gs[3];
    for (int a = 0; a < 3; ++a) {
        gc[a] = std::max(1, (int)std::floor(L[a] / (2.0 * r_max)));
        gs[a] = L[a] / gc[a];
    }
    const size_t ncell = (size_t)gc[0] * gc[1] * gc[2];
    std::vector<std::vector<int>> grid(ncell);
    std::vector<double> rr(n);
    for (int i = 0; i < n; ++i) rr[i] = r_min + (r_max - r_min) * uniform01(s);
    auto wrapd = [](double d, double l) {
        if (d > 0.5 * l) d -= l;
        else if (d < -0.5 * l) d += l;
        return d;
    };
    const long long max_tries = 200000;
    for (int i = 0; i < n; ++i) {
        double x[3];
        bool ok = false;
        for (long long tries = 0; tries < max_tries && !ok; ++tries) {
            for (int a = 0; a < 3; ++a) {
                x[a] = L[a] * uniform01(s);
                if (x[a] >= L[a]) x[a] = 0.0;
            }
            if (allow_overlap) {
                ok = true;
                break;
            }
            int ci[3];
            for (int a = 0; a < 3; ++a) ci[a] = std::min(gc[a] - 1, (int)(x[a] / gs[a]));
            ok = true;
            for (int dk = -1; dk <= 1 && ok; ++dk)
                for (int dj = -1; dj <= 1 && ok; ++dj)
                    for (int di = -1; di <= 1 && ok; ++di) {
                        const size_t c = (size_t)((ci[0] + di + gc[0]) % gc[0]) +
                                         (size_t)((ci[1] + dj + gc[1]) % gc[1]) * gc[0] +
                                         (size_t)((ci[2] + dk + gc[2]) % gc[2]) * gc[0] * gc[1];
                        for (int j : grid[c]) {
                            double d2 = 0.0;
                            for (int a = 0; a < 3; ++a) {
                                const double d = wrapd(x[a] - pos[3 * j + a], L[a]);
                                d2 += d * d;
                            }
                            const double rs = rr[i] + rr[j];
                            if (d2 < rs * rs) {
                                ok = false;
                                break;
                            }
                        }
                    }
        }
        if (!ok) return set_error(nullptr, FIPI_ERR_BAD_PARAMS, "random non-overlapping placement did not converge");
        for (int a = 0; a < 3; ++a) pos[3 * i + a] = x[a];
        int ci[3];
        for (int a = 0; a < 3; ++a) ci[a] = std::min(gc[a] - 1, (int)(x[a] / gs[a]));
        grid[(size_t)ci[0] + (size_t)ci[1] * gc[0] + (size_t)ci[2] * gc[0] * gc[1]].push_back(i);
    }
    if (r)
        for (int i = 0; i < n; ++i) r[i] = rr[i];
    if (cos_theta)
        for (int i = 0; i < n; ++i) {
            const double th = theta_min_deg + (theta_max_deg - theta_min_deg) * uniform01(s);
            cos_theta[i] = (th == 90.0) ? 0.0 : std::cos(th * 3.14159265358979323846 / 180.0);
        }
    return FIPI_OK;
}

}  // extern "C"
