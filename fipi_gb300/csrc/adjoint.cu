// Reverse mode of the FP64 step, device-resident checkpoints and the
// sqrt(N)-checkpointed trajectory gradient.  The reference has neither; the
// step being differentiated is main.cpp:75-219 (CH update, Stokes
// projection, two Heun particle stages) as the forward path computes it.
//
// Cotangents of the Eulerian state are kept as half spectra of the real
// cotangent fields (la = R2C(lambda)).  Every Fourier multiplier of the
// step (the SBDF2 / IMEX coefficients, lambda k^2, the Leray projection
// with its Nyquist average) is real, even and therefore self-adjoint; the
// spectral derivative i k_d (Nyquist index zeroed) has adjoint -i k_d.  One
// reversed step, after the step has been recomputed from its checkpoint
// with u^n and mu^{n+1} kept:
//
//   particles   stage 2, contact forces at p1, stage 1, contact forces at
//               p^n (particles.cu), interpolation cotangents -> part (4 fields)
//   Stokes      lamF = P R2C(la_u) (projection), C2R, pointwise:
//                 L_mu = lamF . grad c,  L_g = lamF mu + part_g,
//                 L_c  = f'(c) L_mu + g (rho1 - rho2)/2 lamF_z + part_c
//               then 5 forward transforms combined in the last Z pass:
//                 L = la_c + R2C(L_c) + lambda k^2 R2C(L_mu) - i k . R2C(L_g)
//   CH          (same Z pass) lam_f, lam_C and the new history cotangents
//               from the SBDF2 / IMEX coefficients; C2R of lam_f, lam_C,
//               pointwise la_u = grad c^n lam_C, and
//                 la_c += R2C(f'(c^n) lam_f) - i k . R2C(u^n lam_C)
//   spreading   la_f_pp = I(p^n) lamF / dV, la_p += (f_pp / dV) grad I(p^n) lamF
//
// 17 transforms per reversed step plus the 13 of the recomputed step.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.hpp"
#include "passes.cuh"

namespace fipi {

// ------------------------------------------------------------ X-pass ops

// Stokes part reversed (see the file comment); in: lamF spectra (3),
// out: R2C of [L_c, L_mu, L_g0, L_g1, L_g2]; lamF is also stored real.
template <typename T> struct OpAdjStokes {
    using C = cplx<T>;
    C* S[5];
    T* lamF[3];
    const T* g[3];   // grad c^{n+1}
    const T* mu;     // mu^{n+1}
    const T* c;      // c^{n+1}
    const T* part;   // 4 x V particle cotangents on c, grad c (NULL: none)
    size_t V;
    T lam_eps;       // lambda / eps^2
    T bz;            // gravity (rho1 - rho2) / 2
    int nx, ny;
    __device__ const C* in(int f) const { return S[f]; }
    __device__ C* out(int f) const { return S[f]; }
    // acc: <L_mu, mu> (mu = lambda (k^2 c_hat)^ + f is linear in lambda: d mu / d lambda = mu / lambda)
    template <class A> __device__ void point(int z, int y, int n, C* v, A& acc) const {
        const size_t row = ((size_t)z * ny + y) * nx;
        const C lf[3] = {v[0], v[1], v[2]};
        C gd[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            reinterpret_cast<C*>(lamF[d] + row)[n] = lf[d];
            gd[d] = reinterpret_cast<const C*>(g[d] + row)[n];
        }
        const C m = reinterpret_cast<const C*>(mu + row)[n];
        const C cc = reinterpret_cast<const C*>(c + row)[n];
        const T lmx = lf[0].x * gd[0].x + lf[1].x * gd[1].x + lf[2].x * gd[2].x;
        const T lmy = lf[0].y * gd[0].y + lf[1].y * gd[1].y + lf[2].y * gd[2].y;
        acc += lmx * m.x + lmy * m.y;
        T lcx = lam_eps * (T(3) * cc.x * cc.x - T(1)) * lmx + bz * lf[2].x;
        T lcy = lam_eps * (T(3) * cc.y * cc.y - T(1)) * lmy + bz * lf[2].y;
        C lg[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) lg[d] = mkc<C>(lf[d].x * m.x, lf[d].y * m.y);
        if (part) {
            const C p0 = reinterpret_cast<const C*>(part + row)[n];
            lcx += p0.x;
            lcy += p0.y;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const C pd = reinterpret_cast<const C*>(part + (1 + d) * V + row)[n];
                lg[d].x += pd.x;
                lg[d].y += pd.y;
            }
        }
        v[0] = mkc<C>(lcx, lcy);
        v[1] = mkc<C>(lmx, lmy);
        v[2] = lg[0];
        v[3] = lg[1];
        v[4] = lg[2];
    }
};

// CH part reversed, real space: in lam_f, lam_C; la_u = grad c^n lam_C;
// out: R2C of [f'(c^n) lam_f, u^n_d lam_C].
template <typename T> struct OpAdjCH {
    using C = cplx<T>;
    C* S[4];
    const T* c0;
    const T* g0[3];
    const T* u[3];
    T* la_u[3];
    T lam_eps;
    int nx, ny;
    __device__ const C* in(int f) const { return S[f]; }
    __device__ C* out(int f) const { return S[f]; }
    // acc: <lam_f, c^3 - c> (f^n = (lambda/eps^2)(c^3 - c): d f / d lambda = (c^3 - c)/eps^2)
    template <class A> __device__ void point(int z, int y, int n, C* v, A& acc) const {
        const size_t row = ((size_t)z * ny + y) * nx;
        const C lf = v[0], lC = v[1];
        const C cc = reinterpret_cast<const C*>(c0 + row)[n];
        acc += lf.x * (cc.x * cc.x * cc.x - cc.x) + lf.y * (cc.y * cc.y * cc.y - cc.y);
        v[0] = mkc<C>(lam_eps * (T(3) * cc.x * cc.x - T(1)) * lf.x, lam_eps * (T(3) * cc.y * cc.y - T(1)) * lf.y);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const C gd = reinterpret_cast<const C*>(g0[d] + row)[n];
            const C ud = reinterpret_cast<const C*>(u[d] + row)[n];
            reinterpret_cast<C*>(la_u[d] + row)[n] = mkc<C>(gd.x * lC.x, gd.y * lC.y);
            v[1 + d] = mkc<C>(ud.x * lC.x, ud.y * lC.y);
        }
    }
};

// -i k_d X with the Nyquist index of d zeroed (adjoint of field::grad).
template <typename C, typename T> __device__ __forceinline__ void sub_ik(C& acc, T k, bool nyq, C X) {
    if (!nyq) {
        acc.x += k * X.y;
        acc.y -= k * X.x;
    }
}

// ------------------------------------------------------------ Z-pass ops
// Last forward Z pass of the Stokes part: forms L, the cotangent of
// c_hat^{n+1}, and reverses the CH update (main.cpp:95-138).  Writes
// lam_f (S[0]) and lam_C (S[1]) and the cotangents of c^n (partial) and of
// the start state's histories.
template <typename T> struct ZOpAdjC {
    using C = cplx<T>;
    C* S[5];
    C* la_c;
    C* la_co;
    C* la_fo;
    C* la_Co;
    KTabs<T> kt;
    StepConsts<T> k;
    int first;
    int conserve;  // mass-conserving mode: the forward step took C^n(0) = 0
    __device__ const C* src(int f) const { return S[f]; }
    __device__ void load(int, int, int, size_t gi, C* v) const {
#pragma unroll
        for (int f = 0; f < 5; ++f) v[f] = S[f][gi];
    }
    __device__ void store(int ix, int iy, int iz, size_t gi, const C* v) const {
        const T kx = kt.kx[ix], ky = kt.ky[iy], kz = kt.kz[iz];
        const T k2 = kt.k2(ix, iy, iz);
        const T k4 = k2 * k2;
        C L = la_c[gi];
        L.x += v[0].x + k.lam * k2 * v[1].x;
        L.y += v[0].y + k.lam * k2 * v[1].y;
        sub_ik(L, kx, ix == k.m, v[2]);
        sub_ik(L, ky, iy == k.ny2, v[3]);
        sub_ik(L, kz, iz == k.nz2, v[4]);
        const C co = la_co[gi], fo = la_fo[gi], Co = la_Co[gi];
        C lf, lC, lc;
        if (first) {
            const T den = k4 * k.s2 + T(1);
            const T af = k2 * k.s1 / den, aC = k.dt / den, ac = T(1) / den;
            lf = mkc<C>(fo.x - af * L.x, fo.y - af * L.y);
            lC = mkc<C>(Co.x - aC * L.x, Co.y - aC * L.y);
            lc = mkc<C>(co.x + ac * L.x, co.y + ac * L.y);
            la_co[gi] = mkc<C>(T(0), T(0));
            la_fo[gi] = mkc<C>(T(0), T(0));
            la_Co[gi] = mkc<C>(T(0), T(0));
        } else {
            const T den = k4 * k.s3 + T(3);
            const T a4 = k2 * k.s4 / den, a2 = k2 * k.s2m / den;
            const T c4 = k.s4c / den, c2 = k.s2c / den;
            lf = mkc<C>(fo.x - a4 * L.x, fo.y - a4 * L.y);
            lC = mkc<C>(Co.x - c4 * L.x, Co.y - c4 * L.y);
            lc = mkc<C>(co.x + T(4) / den * L.x, co.y + T(4) / den * L.y);
            la_co[gi] = mkc<C>(-L.x / den, -L.y / den);
            la_fo[gi] = mkc<C>(a2 * L.x, a2 * L.y);
            la_Co[gi] = mkc<C>(c2 * L.x, c2 * L.y);
        }
        if (conserve && gi == 0) lC = mkc<C>(T(0), T(0));
        la_c[gi] = lc;
        S[0][gi] = lf;
        S[1][gi] = lC;
        S[2][gi] = L;  // the cotangent of c_hat^{n+1}, for the parameter cotangents (read before S[2] is reused)
    }
};

// Cotangents of the mobility and of lambda through the CH update
// (main.cpp:95-138), c_hat^{n+1} = N / D:
//   SBDF2: N = 4 c^n - c^{n-1} - 4 dt M k^2 f^n + 2 dt M k^2 f^{n-1} - ...,
//          D = 3 + 2 dt M lambda k^4
//          dc/dM = (-4 dt k^2 f^n + 2 dt k^2 f^{n-1} - 2 dt lambda k^4 c^{n+1}) / D
//          dc/dlambda = -2 dt M k^4 c^{n+1} / D
//   IMEX (t = 0): N = c^0 - dt M k^2 f^0 - dt C^0, D = 1 + dt M lambda k^4
//          dc/dM = (-dt k^2 f^0 - dt lambda k^4 c^1) / D,  dc/dlambda = -dt M k^4 c^1 / D
// With L = R2C of the real cotangent of c^{n+1}, <lambda_c, dc> = (1/V) sum
// over the full spectrum of Re(conj(L) dc_hat), i.e. over the half spectrum
// with weight 2 off the kx = 0 and kx = nx/2 planes.  Per-block sums of the
// two inner products go to part[0][blk] and part[1][blk].
__global__ void k_adj_param_ch(const cplx<double>* __restrict__ L, const cplx<double>* __restrict__ c1,
                               const cplx<double>* __restrict__ fn, const cplx<double>* __restrict__ fo,
                               KTabs<double> kt, StepConsts<double> k, double M, int first, int ny, int h,
                               size_t SH, double* part) {
    double sM = 0.0, sL = 0.0;
    for (size_t gi = (size_t)blockIdx.x * blockDim.x + threadIdx.x; gi < SH; gi += (size_t)gridDim.x * blockDim.x) {
        const int iy = (int)(gi % ny);
        const size_t q = gi / ny;
        const int ix = (int)(q % h), iz = (int)(q / h);
        const double w = (ix == 0 || ix == k.m) ? 1.0 : 2.0;
        const double k2 = kt.k2(ix, iy, iz), k4 = k2 * k2;
        const cplx<double> l = L[gi], c = c1[gi], f = fn[gi];
        double dMx, dMy, dLx, dLy;
        if (first) {
            const double den = 1.0 + k.s2 * k4;
            dMx = (-k.dt * k2 * f.x - k.dt * k.lam * k4 * c.x) / den;
            dMy = (-k.dt * k2 * f.y - k.dt * k.lam * k4 * c.y) / den;
            dLx = -k.dt * M * k4 * c.x / den;
            dLy = -k.dt * M * k4 * c.y / den;
        } else {
            const cplx<double> g = fo[gi];
            const double den = 3.0 + k.s3 * k4;
            dMx = (k2 * (-4.0 * k.dt * f.x + 2.0 * k.dt * g.x) - 2.0 * k.dt * k.lam * k4 * c.x) / den;
            dMy = (k2 * (-4.0 * k.dt * f.y + 2.0 * k.dt * g.y) - 2.0 * k.dt * k.lam * k4 * c.y) / den;
            dLx = -2.0 * k.dt * M * k4 * c.x / den;
            dLy = -2.0 * k.dt * M * k4 * c.y / den;
        }
        sM += w * (l.x * dMx + l.y * dMy);
        sL += w * (l.x * dLx + l.y * dLy);
    }
    sM = block_sum(sM);
    sL = block_sum(sL);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = sM;
        part[gridDim.x + blockIdx.x] = sL;
    }
}

__global__ void k_param_acc(const double* __restrict__ part, int np, double scale, double* dst) {
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
    s = block_sum(s);
    if (threadIdx.x == 0) *dst += scale * s;
}

// la_c += X0 - i k . (X1, X2, X3)
template <typename T> struct ZOpAdjAcc {
    using C = cplx<T>;
    const C* S[4];
    C* la_c;
    KTabs<T> kt;
    int m, ny2, nz2;
    __device__ const C* src(int f) const { return S[f]; }
    __device__ void load(int, int, int, size_t gi, C* v) const {
#pragma unroll
        for (int f = 0; f < 4; ++f) v[f] = S[f][gi];
    }
    __device__ void store(int ix, int iy, int iz, size_t gi, const C* v) const {
        C L = la_c[gi];
        L.x += v[0].x;
        L.y += v[0].y;
        sub_ik(L, kt.kx[ix], ix == m, v[1]);
        sub_ik(L, kt.ky[iy], iy == ny2, v[2]);
        sub_ik(L, kt.kz[iz], iz == nz2, v[3]);
        la_c[gi] = L;
    }
};

// ------------------------------------------------------------ helpers
namespace {

using D = double;
using CD = cplx<double>;

constexpr int kParamBlocks = 304;  // blocks of the spectral parameter reduction

// Blocks of an FP64 X pass (one partial sum each when it reduces).
int x_blocks(const Geom& g) { return (g.ny / x_rows_of(sizeof(double), g.m)) * g.nz; }

CD* sp(void* p) { return (CD*)p; }

bool particles_on(const fipi_ctx* ctx) { return ctx->P.switch_particle && ctx->pb.n > 0; }

// R2C of a real device field into a spectral array (via AS[0]).
void r2c_into(fipi_ctx* ctx, const D* src, CD* dst) {
    const Geom& g = ctx->g;
    AdjBufs& a = ctx->ad;
    OpR2CN<D, 1> op{{src}, {sp(a.AS[0])}, g.nx, g.ny};
    launch_x<D, 0, 1, false>(ctx, "adjoint: X forward", 1, NoAcc<OpR2CN<D, 1>>{op});
    void* s1[1] = {a.AS[0]};
    launch_y<D>(ctx, 1, s1, s1, -1);
    ZOpStore<D, 1> zs{{sp(a.AS[0])}, {dst}, 0};
    launch_z<D, 1, -1>(ctx, "adjoint: Z forward", 2, zs);
}

// C2R of a spectral array into a real device field (via AS[0]).
void c2r_into(fipi_ctx* ctx, const CD* src, D* dst) {
    const Geom& g = ctx->g;
    AdjBufs& a = ctx->ad;
    ZOpStore<D, 1> zs{{src}, {sp(a.AS[0])}, 0};
    launch_z<D, 1, +1>(ctx, "adjoint: Z inverse", 2, zs);
    void* s1[1] = {a.AS[0]};
    launch_y<D>(ctx, 1, s1, s1, +1);
    OpC2RStore<D, 1> op{{sp(a.AS[0])}, {dst}, g.nx, g.ny};
    launch_x<D, 1, 0, false>(ctx, "adjoint: X inverse", 1, NoAcc<OpC2RStore<D, 1>>{op});
}

fipi_status adjoint_alloc(fipi_ctx* ctx) {
    AdjBufs& a = ctx->ad;
    if (a.la_c) return FIPI_OK;
    const Geom& g = ctx->g;
    const size_t V = (size_t)g.V, SH = (size_t)g.SH;
    auto A = [&](void** ptr, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(ptr, bytes);
        if (e == cudaSuccess) {
            ctx->device_bytes += bytes;
            e = cudaMemsetAsync(*ptr, 0, bytes, ctx->stream);
        }
        return e;
    };
    void** specs[] = {&a.la_c, &a.la_co, &a.la_fo, &a.la_Co, &a.AS[0], &a.AS[1], &a.AS[2], &a.AS[3], &a.AS[4],
                      &a.tfo};
    for (void** p : specs) FIPI_CUDA(ctx, A(p, sizeof(CD) * SH));
    // partial sums: one per X-pass block, or two per block of the spectral reduction
    a.pg_nparts = std::max(x_blocks(g), 2 * kParamBlocks);
    FIPI_CUDA(ctx, A((void**)&a.pg, sizeof(D) * kParamGrads));
    FIPI_CUDA(ctx, A((void**)&a.pg_part, sizeof(D) * (size_t)a.pg_nparts));
    FIPI_CUDA(ctx, A((void**)&a.la_u, sizeof(D) * 3 * V));
    FIPI_CUDA(ctx, A((void**)&a.lamF, sizeof(D) * 3 * V));
    FIPI_CUDA(ctx, A((void**)&a.part, sizeof(D) * 4 * V));
    FIPI_CUDA(ctx, A((void**)&a.tc0, sizeof(D) * V));
    FIPI_CUDA(ctx, A((void**)&a.tg0, sizeof(D) * 3 * V));
    FIPI_CUDA(ctx, A((void**)&a.tu, sizeof(D) * 3 * V));
    FIPI_CUDA(ctx, A((void**)&a.tmu, sizeof(D) * V));
    if (ctx->pb.n > 0) {
        fipi_status st = particles_adjoint_alloc(ctx);
        if (st != FIPI_OK) return st;
    }
    return FIPI_OK;
}

// ------------------------------------------------------------ checkpoints
// Payload regions, each 256-byte aligned.
struct CkLayout {
    size_t c, g, spec, upre, k0, p, fpp, r, cth, bytes;
};

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

CkLayout ck_layout(const fipi_ctx* ctx) {
    const size_t ts = ctx->prec == FIPI_MIXED ? sizeof(float) : sizeof(double);
    const size_t V = (size_t)ctx->g.V, SH = (size_t)ctx->g.SH;
    const size_t n = (size_t)ctx->pb.n;
    CkLayout L{};
    size_t o = 0;
    L.c = o;
    o = up256(o + ts * V);
    L.g = o;
    o = up256(o + 3 * ts * V);
    L.spec = o;  // chat, chat_old, fhat, fhat_old, Chat_old
    o = up256(o + 5 * 2 * ts * SH);
    L.upre = o;
    o = up256(o + 3 * 2 * ts * SH);
    L.k0 = o;
    o = up256(o + 6 * sizeof(double));
    L.p = o;
    o = up256(o + 3 * n * sizeof(double));
    L.fpp = o;
    o = up256(o + 3 * n * sizeof(double));
    L.r = o;
    o = up256(o + n * sizeof(double));
    L.cth = o;
    o = up256(o + n * sizeof(double));
    L.bytes = o;
    return L;
}

struct CkCopy {
    void* slot;
    void* ctxbuf;
    size_t bytes;
};

std::vector<CkCopy> ck_regions(fipi_ctx* ctx, unsigned char* base) {
    const CkLayout L = ck_layout(ctx);
    const size_t ts = ctx->prec == FIPI_MIXED ? sizeof(float) : sizeof(double);
    const size_t V = (size_t)ctx->g.V, SH = (size_t)ctx->g.SH;
    const size_t n = (size_t)ctx->pb.n;
    FieldBufs& b = ctx->fb;
    std::vector<CkCopy> r;
    r.push_back({base + L.c, b.c, ts * V});
    for (int d = 0; d < 3; ++d) r.push_back({base + L.g + d * ts * V, b.g[d], ts * V});
    void* specs[5] = {b.chat, b.chat_old, b.fhat, b.fhat_old, b.Chat_old};
    for (int i = 0; i < 5; ++i) r.push_back({base + L.spec + i * 2 * ts * SH, specs[i], 2 * ts * SH});
    for (int d = 0; d < 3; ++d) r.push_back({base + L.upre + d * 2 * ts * SH, b.upre[d], 2 * ts * SH});
    r.push_back({base + L.k0, ctx->k0, 6 * sizeof(double)});
    if (n > 0) {
        r.push_back({base + L.p, ctx->pb.p, 3 * n * sizeof(double)});
        r.push_back({base + L.fpp, ctx->pb.f_pp, 3 * n * sizeof(double)});
        r.push_back({base + L.r, ctx->pb.r, n * sizeof(double)});
        r.push_back({base + L.cth, ctx->pb.cth, n * sizeof(double)});
    }
    return r;
}

fipi_status slot_ok(fipi_ctx* ctx, int slot) {
    if (slot < 0 || slot >= ctx->ck.slots)
        return set_error(ctx, FIPI_ERR_BAD_ARG, "checkpoint slot out of range (fipi_checkpoint_reserve)");
    return FIPI_OK;
}

fipi_status ck_reserve(fipi_ctx* ctx, int slots) {
    CheckpointStore& ck = ctx->ck;
    const size_t bytes = ck_layout(ctx).bytes;
    if (ck.base && ck.slots >= slots && ck.bytes == bytes) return FIPI_OK;
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ck.base) {
        cudaFree(ck.base);
        ctx->device_bytes -= ck.bytes * (size_t)ck.slots;
        ck.base = nullptr;
    }
    ck.slots = 0;
    ck.t.clear();
    if (slots <= 0) return FIPI_OK;
    cudaError_t e = cudaMalloc((void**)&ck.base, bytes * (size_t)slots);
    if (e != cudaSuccess) {
        ck.base = nullptr;
        return cuda_check(ctx, e, "cudaMalloc (checkpoint slots)");
    }
    ctx->device_bytes += bytes * (size_t)slots;
    ck.slots = slots;
    ck.bytes = bytes;
    ck.t.assign(slots, -1);
    return FIPI_OK;
}

fipi_status ck_save(fipi_ctx* ctx, int slot) {
    fipi_status st = slot_ok(ctx, slot);
    if (st != FIPI_OK) return st;
    unsigned char* base = ctx->ck.base + (size_t)slot * ctx->ck.bytes;
    for (const CkCopy& c : ck_regions(ctx, base))
        FIPI_CUDA(ctx, cudaMemcpyAsync(c.slot, c.ctxbuf, c.bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->ck.t[slot] = ctx->t;
    return FIPI_OK;
}

fipi_status ck_load(fipi_ctx* ctx, int slot) {
    fipi_status st = slot_ok(ctx, slot);
    if (st != FIPI_OK) return st;
    if (ctx->ck.t[slot] < 0) return set_error(ctx, FIPI_ERR_STATE, "checkpoint slot is empty");
    unsigned char* base = ctx->ck.base + (size_t)slot * ctx->ck.bytes;
    for (const CkCopy& c : ck_regions(ctx, base))
        FIPI_CUDA(ctx, cudaMemcpyAsync(c.ctxbuf, c.slot, c.bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->t = ctx->ck.t[slot];
    set_tick(ctx, ctx->t);
    ctx->pb.tau_valid = false;
    ctx->have_phase = true;
    return FIPI_OK;
}

struct CkHeader {
    char magic[8];
    int32_t version, prec, nx, ny, nz, n_p, t, pad;
    uint64_t payload;
    unsigned char rest[16];
};
static_assert(sizeof(CkHeader) == 64, "checkpoint header is 64 bytes");

// ------------------------------------------------------------ adjoint passes
void adjoint_fields(fipi_ctx* ctx, bool first) {
    const Geom& g = ctx->g;
    AdjBufs& a = ctx->ad;
    const size_t V = (size_t)g.V;
    const StepConsts<D> k = make_consts<D>(ctx);
    const KTabs<D> kt = F<D>::ktabs(ctx);
    CD* S[5] = {sp(a.AS[0]), sp(a.AS[1]), sp(a.AS[2]), sp(a.AS[3]), sp(a.AS[4])};
    void* Sv[5] = {a.AS[0], a.AS[1], a.AS[2], a.AS[3], a.AS[4]};
    // lamF_hat = P R2C(la_u)
    OpR2CN<D, 3> o1{{a.la_u, a.la_u + V, a.la_u + 2 * V}, {S[0], S[1], S[2]}, g.nx, g.ny};
    launch_x<D, 0, 3, false>(ctx, "adjoint: X forward u", 3, NoAcc<OpR2CN<D, 3>>{o1});
    launch_y<D>(ctx, 3, Sv, Sv, -1);
    ZOpProj<D> zp{{S[0], S[1], S[2]}, {S[0], S[1], S[2]}, kt, k.mu, g.m, g.ny / 2, g.nz / 2};
    launch_z<D, 3, -1>(ctx, "adjoint: Z forward + projection", 6, zp);
    // lamF real, Stokes pointwise adjoint, 5 forward transforms
    ZOpStore<D, 3> zi{{S[0], S[1], S[2]}, {S[0], S[1], S[2]}, 0};
    launch_z<D, 3, +1>(ctx, "adjoint: Z inverse", 6, zi);
    launch_y<D>(ctx, 3, Sv, Sv, +1);
    const fipi_params& P = ctx->P;
    OpAdjStokes<D> os{{S[0], S[1], S[2], S[3], S[4]},
                      {a.lamF, a.lamF + V, a.lamF + 2 * V},
                      {(const D*)ctx->fb.g[0], (const D*)ctx->fb.g[1], (const D*)ctx->fb.g[2]},
                      a.tmu,
                      (const D*)ctx->fb.c,
                      particles_on(ctx) ? a.part : nullptr,
                      V,
                      k.lam_eps,
                      P.gravity * (P.rho1 - P.rho2) / 2.0,
                      g.nx,
                      g.ny};
    launch_x<D, 3, 5, true>(ctx, "adjoint: X Stokes", particles_on(ctx) ? 12 : 8, os, a.pg_part);
    // lambda through mu^{n+1}: <L_mu, mu> / lambda
    param_acc(ctx, a.pg_part, x_blocks(g), P.lambda != 0.0 ? 1.0 / P.lambda : 0.0, a.pg + kPgLambda);
    launch_y<D>(ctx, 5, Sv, Sv, -1);
    ZOpAdjC<D> zc{{S[0], S[1], S[2], S[3], S[4]}, sp(a.la_c), sp(a.la_co), sp(a.la_fo), sp(a.la_Co), kt, k,
                  first ? 1 : 0, ctx->conserve_mass};
    launch_z<D, 5, -1>(ctx, "adjoint: Z forward + CH", 13, zc);
    {
        // mobility and lambda through the CH update (c_hat^{n+1} = chat, f^n = fhat_old after the
        // recomputed step, f^{n-1} taped before it)
        LaunchScope ls(ctx, "adjoint: CH parameter sums", 4.0 * g.SH * sizeof(CD));
        k_adj_param_ch<<<kParamBlocks, 256, 0, ctx->stream>>>(S[2], sp(ctx->fb.chat), sp(ctx->fb.fhat_old),
                                                               sp(a.tfo), kt, k, P.mobility, first ? 1 : 0, g.ny,
                                                               g.h, (size_t)g.SH, a.pg_part);
    }
    const double invV = 1.0 / (double)g.V;
    param_acc(ctx, a.pg_part, kParamBlocks, invV, a.pg + kPgMobility);
    param_acc(ctx, a.pg_part + kParamBlocks, kParamBlocks, invV, a.pg + kPgLambda);
    if (particles_on(ctx)) particles_adjoint_spread(ctx);
    // lam_f, lam_C real; la_u; 4 forward transforms into la_c
    ZOpStore<D, 2> zi2{{S[0], S[1]}, {S[0], S[1]}, 0};
    launch_z<D, 2, +1>(ctx, "adjoint: Z inverse", 4, zi2);
    launch_y<D>(ctx, 2, Sv, Sv, +1);
    OpAdjCH<D> oc{{S[0], S[1], S[2], S[3]},
                  a.tc0,
                  {a.tg0, a.tg0 + V, a.tg0 + 2 * V},
                  {a.tu, a.tu + V, a.tu + 2 * V},
                  {a.la_u, a.la_u + V, a.la_u + 2 * V},
                  k.lam_eps,
                  g.nx,
                  g.ny};
    launch_x<D, 2, 4, true>(ctx, "adjoint: X CH", 10, oc, a.pg_part);
    // lambda through f^n = (lambda / eps^2)(c^3 - c): <lam_f, c^3 - c> / eps^2
    param_acc(ctx, a.pg_part, x_blocks(g), 1.0 / (P.epsilon * P.epsilon), a.pg + kPgLambda);
    launch_y<D>(ctx, 4, Sv, Sv, -1);
    ZOpAdjAcc<D> za{{S[0], S[1], S[2], S[3]}, sp(a.la_c), kt, g.m, g.ny / 2, g.nz / 2};
    launch_z<D, 4, -1>(ctx, "adjoint: Z forward + accumulate", 6, za);
}

fipi_status adjoint_step_impl(fipi_ctx* ctx, int slot) {
    AdjBufs& a = ctx->ad;
    const Geom& g = ctx->g;
    const size_t V = (size_t)g.V;
    fipi_status st = slot_ok(ctx, slot);
    if (st != FIPI_OK) return st;
    if (ctx->ck.t[slot] != a.t - 1)
        return set_error(ctx, FIPI_ERR_STATE, "the slot must hold the state one step before the cotangent's");
    st = ck_load(ctx, slot);
    if (st != FIPI_OK) return st;
    const int n = ctx->t;
    // the forward step's intermediates that the reverse pass reads
    FieldBufs& b = ctx->fb;
    FIPI_CUDA(ctx, cudaMemcpyAsync(a.tc0, b.c, sizeof(D) * V, cudaMemcpyDeviceToDevice, ctx->stream));
    if (n > 0)  // f_hat^{n-1}: the recomputed step overwrites it (the mobility cotangent reads it)
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.tfo, b.fhat_old, sizeof(CD) * (size_t)g.SH, cudaMemcpyDeviceToDevice,
                                       ctx->stream));
    for (int d = 0; d < 3; ++d)
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.tg0 + d * V, b.g[d], sizeof(D) * V, cudaMemcpyDeviceToDevice, ctx->stream));
    const bool parts = particles_on(ctx);
    if (parts) {
        const size_t b3 = sizeof(D) * 3 * (size_t)ctx->pb.n;
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.tp0, ctx->pb.p, b3, cudaMemcpyDeviceToDevice, ctx->stream));
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.tfpp0, ctx->pb.f_pp, b3, cudaMemcpyDeviceToDevice, ctx->stream));
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.rmp, ctx->d_rmp, sizeof(D), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    ctx->tape_u[0] = a.tu;
    ctx->tape_u[1] = a.tu + V;
    ctx->tape_u[2] = a.tu + 2 * V;
    ctx->tape_mu = a.tmu;
    enqueue_step(ctx);
    ctx->tape_u[0] = ctx->tape_u[1] = ctx->tape_u[2] = nullptr;
    ctx->tape_mu = nullptr;
    if (parts) {
        st = particles_adjoint(ctx);
        if (st != FIPI_OK) return st;
    }
    adjoint_fields(ctx, n == 0);
    FIPI_CUDA(ctx, cudaGetLastError());
    a.t = n;
    return check_status(ctx);
}

// Reverses step n without recomputing it: slot_n holds the state at the
// start of the step, slot_n1 the state after it, and tape the u^n and
// mu^{n+1} the step wrote when it ran (4V doubles) -- what the trajectory's
// segment sweep leaves.  Gives the same cotangents as adjoint_step_impl,
// which recomputes the step from slot_n to obtain the same inputs.
fipi_status adjoint_reverse_pair(fipi_ctx* ctx, int slot_n, int slot_n1, const double* tape) {
    AdjBufs& a = ctx->ad;
    const Geom& g = ctx->g;
    const size_t V = (size_t)g.V, SH = (size_t)g.SH;
    const int n = ctx->ck.t[slot_n];
    if (n != a.t - 1 || ctx->ck.t[slot_n1] != a.t)
        return set_error(ctx, FIPI_ERR_STATE, "the slots must hold the states before and after the reversed step");
    const CkLayout L = ck_layout(ctx);
    const unsigned char* sn = ctx->ck.base + (size_t)slot_n * ctx->ck.bytes;
    const bool parts = particles_on(ctx);
    // inputs of the reverse pass from the step's start state
    FIPI_CUDA(ctx, cudaMemcpyAsync(a.tc0, sn + L.c, sizeof(D) * V, cudaMemcpyDeviceToDevice, ctx->stream));
    FIPI_CUDA(ctx, cudaMemcpyAsync(a.tg0, sn + L.g, sizeof(D) * 3 * V, cudaMemcpyDeviceToDevice, ctx->stream));
    if (n > 0)  // f_hat^{n-1}: the start state's f_hat history (spectral region 3 of the slot)
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.tfo, sn + L.spec + 3 * 2 * sizeof(D) * SH, sizeof(CD) * SH,
                                       cudaMemcpyDeviceToDevice, ctx->stream));
    if (parts) {
        const size_t b3 = sizeof(D) * 3 * (size_t)ctx->pb.n;
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.tp0, sn + L.p, b3, cudaMemcpyDeviceToDevice, ctx->stream));
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.tfpp0, sn + L.fpp, b3, cudaMemcpyDeviceToDevice, ctx->stream));
        set_tick(ctx, n);  // ramp(n + 1, 0.2 t_end) of the reversed step
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.rmp, ctx->d_rmp, sizeof(D), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    FIPI_CUDA(ctx, cudaMemcpyAsync(a.tu, tape, sizeof(D) * 3 * V, cudaMemcpyDeviceToDevice, ctx->stream));
    FIPI_CUDA(ctx, cudaMemcpyAsync(a.tmu, tape + 3 * V, sizeof(D) * V, cudaMemcpyDeviceToDevice, ctx->stream));
    // the step's end state, as the recomputed step would have left it
    fipi_status st = ck_load(ctx, slot_n1);
    if (st != FIPI_OK) return st;
    if (parts) {
        st = particles_adjoint(ctx);
        if (st != FIPI_OK) return st;
    }
    adjoint_fields(ctx, n == 0);
    FIPI_CUDA(ctx, cudaGetLastError());
    a.t = n;
    return FIPI_OK;
}

fipi_status adjoint_seed_impl(fipi_ctx* ctx, const double* dc, const double* du, const double* dp,
                              const double* dfpp) {
    if (ctx->prec != FIPI_FP64)
        return set_error(ctx, FIPI_ERR_UNSUPPORTED, "the adjoint is built for FIPI_FP64 contexts");
    if (ctx->couple_u || ctx->brown_kt > 0.0)
        return set_error(ctx, FIPI_ERR_UNSUPPORTED, "the adjoint is built for the reference's particle model "
                                                    "(fluid coupling and Brownian force off)");
    if (!ctx->have_phase) return set_error(ctx, FIPI_ERR_STATE, "fipi_set_phase must come first");
    fipi_status st = adjoint_alloc(ctx);
    if (st != FIPI_OK) return st;
    AdjBufs& a = ctx->ad;
    const Geom& g = ctx->g;
    const size_t V = (size_t)g.V, SH = (size_t)g.SH;
    const int n = ctx->pb.n;
    if (dc) {
        FIPI_CUDA(ctx, cudaMemcpyAsync(a.lamF, dc, sizeof(D) * V, cudaMemcpyHostToDevice, ctx->stream));
        r2c_into(ctx, a.lamF, sp(a.la_c));
    } else {
        FIPI_CUDA(ctx, cudaMemsetAsync(a.la_c, 0, sizeof(CD) * SH, ctx->stream));
    }
    void* hist[3] = {a.la_co, a.la_fo, a.la_Co};
    for (void* h : hist) FIPI_CUDA(ctx, cudaMemsetAsync(h, 0, sizeof(CD) * SH, ctx->stream));
    FIPI_CUDA(ctx, cudaMemsetAsync(a.pg, 0, sizeof(D) * kParamGrads, ctx->stream));
    if (n > 0) FIPI_CUDA(ctx, cudaMemsetAsync(a.dct, 0, sizeof(D) * n, ctx->stream));
    if (du) FIPI_CUDA(ctx, cudaMemcpyAsync(a.la_u, du, sizeof(D) * 3 * V, cudaMemcpyHostToDevice, ctx->stream));
    else FIPI_CUDA(ctx, cudaMemsetAsync(a.la_u, 0, sizeof(D) * 3 * V, ctx->stream));
    if (n > 0) {
        if (dp) {
            st = upload_soa(ctx, dp, a.la_p, n);
            if (st != FIPI_OK) return st;
        } else {
            FIPI_CUDA(ctx, cudaMemsetAsync(a.la_p, 0, sizeof(D) * 3 * n, ctx->stream));
        }
        if (dfpp) {
            st = upload_soa(ctx, dfpp, a.la_fpp, n);
            if (st != FIPI_OK) return st;
        } else {
            FIPI_CUDA(ctx, cudaMemsetAsync(a.la_fpp, 0, sizeof(D) * 3 * n, ctx->stream));
        }
    }
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    a.t = ctx->t;
    a.ready = true;
    return check_status(ctx);
}

fipi_status adjoint_ready(fipi_ctx* ctx) {
    if (ctx->prec != FIPI_FP64)
        return set_error(ctx, FIPI_ERR_UNSUPPORTED, "the adjoint is built for FIPI_FP64 contexts");
    if (ctx->couple_u || ctx->brown_kt > 0.0)
        return set_error(ctx, FIPI_ERR_UNSUPPORTED, "the adjoint is built for the reference's particle model "
                                                    "(fluid coupling and Brownian force off)");
    if (!ctx->ad.ready) return set_error(ctx, FIPI_ERR_STATE, "fipi_adjoint_seed must come first");
    return FIPI_OK;
}

}  // namespace

void param_acc(fipi_ctx* ctx, const double* part, int np, double scale, double* dst) {
    LaunchScope ls(ctx, "adjoint: parameter sum", 0.0);
    k_param_acc<<<1, 256, 0, ctx->stream>>>(part, np, scale, dst);
}

void adjoint_free(fipi_ctx* ctx) {
    AdjBufs& a = ctx->ad;
    void* all[] = {a.la_c, a.la_co, a.la_fo, a.la_Co, a.AS[0], a.AS[1], a.AS[2], a.AS[3], a.AS[4],
                   a.la_u, a.lamF, a.part, a.tc0, a.tg0, a.tu, a.tmu, a.pg, a.pg_part, a.tfo, a.seg_tape};
    for (void* p : all)
        if (p) cudaFree(p);
    particles_adjoint_free(ctx);
    a = AdjBufs{};
    if (ctx->ck.base) cudaFree(ctx->ck.base);
    ctx->ck = CheckpointStore{};
}

}  // namespace fipi

using namespace fipi;

extern "C" {

fipi_status fipi_checkpoint_reserve(fipi_ctx* ctx, int slots) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    if (slots < 0) return set_error(ctx, FIPI_ERR_BAD_ARG, "slots < 0");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    return ck_reserve(ctx, slots);
}

fipi_status fipi_checkpoint_bytes(const fipi_ctx* ctx, size_t* bytes) {
    if (!ctx || !bytes) return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    *bytes = ck_layout(ctx).bytes;
    return FIPI_OK;
}

fipi_status fipi_checkpoint_save(fipi_ctx* ctx, int slot) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    if (!ctx->have_phase) return set_error(ctx, FIPI_ERR_STATE, "fipi_set_phase must come first");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = ck_save(ctx, slot);
    if (st != FIPI_OK) return st;
    return check_status(ctx);
}

fipi_status fipi_checkpoint_load(fipi_ctx* ctx, int slot) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = ck_load(ctx, slot);
    if (st != FIPI_OK) return st;
    return check_status(ctx);
}

fipi_status fipi_checkpoint_export(fipi_ctx* ctx, int slot, void* blob, size_t blob_bytes) {
    if (!ctx || !blob) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = slot_ok(ctx, slot);
    if (st != FIPI_OK) return st;
    if (ctx->ck.t[slot] < 0) return set_error(ctx, FIPI_ERR_STATE, "checkpoint slot is empty");
    const size_t pay = ctx->ck.bytes;
    if (blob_bytes < sizeof(CkHeader) + pay) return set_error(ctx, FIPI_ERR_BAD_ARG, "blob too small");
    CkHeader h{};
    std::memcpy(h.magic, "FIPICKP1", 8);
    h.version = 1;
    h.prec = (int32_t)ctx->prec;
    h.nx = ctx->P.nx;
    h.ny = ctx->P.ny;
    h.nz = ctx->P.nz;
    h.n_p = ctx->pb.n;
    h.t = ctx->ck.t[slot];
    h.payload = pay;
    std::memcpy(blob, &h, sizeof(h));
    FIPI_CUDA(ctx, d2h(ctx, (unsigned char*)blob + sizeof(h), ctx->ck.base + (size_t)slot * pay, pay));
    return FIPI_OK;
}

fipi_status fipi_checkpoint_import(fipi_ctx* ctx, int slot, const void* blob, size_t blob_bytes) {
    if (!ctx || !blob) return set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = slot_ok(ctx, slot);
    if (st != FIPI_OK) return st;
    if (blob_bytes < sizeof(CkHeader)) return set_error(ctx, FIPI_ERR_BAD_ARG, "blob too small");
    CkHeader h;
    std::memcpy(&h, blob, sizeof(h));
    const size_t pay = ctx->ck.bytes;
    if (std::memcmp(h.magic, "FIPICKP1", 8) != 0 || h.version != 1)
        return set_error(ctx, FIPI_ERR_BAD_ARG, "not a FIPI checkpoint");
    if (h.prec != (int32_t)ctx->prec || h.nx != ctx->P.nx || h.ny != ctx->P.ny || h.nz != ctx->P.nz ||
        h.n_p != ctx->pb.n || h.payload != pay || h.t < 0)
        return set_error(ctx, FIPI_ERR_BAD_ARG, "checkpoint does not match this context");
    if (blob_bytes < sizeof(CkHeader) + pay) return set_error(ctx, FIPI_ERR_BAD_ARG, "blob too small");
    FIPI_CUDA(ctx, h2d(ctx, ctx->ck.base + (size_t)slot * pay, (const unsigned char*)blob + sizeof(h), pay));
    ctx->ck.t[slot] = h.t;
    return FIPI_OK;
}

fipi_status fipi_adjoint_seed(fipi_ctx* ctx, const double* dc, const double* du, const double* dp,
                              const double* df_pp) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = check_status(ctx);
    if (st != FIPI_OK) return st;
    return adjoint_seed_impl(ctx, dc, du, dp, df_pp);
}

fipi_status fipi_adjoint_step(fipi_ctx* ctx, int slot) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = adjoint_ready(ctx);
    if (st != FIPI_OK) return st;
    return adjoint_step_impl(ctx, slot);
}

fipi_status fipi_adjoint_get(fipi_ctx* ctx, double* dc, double* du, double* dp, double* df_pp) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = adjoint_ready(ctx);
    if (st != FIPI_OK) return st;
    AdjBufs& a = ctx->ad;
    const size_t V = (size_t)ctx->g.V;
    const int n = ctx->pb.n;
    if (dc) {
        c2r_into(ctx, sp(a.la_c), a.lamF);
        FIPI_CUDA(ctx, d2h(ctx, dc, a.lamF, sizeof(D) * V));
    }
    if (du) FIPI_CUDA(ctx, d2h(ctx, du, a.la_u, sizeof(D) * 3 * V));
    if (n > 0 && dp) {
        st = download_soa(ctx, a.la_p, dp, n);
        if (st != FIPI_OK) return st;
    }
    if (n > 0 && df_pp) {
        st = download_soa(ctx, a.la_fpp, df_pp, n);
        if (st != FIPI_OK) return st;
    }
    return check_status(ctx);
}

fipi_status fipi_adjoint_get_params(fipi_ctx* ctx, fipi_param_grads* out, double* dcos_theta) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = adjoint_ready(ctx);
    if (st != FIPI_OK) return st;
    const fipi_params& P = ctx->P;
    AdjBufs& a = ctx->ad;
    if (out) {
        if (P.lambda == 0.0)
            return set_error(ctx, FIPI_ERR_UNSUPPORTED, "the lambda (and sigma) cotangents need lambda != 0");
        double pg[kParamGrads];
        FIPI_CUDA(ctx, d2h(ctx, pg, a.pg, sizeof(pg)));
        out->mobility = pg[kPgMobility];
        out->lambda = pg[kPgLambda];
        out->k_n = pg[kPgKn];
        out->sigma_attach = pg[kPgSigmaAttach];
        // lambda = sigma eps 3 / 2 / sqrt 2 (head.hpp:47), k_n = 0.5 sigma (parameter.hpp:18)
        out->sigma = pg[kPgSigmaAttach] + pg[kPgLambda] * (P.epsilon * 3.0 / 2.0 / std::sqrt(2.0)) +
                     pg[kPgKn] * 0.5;
    }
    const int n = ctx->pb.n;
    if (dcos_theta && n > 0) FIPI_CUDA(ctx, d2h(ctx, dcos_theta, a.dct, sizeof(D) * (size_t)n));
    return check_status(ctx);
}

fipi_status fipi_adjoint_get_history(fipi_ctx* ctx, double* dc_old, double* df_old, double* dconv_old) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    fipi_status st = adjoint_ready(ctx);
    if (st != FIPI_OK) return st;
    AdjBufs& a = ctx->ad;
    const size_t V = (size_t)ctx->g.V;
    double* outs[3] = {dc_old, df_old, dconv_old};
    void* srcs[3] = {a.la_co, a.la_fo, a.la_Co};
    for (int i = 0; i < 3; ++i) {
        if (!outs[i]) continue;
        c2r_into(ctx, sp(srcs[i]), a.lamF);
        FIPI_CUDA(ctx, d2h(ctx, outs[i], a.lamF, sizeof(D) * V));
    }
    return check_status(ctx);
}

fipi_status fipi_trajectory_forward(fipi_ctx* ctx, int nsteps, int stride) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    if (nsteps < 1) return set_error(ctx, FIPI_ERR_BAD_ARG, "nsteps < 1");
    if (!ctx->have_phase) return set_error(ctx, FIPI_ERR_STATE, "fipi_set_phase must come first");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    CheckpointStore::Traj tr;
    tr.t0 = ctx->t;
    tr.n = nsteps;
    tr.s = stride > 0 ? stride : (int)std::ceil(std::sqrt((double)nsteps));
    if (tr.s > nsteps) tr.s = nsteps;
    tr.K = (nsteps + tr.s - 1) / tr.s;
    fipi_status st = ck_reserve(ctx, tr.K + tr.s + 1);
    if (st != FIPI_OK) return st;
    for (int k = 0; k < tr.K; ++k) {
        st = ck_save(ctx, k);
        if (st != FIPI_OK) return st;
        const int len = std::min(tr.s, nsteps - k * tr.s);
        st = fipi_step(ctx, len);
        if (st != FIPI_OK) return st;
    }
    ctx->ck.traj = tr;
    return FIPI_OK;
}

fipi_status fipi_trajectory_backward(fipi_ctx* ctx, const double* dc, const double* du, const double* dp,
                                     const double* df_pp) {
    if (!ctx) return set_error(ctx, FIPI_ERR_BAD_ARG, "ctx is NULL");
    FIPI_CUDA(ctx, cudaSetDevice(ctx->device));
    CheckpointStore::Traj* tr = &ctx->ck.traj;
    if (tr->t0 < 0) return set_error(ctx, FIPI_ERR_STATE, "fipi_trajectory_forward must come first");
    if (ctx->t != tr->t0 + tr->n)
        return set_error(ctx, FIPI_ERR_STATE, "the state moved since fipi_trajectory_forward");
    if (ctx->ck.slots < tr->K + tr->s + 1) return set_error(ctx, FIPI_ERR_STATE, "checkpoint slots were released");
    fipi_status st = adjoint_seed_impl(ctx, dc, du, dp, df_pp);
    if (st != FIPI_OK) return st;
    // per-step tapes of one segment: u^n and mu^{n+1} (4V doubles per step)
    AdjBufs& a = ctx->ad;
    const size_t V = (size_t)ctx->g.V;
    if (a.seg_tape_steps < tr->s) {
        if (a.seg_tape) {
            cudaFree(a.seg_tape);
            ctx->device_bytes -= sizeof(D) * 4 * V * (size_t)a.seg_tape_steps;
            a.seg_tape = nullptr;
            a.seg_tape_steps = 0;
        }
        FIPI_CUDA(ctx, cudaMalloc((void**)&a.seg_tape, sizeof(D) * 4 * V * (size_t)tr->s));
        a.seg_tape_steps = tr->s;
        ctx->device_bytes += sizeof(D) * 4 * V * (size_t)tr->s;
    }
    // Each segment is run once more from its checkpoint with its tapes kept
    // and its states (the one after the last step too) in the slots K..K+len;
    // its steps are then reversed from those without recomputing them.
    for (int k = tr->K - 1; k >= 0; --k) {
        const int len = std::min(tr->s, tr->n - k * tr->s);
        st = ck_load(ctx, k);
        if (st != FIPI_OK) return st;
        for (int j = 0; j < len; ++j) {
            st = ck_save(ctx, tr->K + j);
            if (st != FIPI_OK) return st;
            double* tp = a.seg_tape + 4 * V * (size_t)j;
            ctx->tape_u[0] = tp;
            ctx->tape_u[1] = tp + V;
            ctx->tape_u[2] = tp + 2 * V;
            ctx->tape_mu = tp + 3 * V;
            enqueue_step(ctx);  // direct launches: the step graphs hold no tape
            ctx->tape_u[0] = ctx->tape_u[1] = ctx->tape_u[2] = nullptr;
            ctx->tape_mu = nullptr;
        }
        st = ck_save(ctx, tr->K + len);
        if (st != FIPI_OK) return st;
        st = check_status(ctx);
        if (st != FIPI_OK) return st;
        for (int j = len - 1; j >= 0; --j) {
            st = adjoint_reverse_pair(ctx, tr->K + j, tr->K + j + 1, a.seg_tape + 4 * V * (size_t)j);
            if (st != FIPI_OK) return st;
        }
        st = check_status(ctx);
        if (st != FIPI_OK) return st;
    }
    tr->t0 = -1;  // the state is no longer the trajectory's end
    return FIPI_OK;
}

}  // extern "C"
