// Eulerian side of the FIPI step on sm_103a: the pseudo-spectral
// Cahn-Hilliard update and the Stokes projection (main.cpp:79-181 of the
// reference), as 3-pass R2C/C2R FFTs with the element-wise work fused into
// the passes.  Per step (13 transforms):
//
//   A  u_hat -> u (3 inverse), conv = u . grad c, C_hat = R2C(conv)
//      with the SBDF2 / IMEX update fused into the last forward Z pass
//   B  c^{n+1} = C2R(c_hat), f = (lambda/eps^2)(c^3 - c) fused, f_hat = R2C(f)
//   C  mu = C2R(lambda k^2 c_hat + f_hat), grad c = C2R(i k c_hat) (4 inverse),
//      F = mu grad c + spread + buoyancy fused, F_hat = R2C(F) (3 forward)
//      with the Leray projection fused into the last Z pass -> u_hat
//
// Template parameter T is the arithmetic type: double (plain FP64 form) or
// float (mixed form, whose k = 0 mode of c lives in FP64 scalars).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "ctx.hpp"
#include "passes.cuh"


namespace fipi {

// ------------------------------------------------------------ X-pass ops
// R2C of c and of f = (lambda/eps^2)(c^3 - c) from the real c (set-up).
template <typename T> struct OpInitCF {
    using C = cplx<T>;
    const T* c;
    C* o0;
    C* o1;
    T lam_eps;
    int nx, ny;
    __device__ C* out(int f) const { return f == 0 ? o0 : o1; }
    __device__ const C* in(int) const { return nullptr; }
    __device__ void point(int z, int y, int n, C* v) const {
        const C cc = reinterpret_cast<const C*>(c + ((size_t)z * ny + y) * nx)[n];
        v[0] = cc;
        v[1] = mkc<C>((cc.x * cc.x * cc.x - cc.x) * lam_eps, (cc.y * cc.y * cc.y - cc.y) * lam_eps);
    }
};

// R2C of one real field (fine-grained fipi_fft_r2c).
template <typename T> struct OpR2C {
    using C = cplx<T>;
    const T* src;
    C* o0;
    int nx, ny;
    __device__ C* out(int) const { return o0; }
    __device__ const C* in(int) const { return nullptr; }
    __device__ void point(int z, int y, int n, C* v) const {
        v[0] = reinterpret_cast<const C*>(src + ((size_t)z * ny + y) * nx)[n];
    }
};


// Step A: u (3 inverse) . grad c -> conv (1 forward).  main.cpp:91-92
template <typename T, bool MIXED> struct OpConv {
    using C = cplx<T>;
    const C* uS[3];
    const T* g[3];
    C* o0;
    double* partials;
    T* tape_u[3];  // non-NULL: u is also stored (adjoint recompute)
    int nx, ny;
    __device__ const C* in(int f) const { return uS[f]; }
    __device__ C* out(int) const { return o0; }
    template <class A> __device__ void point(int z, int y, int n, C* v, A& acc) const {
        point(z, y, n, v, acc, XGlobalRow<T, 3>{{g[0], g[1], g[2]}, ((size_t)z * ny + y) * nx});
    }
    template <class A, class R> __device__ void point(int z, int y, int n, C* v, A& acc, const R& r) const {
        T s0 = T(0), s1 = T(0);
        if (tape_u[0]) {
            const size_t row = ((size_t)z * ny + y) * nx;
#pragma unroll
            for (int d = 0; d < 3; ++d) reinterpret_cast<C*>(tape_u[d] + row)[n] = v[d];
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const C gg = r.get(d, n);
            s0 += v[d].x * gg.x;
            s1 += v[d].y * gg.y;
        }
        v[0] = mkc<C>(s0, s1);
        if (MIXED) acc += s0 + s1;  // per-thread FP32 partial; FP64 from the block sum on
    }
    // k_xpass_stream: u_f . (grad c)_f accumulated field by field; the rows
    // of grad_F c are prefetched into L2 at the start of the block and read
    // in round F
    struct State {
        C s;
    };
    static constexpr int emit_after(int f) { return f == 2 ? 0 : -1; }
    __device__ void prefetch_rows(int z, int y0, int rows) const {
        const size_t row = ((size_t)z * ny + y0) * nx;
        const uint32_t bytes = (uint32_t)((size_t)rows * nx * sizeof(T));
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if ((((uintptr_t)(g[d] + row)) | bytes) % 16 == 0) prefetch_l2_bulk(g[d] + row, bytes);
    }
    template <int F, class A> __device__ C take(int z, int y, int n, C v, State& st, A& acc) const {
        const size_t row = ((size_t)z * ny + y) * nx;
        const C gg = reinterpret_cast<const C*>(g[F] + row)[n];
        if (tape_u[0]) reinterpret_cast<C*>(tape_u[F] + row)[n] = v;
        if (F == 0) {
            T s0 = T(0), s1 = T(0);
            s0 += v.x * gg.x;
            s1 += v.y * gg.y;
            st.s = mkc<C>(s0, s1);
        } else {
            st.s.x += v.x * gg.x;
            st.s.y += v.y * gg.y;
        }
        if (F == 2 && MIXED) acc += st.s.x + st.s.y;
        return st.s;
    }
};

// Step B: c = C2R(c_hat) (+ FP64 mean in the mixed form), f = (lambda/eps^2)(c^3 - c).
template <typename T, bool MIXED> struct OpCF {
    using C = cplx<T>;
    const C* cS;
    T* c;
    C* o0;
    const float* cbar;  // mixed: mean of c (the FP64 k = 0 mode / V) rounded to FP32
    T lam_eps;
    int nx, ny;
    __device__ const C* in(int) const { return cS; }
    __device__ C* out(int) const { return o0; }
    template <class A> __device__ void point(int z, int y, int n, C* v, A&) const {
        C cc = v[0];
        if (MIXED) {
            const T cb = (T)*cbar;
            cc.x += cb;
            cc.y += cb;
        }
        reinterpret_cast<C*>(c + ((size_t)z * ny + y) * nx)[n] = cc;
        v[0] = mkc<C>((cc.x * cc.x * cc.x - cc.x) * lam_eps, (cc.y * cc.y * cc.y - cc.y) * lam_eps);
    }
    // k_xpass_stream
    struct State {};
    static constexpr int emit_after(int f) { return f == 0 ? 0 : -1; }
    template <int F, class A> __device__ C take(int z, int y, int n, C v, State&, A& acc) const {
        point(z, y, n, &v, acc);
        return v;
    }
};

// Step C: mu, grad c (4 inverse) -> F = mu grad c + spread + buoyancy (3 forward).
// main.cpp:149-172; the spread term is cluster::compute_f_r.
template <typename T> struct OpForce {
    using C = cplx<T>;
    const C* S[4];
    T* g[3];
    const T* c;
    const T* fsp[3];
    int spread;
    T rho1, rho2, gravity;
    T* tape_mu;  // non-NULL: mu is also stored (adjoint recompute)
    int nx, ny;
    __device__ const C* in(int f) const { return S[f]; }
    __device__ C* out(int f) const { return const_cast<C*>(S[f]); }
    // the rows of c and of the spread force are contiguous per tile
    __device__ void prefetch_rows(int z, int y0, int rows) const {
        const size_t row = ((size_t)z * ny + y0) * nx;
        const uint32_t bytes = (uint32_t)((size_t)rows * nx * sizeof(T));
        auto pf = [&](const T* a) {
            if ((((uintptr_t)(a + row)) | bytes) % 16 == 0) prefetch_l2_bulk(a + row, bytes);
        };
        if (gravity != T(0)) pf(c);
        if (spread)
            for (int d = 0; d < 3; ++d) pf(fsp[d]);
    }
    template <class A> __device__ void point(int z, int y, int n, C* v, A& acc) const {
        point(z, y, n, v, acc, XGlobalRow<T, 4>{{c, fsp[0], fsp[1], fsp[2]}, ((size_t)z * ny + y) * nx});
    }
    template <class A, class R> __device__ void point(int z, int y, int n, C* v, A&, const R& r) const {
        const size_t row = ((size_t)z * ny + y) * nx;
        const C mu = v[0];
        if (tape_mu) reinterpret_cast<C*>(tape_mu + row)[n] = mu;
        // buoyancy ((1+c)/2 rho1 + (1-c)/2 rho2) g, g = (0, 0, gravity); with
        // gravity = 0 it adds exactly zero and c is not read
        T b0 = T(0), b1 = T(0);
        if (gravity != T(0)) {
            const C cc = r.get(0, n);
            b0 = ((cc.x + T(1)) / T(2)) * rho1 + ((cc.x * T(-1) + T(1)) / T(2)) * rho2;
            b1 = ((cc.y + T(1)) / T(2)) * rho1 + ((cc.y * T(-1) + T(1)) / T(2)) * rho2;
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const C gd = v[1 + d];
            reinterpret_cast<C*>(g[d] + row)[n] = gd;
            T f0 = mu.x * gd.x, f1 = mu.y * gd.y;
            if (spread) {
                const C sp = r.get(1 + d, n);
                f0 += sp.x;
                f1 += sp.y;
            }
            if (d == 2 && gravity != T(0)) {
                f0 += b0 * gravity;
                f1 += b1 * gravity;
            }
            v[d] = mkc<C>(f0, f1);
        }
    }
};

// ------------------------------------------------------------ Z-pass ops
// Z forward with the Cahn-Hilliard update (main.cpp:95-138) fused.
// The conv spectrum C^n is the transformed input; c_hat^{n+1} is written
// over c_hat^{n-1} at the same index.
//
// FP64 form: the reference's histories and evaluation order (bit parity):
// C^n is written over C^{n-1}.
// Mixed form: the three histories enter the SBDF2 numerator only as
// H^n = -c_hat^{n-1} + 2 dt M k^2 f_hat^{n-1} + 2 dt C^{n-1}, so the step
// stores H^{n+1} = -c_hat^n + 2 dt M k^2 f_hat^n + 2 dt C^n (in the C^{n-1}
// array) and reads it back at the next step instead of the three arrays:
// two spectral reads fewer per step.  (The history term carries the
// mobility of the step that stored it.)
template <typename T, bool MIXED> struct ZOpCH {
    using C = cplx<T>;
    const C* conv;
    const C* chat;
    C* chat_old;  // in: c^{n-1} (FP64); out: c^{n+1}
    const C* fhat;
    const C* fhat_old;
    C* Chat_old;  // FP64: in C^{n-1}, out C^n;  mixed: in H^n, out H^{n+1}
    KTabs<T> kt;
    StepConsts<T> k;
    int first;     // t == 0
    int conserve;  // mass-conserving mode: the k = 0 mode of C^n is taken as 0
    __device__ void load(int, int, int, size_t gi, C* v) const { v[0] = conv[gi]; }
    __device__ void store(int ix, int iy, int iz, size_t gi, const C* v) const {
        Pre p;
        pre(gi, p);
        update(ix, iy, iz, gi, v[0], p);
    }
    struct Pre {
        C c, f, co, fo, Co;  // mixed: Co holds H^n, co and fo unused
    };
    __device__ void pre(size_t gi, Pre& p) const {
        p.c = chat[gi];
        p.f = fhat[gi];
        if (!first) {
            if constexpr (!MIXED) {
                p.co = chat_old[gi];
                p.fo = fhat_old[gi];
            }
            p.Co = Chat_old[gi];
        }
    }
    // Writes c_hat^{n+1} and the history at gi and returns c_hat^{n+1}.
    __device__ C update(int ix, int iy, int iz, size_t gi, C Cn, const Pre& p) const {
        if (conserve && gi == 0) Cn = mkc<C>(T(0), T(0));
        const C c = p.c;
        const C f = p.f;
        const T k2 = kt.k2(ix, iy, iz);
        const T k4 = k2 * k2;
        C out;
        if (first) {
            const T a = k2 * k.s1;
            T re = c.x - a * f.x, im = c.y - a * f.y;
            re -= Cn.x * k.dt;
            im -= Cn.y * k.dt;
            const T den = k4 * k.s2 + T(1);
            out = mkc<C>(re / den, im / den);
        } else if constexpr (!MIXED) {
            const C co = p.co;
            const C fo = p.fo;
            const C Co = p.Co;
            T re = c.x * T(4) - co.x, im = c.y * T(4) - co.y;
            const T a4 = k2 * k.s4, a2 = k2 * k.s2m;
            re -= a4 * f.x;
            im -= a4 * f.y;
            re += a2 * fo.x;
            im += a2 * fo.y;
            re -= Cn.x * k.s4c;
            im -= Cn.y * k.s4c;
            re += Co.x * k.s2c;
            im += Co.y * k.s2c;
            const T den = k4 * k.s3 + T(3);
            out = mkc<C>(re / den, im / den);
        } else {
            const T a4 = k2 * k.s4;
            T re = c.x * T(4) + p.Co.x, im = c.y * T(4) + p.Co.y;
            re -= a4 * f.x;
            im -= a4 * f.y;
            re -= Cn.x * k.s4c;
            im -= Cn.y * k.s4c;
            const T den = k4 * k.s3 + T(3);
            out = mkc<C>(re / den, im / den);
        }
        if (MIXED && gi == 0) out = mkc<C>(T(0), T(0));  // k = 0 lives in FP64 scalars
        chat_old[gi] = out;
        if constexpr (MIXED) {
            const T a2 = k2 * k.s2m;  // H^{n+1} = -c^n + 2 dt M k^2 f^n + 2 dt C^n
            Chat_old[gi] = mkc<C>(a2 * f.x + k.s2c * Cn.x - c.x, a2 * f.y + k.s2c * Cn.y - c.y);
        } else {
            Chat_old[gi] = Cn;
        }
        return out;
    }
};

// FP64 k = 0 update of the mixed form: c_hat(0) follows the same IMEX /
// SBDF2 recurrence with k = 0 (the f terms vanish), C(0) from the FP64
// per-block sums of conv.  k0 = [c0, c0_old, C0_old, C0_cur].
// All threads of one block call it.
__device__ __forceinline__ void k0_update_block(double* k0, const double* partials, int np, int first, double dt,
                                                double invV, int conserve) {
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partials[i];
    s = block_sum(s);
    if (conserve) s = 0.0;  // mass-conserving mode: C(0) = 0
    if (threadIdx.x == 0) {
        const double c0 = k0[0], c0o = k0[1], C0o = k0[2];
        double nw;
        if (first) {
            nw = c0 - s * dt;
        } else {
            double re = c0 * 4.0 - c0o;
            re -= s * (4.0 * dt);
            re += C0o * (2.0 * dt);
            nw = re / 3.0;
        }
        k0[1] = c0;
        k0[0] = nw;
        k0[2] = s;
        k0[3] = s;
        *reinterpret_cast<float*>(k0 + 4) = (float)(nw * invV);  // mean of c for the FP32 fields
    }
}

// Round trip A -> B (k_zpass_rt, NF = NB = 1): the CH update of ZOpCH in
// the forward Z pass, then the inverse Z transform of c_hat^{n+1} (the
// first pass of c^{n+1} = C2R(c_hat^{n+1})) into `out`.
// In the mixed form the first block also advances the FP64 k = 0 record
// from the conv pass's block sums (nothing else in this pass reads it).
template <typename T, bool MIXED> struct ZOpCHRt {
    using C = cplx<T>;
    ZOpCH<T, MIXED> ch;
    C* out;
    double* k0;
    const double* partials;
    int np;
    double dt, invV;
    __device__ void prologue() const {
        if (MIXED && blockIdx.x == 0 && blockIdx.y == 0)
            k0_update_block(k0, partials, np, ch.first, dt, invV, ch.conserve);
    }
    __device__ void load(int, int, int, size_t gi, C* v) const { v[0] = ch.conv[gi]; }
    __device__ const C* src(int) const { return ch.conv; }
    using PreT = typename ZOpCH<T, MIXED>::Pre;
    __device__ void pre(int, int, int, size_t gi, PreT& p) const { ch.pre(gi, p); }
    __device__ void mid(int ix, int iy, int iz, size_t gi, const C* vi, C* vo, const PreT& p) const {
        vo[0] = ch.update(ix, iy, iz, gi, vi[0], p);
    }
    __device__ void mid(int ix, int iy, int iz, size_t gi, const C* vi, C* vo) const {
        PreT p;
        ch.pre(gi, p);
        mid(ix, iy, iz, gi, vi, vo, p);
    }
    __device__ void store2(int, int, int, size_t gi, const C* v) const { out[gi] = v[0]; }
    // register round trip (k_zpass_rr)
    struct State {
        C c;
    };
    __device__ void rr_mid(int ix, int iy, int iz, size_t gi, const C* w, State& st) const {
        PreT p;
        ch.pre(gi, p);
        st.c = ch.update(ix, iy, iz, gi, w[0], p);
    }
    __device__ C rr_out(int, int, int, int, const State& st) const { return st.c; }
    __device__ void rr_store(int, size_t gi, C v) const { out[gi] = v; }
};

// Round trip B -> C (NF = 1, NB = 4): the forward Z transform of f gives
// f_hat^{n+1} (stored); mu_hat = lambda k^2 c_hat + f_hat (main.cpp:157) and
// i k_d c_hat with the Nyquist index of d zeroed (field.cpp:288-328) are
// transformed back along z into out[0..3] (the inverses of mu and grad c).
template <typename T> struct ZOpFRt {
    using C = cplx<T>;
    const C* fin;
    C* fhat_out;
    const C* chat;
    C* out[4];
    KTabs<T> kt;
    T lam;
    int m, ny2, nz2;
    __device__ void prologue() const {}
    __device__ void load(int, int, int, size_t gi, C* v) const { v[0] = fin[gi]; }
    __device__ const C* src(int) const { return fin; }
    struct PreT {
        C c;
    };
    __device__ void pre(int, int, int, size_t gi, PreT& p) const { p.c = chat[gi]; }
    __device__ void mid(int ix, int iy, int iz, size_t gi, const C* vi, C* vo) const {
        PreT p;
        pre(ix, iy, iz, gi, p);
        mid(ix, iy, iz, gi, vi, vo, p);
    }
    __device__ void mid(int ix, int iy, int iz, size_t gi, const C* vi, C* vo, const PreT& p) const {
        const C f = vi[0];
        fhat_out[gi] = f;
        const C c = p.c;
        const T a = kt.k2(ix, iy, iz) * lam;
        vo[0] = mkc<C>(a * c.x + f.x, a * c.y + f.y);
        const T kx = kt.kx[ix], ky = kt.ky[iy], kz = kt.kz[iz];
        vo[1] = (ix == m) ? mkc<C>(T(0), T(0)) : mkc<C>(-kx * c.y, kx * c.x);
        vo[2] = (iy == ny2) ? mkc<C>(T(0), T(0)) : mkc<C>(-ky * c.y, ky * c.x);
        vo[3] = (iz == nz2) ? mkc<C>(T(0), T(0)) : mkc<C>(-kz * c.y, kz * c.x);
    }
    __device__ void store2(int, int, int, size_t gi, const C* v) const {
#pragma unroll
        for (int b = 0; b < 4; ++b) out[b][gi] = v[b];
    }
    // register round trip (k_zpass_rr): the outputs are formed one at a time;
    // f_hat is kept for output 0 only, c_hat (the staged aux tile) is read
    // again for each output
    struct State {
        C f;
    };
    __device__ const C* aux() const { return chat; }
    __device__ void rr_mid(int, int, int, size_t gi, const C* w, C, State& st) const {
        fhat_out[gi] = w[0];
        st.f = w[0];
    }
    __device__ C rr_out(int b, int ix, int iy, int iz, const State& st, C c) const {
        if (b == 0) {
            const T a = kt.k2(ix, iy, iz) * lam;
            return mkc<C>(a * c.x + st.f.x, a * c.y + st.f.y);
        }
        const T kd = b == 1 ? kt.kx[ix] : b == 2 ? kt.ky[iy] : kt.kz[iz];
        const bool nyq = b == 1 ? ix == m : b == 2 ? iy == ny2 : iz == nz2;
        return nyq ? mkc<C>(T(0), T(0)) : mkc<C>(-kd * c.y, kd * c.x);
    }
    __device__ void rr_store(int b, size_t gi, C v) const { out[b][gi] = v; }
};

// Round trip C -> next A (NF = NB = 3): the Leray projection of ZOpProj in
// the forward Z pass, then the inverse Z transform of u_hat into upre — the
// velocity state the next step's conv pass starts from (u_hat itself is
// never stored).
template <typename T> struct ZOpProjRt {
    using C = cplx<T>;
    ZOpProj<T> pj;
    C* upre[3];
    __device__ const C* src(int f) const { return pj.in[f]; }
    __device__ void prologue() const {}
    __device__ void load(int, int, int, size_t gi, C* v) const {
        v[0] = pj.in[0][gi];
        v[1] = pj.in[1][gi];
        v[2] = pj.in[2][gi];
    }
    __device__ void mid(int ix, int iy, int iz, size_t, const C* vi, C* vo) const { pj.compute(ix, iy, iz, vi, vo); }
    __device__ void store2(int, int, int, size_t gi, const C* v) const {
        upre[0][gi] = v[0];
        upre[1][gi] = v[1];
        upre[2][gi] = v[2];
    }
    // register round trip (k_zpass_rr)
    struct State {
        C u[3];
    };
    __device__ void rr_mid(int ix, int iy, int iz, size_t, const C* w, State& st) const { pj.compute(ix, iy, iz, w, st.u); }
    __device__ C rr_out(int b, int, int, int, const State& st) const { return st.u[b]; }
    __device__ void rr_store(int b, size_t gi, C v) const { upre[b][gi] = v; }
};

// Z inverse prologue: mu_hat = lambda k^2 c_hat + f_hat (main.cpp:157).
template <typename T> struct ZOpMu {
    using C = cplx<T>;
    const C* chat;
    const C* fhat;
    C* out;
    KTabs<T> kt;
    T lam;
    __device__ void load(int ix, int iy, int iz, size_t gi, C* v) const {
        const T a = kt.k2(ix, iy, iz) * lam;
        const C c = chat[gi], f = fhat[gi];
        v[0] = mkc<C>(a * c.x + f.x, a * c.y + f.y);
    }
    __device__ void store(int, int, int, size_t gi, const C* v) const { out[gi] = v[0]; }
};

// Z inverse prologue: i k_d c_hat, zero at the Nyquist index of d (field.cpp:288-328).
template <typename T> struct ZOpGrad {
    using C = cplx<T>;
    const C* chat;
    C* out[3];
    KTabs<T> kt;
    int m, ny2, nz2;
    __device__ void load(int ix, int iy, int iz, size_t gi, C* v) const {
        const C c = chat[gi];
        const T kx = kt.kx[ix], ky = kt.ky[iy], kz = kt.kz[iz];
        v[0] = (ix == m) ? mkc<C>(T(0), T(0)) : mkc<C>(-kx * c.y, kx * c.x);
        v[1] = (iy == ny2) ? mkc<C>(T(0), T(0)) : mkc<C>(-ky * c.y, ky * c.x);
        v[2] = (iz == nz2) ? mkc<C>(T(0), T(0)) : mkc<C>(-kz * c.y, kz * c.x);
    }
    __device__ void store(int, int, int, size_t gi, const C* v) const {
        out[0][gi] = v[0];
        out[1][gi] = v[1];
        out[2][gi] = v[2];
    }
};




// FP64 per-block sums for mass and free energy (main.cpp:232, field.cpp:507-516).
template <typename T>
__global__ void k_diag(const T* __restrict__ c, const T* __restrict__ g0, const T* __restrict__ g1,
                       const T* __restrict__ g2, size_t V, double lam, double e2, double dv,
                       double* partials, int mode) {
    double s = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < V; i += (size_t)gridDim.x * blockDim.x) {
        const double cr = (double)c[i];
        if (mode == 0) {
            s += cr;
        } else {
            const double a = g0[i], b = g1[i], d = g2[i];
            double g2s = a * a;
            g2s += b * b;
            g2s += d * d;
            const double w = cr * cr - 1.0;
            const double fe = (g2s * 0.5 + (w * w) * e2) * lam;
            s += fe * dv;
        }
    }
    s = block_sum(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}


// grad c (real, 3 fields) from c_hat.
template <typename T> void grad_from_chat(fipi_ctx* ctx, const cplx<T>* chat, T* const g3[3]) {
    using C = cplx<T>;
    const Geom& g = ctx->g;
    ZOpGrad<T> zg{chat, {F<T>::S(ctx, 1), F<T>::S(ctx, 2), F<T>::S(ctx, 3)}, F<T>::ktabs(ctx), g.m,
                  g.ny / 2, g.nz / 2};
    launch_z<T, 3, +1>(ctx, "Z inverse grad", 4, zg);
    void* sp[3] = {ctx->fb.S[1], ctx->fb.S[2], ctx->fb.S[3]};
    launch_y<T>(ctx, 3, sp, sp, +1);
    OpC2RStore<T, 3> op{{F<T>::S(ctx, 1), F<T>::S(ctx, 2), F<T>::S(ctx, 3)}, {g3[0], g3[1], g3[2]}, g.nx, g.ny};
    launch_x<T, 3, 0, false>(ctx, "X inverse store", 3, NoAcc<OpC2RStore<T, 3>>{op});
    (void)sizeof(C);
}

// ------------------------------------------------------------ allocation
template <typename T> static fipi_status alloc_fields_t(fipi_ctx* ctx) {
    using C = cplx<T>;
    const Geom& g = ctx->g;
    FieldBufs& b = ctx->fb;
    const size_t V = (size_t)g.V, SH = (size_t)g.SH;
    auto A = [&](void** p, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) ctx->device_bytes += bytes;
        return e;
    };
    FIPI_CUDA(ctx, A(&b.twx, sizeof(C) * g.nx));
    FIPI_CUDA(ctx, A(&b.twy, sizeof(C) * g.ny));
    FIPI_CUDA(ctx, A(&b.twz, sizeof(C) * g.nz));
    FIPI_CUDA(ctx, A(&b.kx, sizeof(T) * (g.m + 1)));
    FIPI_CUDA(ctx, A(&b.ky, sizeof(T) * g.ny));
    FIPI_CUDA(ctx, A(&b.kz, sizeof(T) * g.nz));
    FIPI_CUDA(ctx, A(&b.c, sizeof(T) * V));
    for (int d = 0; d < 3; ++d) {
        FIPI_CUDA(ctx, A(&b.g[d], sizeof(T) * V));
        FIPI_CUDA(ctx, A(&b.fsp[d], sizeof(T) * V));
        FIPI_CUDA(ctx, cudaMemsetAsync(b.fsp[d], 0, sizeof(T) * V, ctx->stream));
        FIPI_CUDA(ctx, A(&b.upre[d], sizeof(C) * SH));
        FIPI_CUDA(ctx, cudaMemsetAsync(b.upre[d], 0, sizeof(C) * SH, ctx->stream));
    }
    FIPI_CUDA(ctx, A(&b.ureal, sizeof(T) * V * 3));
    void** specs[] = {&b.chat, &b.chat_old, &b.fhat, &b.fhat_old, &b.Chat_old, &b.S[0], &b.S[1], &b.S[2], &b.S[3]};
    for (void** p : specs) {
        FIPI_CUDA(ctx, A(p, sizeof(C) * SH));
        FIPI_CUDA(ctx, cudaMemsetAsync(*p, 0, sizeof(C) * SH, ctx->stream));
    }
    // twiddles and wave numbers, computed in extended precision on the host
    auto twiddles = [&](int n) {
        std::vector<C> t(n);
        const long double two_pi = 6.283185307179586476925286766559005768L;
        for (int q = 0; q < n; ++q) {
            const long double a = two_pi * (long double)q / (long double)n;
            t[q].x = (T)cosl(a);
            t[q].y = (T)(-sinl(a));
        }
        return t;
    };
    auto tx = twiddles(g.nx), ty = twiddles(g.ny), tz = twiddles(g.nz);
    FIPI_CUDA(ctx, h2d(ctx, b.twx, tx.data(), sizeof(C) * g.nx));
    FIPI_CUDA(ctx, h2d(ctx, b.twy, ty.data(), sizeof(C) * g.ny));
    FIPI_CUDA(ctx, h2d(ctx, b.twz, tz.data(), sizeof(C) * g.nz));
    // field.cpp:100-121: i*2.0*pi/L for i <= N/2 else (i - N)*2.0*pi/L
    const fipi_params& P = ctx->P;
    auto waves = [&](int n, int count, double L) {
        std::vector<T> k(count);
        for (int i = 0; i < count; ++i) k[i] = (T)((i <= n / 2) ? i * 2.0 * P.pi / L : (i - n) * 2.0 * P.pi / L);
        return k;
    };
    auto kx = waves(g.nx, g.m + 1, P.lx), ky = waves(g.ny, g.ny, P.ly), kz = waves(g.nz, g.nz, P.lz);
    FIPI_CUDA(ctx, h2d(ctx, b.kx, kx.data(), sizeof(T) * (g.m + 1)));
    FIPI_CUDA(ctx, h2d(ctx, b.ky, ky.data(), sizeof(T) * g.ny));
    FIPI_CUDA(ctx, h2d(ctx, b.kz, kz.data(), sizeof(T) * g.nz));
    return FIPI_OK;
}

fipi_status fields_alloc(fipi_ctx* ctx) {
    const fipi_params& P = ctx->P;
    Geom& g = ctx->g;
    g.nx = P.nx;
    g.ny = P.ny;
    g.nz = P.nz;
    g.m = P.nx / 2;
    g.h = P.nx / 2 + 1;
    g.lm = ilog2i(g.m);
    g.ly = ilog2i(g.ny);
    g.lz = ilog2i(g.nz);
    g.V = (long long)P.nx * P.ny * P.nz;
    g.SH = (long long)P.nz * g.h * P.ny;
    fipi_status st = (ctx->prec == FIPI_MIXED) ? alloc_fields_t<float>(ctx) : alloc_fields_t<double>(ctx);
    if (st != FIPI_OK) return st;
    ctx->n_partials = (g.ny / 8) * g.nz;  // upper bound of X-pass blocks (TY >= 8)
    if (ctx->n_partials < 1024) ctx->n_partials = 1024;
    FIPI_CUDA(ctx, cudaMalloc(&ctx->partials, sizeof(double) * ctx->n_partials));
    FIPI_CUDA(ctx, cudaMalloc(&ctx->k0, sizeof(double) * 6));
    FIPI_CUDA(ctx, cudaMemsetAsync(ctx->k0, 0, sizeof(double) * 6, ctx->stream));
    ctx->device_bytes += sizeof(double) * (ctx->n_partials + 4);
    return FIPI_OK;
}

void fields_free(fipi_ctx* ctx) {
    FieldBufs& b = ctx->fb;
    void* all[] = {b.twx, b.twy, b.twz, b.kx, b.ky, b.kz, b.c, b.ureal, b.chat, b.chat_old, b.fhat,
                   b.fhat_old, b.Chat_old, b.S[0], b.S[1], b.S[2], b.S[3], b.g[0], b.g[1], b.g[2],
                   b.fsp[0], b.fsp[1], b.fsp[2], b.upre[0], b.upre[1], b.upre[2], ctx->partials, ctx->k0};
    for (void* p : all)
        if (p) cudaFree(p);
    b = FieldBufs{};
    ctx->partials = nullptr;
    ctx->k0 = nullptr;
}


// t = 0 state: c, c_hat, f_hat, grad c (everything main.cpp:81-92 needs).
// FP64 values into a T field from host memory or, with `dev`, from device
// memory of the context's device (no host copy).
template <typename T> static fipi_status load_real(fipi_ctx* ctx, const double* src, T* dst, size_t n, bool dev) {
    if (!dev) return upload<T>(ctx, src, dst, n);
    if (sizeof(T) == sizeof(double)) {
        FIPI_CUDA(ctx, cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        LaunchScope ls(ctx, "convert", 0.0);
        k_convert<double, T><<<1024, 256, 0, ctx->stream>>>(src, dst, n);
    }
    return FIPI_OK;
}
template <typename T> static fipi_status store_real(fipi_ctx* ctx, const T* src, double* dst, size_t n, bool dev) {
    if (!dev) return download<T>(ctx, src, dst, n);
    if (sizeof(T) == sizeof(double)) {
        FIPI_CUDA(ctx, cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        LaunchScope ls(ctx, "convert", 0.0);
        k_convert<T, double><<<1024, 256, 0, ctx->stream>>>(src, dst, n);
    }
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return FIPI_OK;
}

// Compensated (Neumaier) FP64 sum of device values in a fixed order:
// kSumBlocks x 256 strided partial sums, then one thread over the partials.
constexpr int kSumBlocks = 1024;
__device__ __forceinline__ void neumaier_add(double& s, double& c, double x) {
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
    s = t;
}
__global__ void k_sum_partials(const double* __restrict__ x, size_t n, double* part) {
    __shared__ double sh[256];
    double s = 0.0, c = 0.0;
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)kSumBlocks * 256) neumaier_add(s, c, x[i]);
    sh[threadIdx.x] = s + c;
    __syncthreads();
    if (threadIdx.x == 0) {
        double bs = 0.0, bc = 0.0;
        for (int k = 0; k < 256; ++k) neumaier_add(bs, bc, sh[k]);
        part[blockIdx.x] = bs + bc;
    }
}
// k0 = {sum, sum, 0, 0}: the mixed form's FP64 k = 0 record of a new phase field
__global__ void k_sum_k0(const double* __restrict__ part, double* k0) {
    double s = 0.0, c = 0.0;
    for (int k = 0; k < kSumBlocks; ++k) neumaier_add(s, c, part[k]);
    k0[0] = k0[1] = s + c;
    k0[2] = k0[3] = 0.0;
}

template <typename T> static fipi_status set_phase_t(fipi_ctx* ctx, const double* c_src, bool dev) {
    const Geom& g = ctx->g;
    const bool mixed = ctx->prec == FIPI_MIXED;
    fipi_status st = load_real<T>(ctx, c_src, (T*)ctx->fb.c, (size_t)g.V, dev);
    if (st != FIPI_OK) return st;
    if (mixed && dev) {
        double* part = nullptr;
        FIPI_CUDA(ctx, cudaMallocAsync((void**)&part, sizeof(double) * kSumBlocks, ctx->stream));
        {
            LaunchScope ls(ctx, "phase sum", 0.0);
            k_sum_partials<<<kSumBlocks, 256, 0, ctx->stream>>>(c_src, (size_t)g.V, part);
            k_sum_k0<<<1, 1, 0, ctx->stream>>>(part, ctx->k0);
        }
        FIPI_CUDA(ctx, cudaFreeAsync(part, ctx->stream));
    } else if (mixed) {
        // FP64 k = 0 mode: sum of c (Neumaier)
        double s = 0.0, comp = 0.0;
        for (long long i = 0; i < g.V; ++i) {
            const double x = c_src[i];
            const double t = s + x;
            comp += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
            s = t;
        }
        const double k0h[4] = {s + comp, s + comp, 0.0, 0.0};
        FIPI_CUDA(ctx, cudaMemcpyAsync(ctx->k0, k0h, sizeof(k0h), cudaMemcpyHostToDevice, ctx->stream));
    }
    const StepConsts<T> k = make_consts<T>(ctx);
    OpInitCF<T> op{(const T*)ctx->fb.c, F<T>::S(ctx, 0), F<T>::S(ctx, 1), k.lam_eps, g.nx, g.ny};
    launch_x<T, 0, 2, false>(ctx, "X forward c,f", 1, NoAcc<OpInitCF<T>>{op});
    void* sp[2] = {ctx->fb.S[0], ctx->fb.S[1]};
    launch_y<T>(ctx, 2, sp, sp, -1);
    ZOpStore<T, 2> zs{{F<T>::S(ctx, 0), F<T>::S(ctx, 1)}, {F<T>::sp(ctx->fb.chat), F<T>::sp(ctx->fb.fhat)}, mixed ? 1 : 0};
    launch_z<T, 2, -1>(ctx, "Z forward store", 4, zs);
    T* g3[3] = {(T*)ctx->fb.g[0], (T*)ctx->fb.g[1], (T*)ctx->fb.g[2]};
    grad_from_chat<T>(ctx, F<T>::sp(ctx->fb.chat), g3);
    FIPI_CUDA(ctx, cudaGetLastError());
    return FIPI_OK;
}

fipi_status fields_set_phase(fipi_ctx* ctx, const double* c, bool dev) {
    return ctx->prec == FIPI_MIXED ? set_phase_t<float>(ctx, c, dev) : set_phase_t<double>(ctx, c, dev);
}

// The velocity state is upre = Z^-1 u_hat (the first pass of the inverse
// transform u = C2R(u_hat), which is what the next step starts from);
// u_hat itself is not kept.  set_velocity: u_hat = R2C(u), then Z^-1.
template <typename T> static fipi_status set_velocity_t(fipi_ctx* ctx, const double* u_src, bool dev) {
    const Geom& g = ctx->g;
    for (int d = 0; d < 3; ++d) {
        T* tmp = (T*)ctx->fb.ureal + (size_t)d * g.V;
        fipi_status st = load_real<T>(ctx, u_src + (size_t)d * g.V, tmp, (size_t)g.V, dev);
        if (st != FIPI_OK) return st;
        OpR2C<T> op{tmp, F<T>::S(ctx, d), g.nx, g.ny};
        launch_x<T, 0, 1, false>(ctx, "X forward", 1, NoAcc<OpR2C<T>>{op});
    }
    void* s3[3] = {ctx->fb.S[0], ctx->fb.S[1], ctx->fb.S[2]};
    launch_y<T>(ctx, 3, s3, s3, -1);
    ZOpStore<T, 3> zf{{F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2)},
                      {F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2)}, 0};
    launch_z<T, 3, -1>(ctx, "Z forward store", 6, zf);
    FieldBufs& b = ctx->fb;
    ZOpStore<T, 3> zi{{F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2)},
                      {F<T>::sp(b.upre[0]), F<T>::sp(b.upre[1]), F<T>::sp(b.upre[2])}, 0};
    launch_z<T, 3, +1>(ctx, "Z inverse copy", 6, zi);
    FIPI_CUDA(ctx, cudaGetLastError());
    return FIPI_OK;
}

fipi_status fields_set_velocity(fipi_ctx* ctx, const double* u, bool dev) {
    return ctx->prec == FIPI_MIXED ? set_velocity_t<float>(ctx, u, dev) : set_velocity_t<double>(ctx, u, dev);
}

fipi_status fields_get_phase(fipi_ctx* ctx, double* c, bool dev) {
    if (ctx->prec == FIPI_MIXED) return store_real<float>(ctx, (const float*)ctx->fb.c, c, (size_t)ctx->g.V, dev);
    return store_real<double>(ctx, (const double*)ctx->fb.c, c, (size_t)ctx->g.V, dev);
}

// Real velocity u (3 x V) into fb.ureal from the velocity state.
template <typename T> static void velocity_real_t(fipi_ctx* ctx) {
    const Geom& g = ctx->g;
    void* up[3] = {ctx->fb.upre[0], ctx->fb.upre[1], ctx->fb.upre[2]};
    void* sp[3] = {ctx->fb.S[0], ctx->fb.S[1], ctx->fb.S[2]};
    launch_y<T>(ctx, 3, up, sp, +1);
    T* ur = (T*)ctx->fb.ureal;
    OpC2RStore<T, 3> op{{F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2)}, {ur, ur + g.V, ur + 2 * g.V}, g.nx, g.ny};
    launch_x<T, 3, 0, false>(ctx, "X inverse store", 3, NoAcc<OpC2RStore<T, 3>>{op});
}

void fields_velocity_real(fipi_ctx* ctx) {
    if (ctx->prec == FIPI_MIXED) velocity_real_t<float>(ctx);
    else velocity_real_t<double>(ctx);
}

template <typename T> static fipi_status get_velocity_t(fipi_ctx* ctx, double* u, bool dev) {
    velocity_real_t<T>(ctx);
    FIPI_CUDA(ctx, cudaGetLastError());
    return store_real<T>(ctx, (T*)ctx->fb.ureal, u, (size_t)ctx->g.V * 3, dev);
}

fipi_status fields_get_grad(fipi_ctx* ctx, double* g_host) {
    const size_t V = (size_t)ctx->g.V;
    for (int d = 0; d < 3; ++d) {
        fipi_status st = ctx->prec == FIPI_MIXED
                             ? download<float>(ctx, (const float*)ctx->fb.g[d], g_host + d * V, V)
                             : download<double>(ctx, (const double*)ctx->fb.g[d], g_host + d * V, V);
        if (st != FIPI_OK) return st;
    }
    return FIPI_OK;
}

fipi_status fields_get_velocity(fipi_ctx* ctx, double* u, bool dev) {
    return ctx->prec == FIPI_MIXED ? get_velocity_t<float>(ctx, u, dev) : get_velocity_t<double>(ctx, u, dev);
}

// ------------------------------------------------------------ the step
template <typename T, bool MIXED> static void step_ch_t(fipi_ctx* ctx, int t) {
    const Geom& g = ctx->g;
    FieldBufs& b = ctx->fb;
    const StepConsts<T> k = make_consts<T>(ctx);
    const KTabs<T> kt = F<T>::ktabs(ctx);
    // A: u^n (its Z inverse kept in upre by the previous step) -> Y inverse;
    //    X inverse with conv = u . grad c and the R2C of conv; Y forward;
    //    Z forward + CH update + Z inverse of c_hat^{n+1}
    void* up[3] = {b.upre[0], b.upre[1], b.upre[2]};
    void* s3[3] = {b.S[0], b.S[1], b.S[2]};
    launch_y<T>(ctx, 3, up, s3, +1);
    OpConv<T, MIXED> oc{{F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2)},
                        {(const T*)b.g[0], (const T*)b.g[1], (const T*)b.g[2]}, F<T>::S(ctx, 3), ctx->partials,
                        {(T*)ctx->tape_u[0], (T*)ctx->tape_u[1], (T*)ctx->tape_u[2]}, g.nx, g.ny};
    launch_xs<T, 3, 1, MIXED>(ctx, "X inverse u, conv, forward", 3, oc, ctx->partials);
    void* s1[1] = {b.S[3]};
    launch_y<T>(ctx, 1, s1, s1, -1);
    ZOpCH<T, MIXED> zc{F<T>::S(ctx, 3), F<T>::sp(b.chat), F<T>::sp(b.chat_old), F<T>::sp(b.fhat),
                       F<T>::sp(b.fhat_old), F<T>::sp(b.Chat_old), kt, k, t == 0 ? 1 : 0, ctx->conserve_mass};
    ZOpCHRt<T, MIXED> zcr{zc, F<T>::S(ctx, 0), ctx->k0, ctx->partials, (g.ny / x_rows_of(sizeof(T), g.m)) * g.nz,
                          ctx->P.dt, 1.0 / (double)g.V};
    // spectral arrays: conv, c, f read, c^{n+1}, history, Z^-1 c^{n+1} written; for
    // t > 0 also the history (mixed: H) or the three histories (FP64) read
    launch_zrt<T, 1, 1, -1, 16 / (sizeof(T) / 4), true>(ctx, t == 0 ? "Z forward + IMEX update + inverse" : "Z forward + SBDF2 update + inverse",
                                t == 0 ? 6 : (MIXED ? 7 : 9), zcr);
    std::swap(b.chat, b.chat_old);  // chat = c^{n+1}, chat_old = c^n
    // B: Y inverse; X inverse c^{n+1} (stored) with f = (lambda/eps^2)(c^3 - c) and its
    //    R2C; Y forward; Z forward f (f_hat^{n+1} stored) + Z inverse of mu_hat, i k c_hat
    void* s0[1] = {b.S[0]};
    launch_y<T>(ctx, 1, s0, s0, +1);
    OpCF<T, MIXED> ocf{F<T>::S(ctx, 0), (T*)b.c, F<T>::S(ctx, 1), reinterpret_cast<const float*>(ctx->k0 + 4),
                       k.lam_eps, g.nx, g.ny};
    launch_xs<T, 1, 1, false>(ctx, "X inverse c, f, forward", 1, ocf);
    void* s1b[1] = {b.S[1]};
    launch_y<T>(ctx, 1, s1b, s1b, -1);
    ZOpFRt<T> zf{F<T>::S(ctx, 1), F<T>::sp(b.fhat_old), F<T>::sp(b.chat),
                 {F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2), F<T>::S(ctx, 3)}, kt, k.lam, g.m, g.ny / 2,
                 g.nz / 2};
    launch_zrt<T, 1, 4, -1, 8 / (sizeof(T) / 4), false>(ctx, "Z forward f + inverse mu, grad", 7, zf);
    std::swap(b.fhat, b.fhat_old);  // fhat = f^{n+1}, fhat_old = f^n
}

void fields_step_ch(fipi_ctx* ctx, int t) {
    if (ctx->prec == FIPI_MIXED) step_ch_t<float, true>(ctx, t);
    else step_ch_t<double, false>(ctx, t);
}

// C: Y inverse of mu, grad c; X inverse with grad c stored and
//    F = mu grad c + spread + buoyancy, R2C of F; Y forward; Z forward +
//    projection (u_hat stored) + Z inverse of u_hat for the next step.
template <typename T> static void step_stokes_t(fipi_ctx* ctx) {
    const Geom& g = ctx->g;
    FieldBufs& b = ctx->fb;
    const StepConsts<T> k = make_consts<T>(ctx);
    const KTabs<T> kt = F<T>::ktabs(ctx);
    void* s4[4] = {b.S[0], b.S[1], b.S[2], b.S[3]};
    launch_y<T>(ctx, 4, s4, s4, +1);
    OpForce<T> of{{F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2), F<T>::S(ctx, 3)},
                  {(T*)b.g[0], (T*)b.g[1], (T*)b.g[2]},
                  (const T*)b.c,
                  {(const T*)b.fsp[0], (const T*)b.fsp[1], (const T*)b.fsp[2]},
                  (ctx->P.switch_particle && ctx->P.n_p > 0) ? 1 : 0,
                  k.rho1, k.rho2, k.gravity, (T*)ctx->tape_mu, g.nx, g.ny};
    // real arrays: grad c written; the spread grid and c (buoyancy) read when they matter
    const int nreal = 3 + (of.spread ? 3 : 0) + (ctx->P.gravity != 0.0 ? 1 : 0);
    launch_x<T, 4, 3, false>(ctx, "X inverse mu,grad, force, forward", nreal, of);
    void* s3[3] = {b.S[0], b.S[1], b.S[2]};
    launch_y<T>(ctx, 3, s3, s3, -1);
    ZOpProj<T> zp{{F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2)}, {nullptr, nullptr, nullptr}, kt, k.mu, g.m,
                  g.ny / 2, g.nz / 2};
    ZOpProjRt<T> zpr{zp, {F<T>::sp(b.upre[0]), F<T>::sp(b.upre[1]), F<T>::sp(b.upre[2])}};
    launch_zrt<T, 3, 3, -1, 16 / (sizeof(T) / 4), true>(ctx, "Z forward + projection + inverse", 6, zpr);
}


void fields_step_stokes(fipi_ctx* ctx) {
    if (ctx->prec == FIPI_MIXED) step_stokes_t<float>(ctx);
    else step_stokes_t<double>(ctx);
}

// ------------------------------------------------------------ diagnostics
template <typename T> static fipi_status diag_t(fipi_ctx* ctx, int mode, double* out) {
    const Geom& g = ctx->g;
    const fipi_params& P = ctx->P;
    const int nb = 1024;
    const double dx = P.lx / P.nx, dy = P.ly / P.ny, dz = P.lz / P.nz;
    const double dv = (mode == 0) ? dx * dy * dz : dx * dx * dx;  // field.cpp:512 uses cubic(dx)
    LaunchScope ls(ctx, "diagnostic reduce", (mode == 0 ? 1.0 : 4.0) * g.V * sizeof(T));
    k_diag<T><<<nb, 256, 0, ctx->stream>>>((const T*)ctx->fb.c, (const T*)ctx->fb.g[0], (const T*)ctx->fb.g[1],
                                           (const T*)ctx->fb.g[2], (size_t)g.V, P.lambda,
                                           0.25 / (P.epsilon * P.epsilon), dv, ctx->partials, mode);
    std::vector<double> h(nb);
    FIPI_CUDA(ctx, cudaMemcpyAsync(h.data(), ctx->partials, sizeof(double) * nb, cudaMemcpyDeviceToHost, ctx->stream));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double s = 0.0, comp = 0.0;
    for (double x : h) {
        const double t = s + x;
        comp += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    *out = (mode == 0) ? (s + comp) * dv : (s + comp);  // mass: sum(c) dx dy dz; energy: dv inside
    return FIPI_OK;
}

fipi_status fields_mass(fipi_ctx* ctx, double* out) {
    if (ctx->prec == FIPI_MIXED) {
        double k0h[4];
        FIPI_CUDA(ctx, cudaMemcpyAsync(k0h, ctx->k0, sizeof(k0h), cudaMemcpyDeviceToHost, ctx->stream));
        FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const fipi_params& P = ctx->P;
        *out = k0h[0] * ((P.lx / P.nx) * (P.ly / P.ny) * (P.lz / P.nz));
        return FIPI_OK;
    }
    return diag_t<double>(ctx, 0, out);
}

fipi_status fields_free_energy(fipi_ctx* ctx, double* out) {
    return ctx->prec == FIPI_MIXED ? diag_t<float>(ctx, 1, out) : diag_t<double>(ctx, 1, out);
}

// ------------------------------------------------------------ fine-grained
template <typename T> static fipi_status r2c_t(fipi_ctx* ctx, const double* in, double* out) {
    using C = cplx<T>;
    const Geom& g = ctx->g;
    T* tmp = (T*)ctx->fb.ureal;
    fipi_status st = upload<T>(ctx, in, tmp, (size_t)g.V);
    if (st != FIPI_OK) return st;
    OpR2C<T> op{tmp, F<T>::S(ctx, 0), g.nx, g.ny};
    launch_x<T, 0, 1, false>(ctx, "X forward", 1, NoAcc<OpR2C<T>>{op});
    void* sp[1] = {ctx->fb.S[0]};
    launch_y<T>(ctx, 1, sp, sp, -1);
    ZOpStore<T, 1> zs{{F<T>::S(ctx, 0)}, {F<T>::S(ctx, 1)}, 0};
    launch_z<T, 1, -1>(ctx, "Z forward store", 2, zs);
    FIPI_CUDA(ctx, cudaGetLastError());
    return download<T>(ctx, (const T*)F<T>::S(ctx, 1), out, (size_t)g.SH * 2);
    (void)sizeof(C);
}

fipi_status fields_fft_r2c(fipi_ctx* ctx, const double* in, double* out) {
    return ctx->prec == FIPI_MIXED ? r2c_t<float>(ctx, in, out) : r2c_t<double>(ctx, in, out);
}

template <typename T> static fipi_status c2r_t(fipi_ctx* ctx, const double* in, double* out) {
    const Geom& g = ctx->g;
    fipi_status st = upload<T>(ctx, in, (T*)F<T>::S(ctx, 0), (size_t)g.SH * 2);
    if (st != FIPI_OK) return st;
    ZOpStore<T, 1> zs{{F<T>::S(ctx, 0)}, {F<T>::S(ctx, 1)}, 0};
    launch_z<T, 1, +1>(ctx, "Z inverse copy", 2, zs);
    void* sp[1] = {ctx->fb.S[1]};
    launch_y<T>(ctx, 1, sp, sp, +1);
    T* dst = (T*)ctx->fb.ureal;
    OpC2RStore<T, 1> op{{F<T>::S(ctx, 1)}, {dst}, g.nx, g.ny};
    launch_x<T, 1, 0, false>(ctx, "X inverse store", 1, NoAcc<OpC2RStore<T, 1>>{op});
    FIPI_CUDA(ctx, cudaGetLastError());
    return download<T>(ctx, dst, out, (size_t)g.V);
}

fipi_status fields_fft_c2r(fipi_ctx* ctx, const double* in, double* out) {
    return ctx->prec == FIPI_MIXED ? c2r_t<float>(ctx, in, out) : c2r_t<double>(ctx, in, out);
}

template <typename T> static fipi_status grad_t(fipi_ctx* ctx, const double* c, double* out) {
    const Geom& g = ctx->g;
    T* tmp = (T*)ctx->fb.ureal;
    fipi_status st = upload<T>(ctx, c, tmp, (size_t)g.V);
    if (st != FIPI_OK) return st;
    OpR2C<T> op{tmp, F<T>::S(ctx, 0), g.nx, g.ny};
    launch_x<T, 0, 1, false>(ctx, "X forward", 1, NoAcc<OpR2C<T>>{op});
    void* sp[1] = {ctx->fb.S[0]};
    launch_y<T>(ctx, 1, sp, sp, -1);
    ZOpStore<T, 1> zs{{F<T>::S(ctx, 0)}, {F<T>::S(ctx, 0)}, 0};
    launch_z<T, 1, -1>(ctx, "Z forward store", 2, zs);
    T* g3[3] = {tmp, tmp + g.V, tmp + 2 * g.V};
    grad_from_chat<T>(ctx, F<T>::S(ctx, 0), g3);
    FIPI_CUDA(ctx, cudaGetLastError());
    return download<T>(ctx, tmp, out, (size_t)g.V * 3);
}

fipi_status fields_grad(fipi_ctx* ctx, const double* c, double* out) {
    return ctx->prec == FIPI_MIXED ? grad_t<float>(ctx, c, out) : grad_t<double>(ctx, c, out);
}

// field::div (field.cpp:332-361) + field::ifft, real part: the divergence
// of a real vector field.  The reference leaves the Nyquist index in; its
// contribution to the inverse transform is purely imaginary (i k_d at the
// self-conjugate Nyquist plane of d), so the real part equals the inverse
// with that plane zeroed, which is what the round-trip Z pass forms.
template <typename T> struct ZOpDivRt {
    using C = cplx<T>;
    const C* in[3];
    C* out;
    KTabs<T> kt;
    int m, ny2, nz2;
    __device__ const C* src(int f) const { return in[f]; }
    __device__ void prologue() const {}
    __device__ void load(int, int, int, size_t gi, C* v) const {
        v[0] = in[0][gi];
        v[1] = in[1][gi];
        v[2] = in[2][gi];
    }
    __device__ void mid(int ix, int iy, int iz, size_t, const C* vi, C* vo) const {
        const T k[3] = {ix == m ? T(0) : kt.kx[ix], iy == ny2 ? T(0) : kt.ky[iy], iz == nz2 ? T(0) : kt.kz[iz]};
        T re = T(0), im = T(0);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            re += -k[d] * vi[d].y;
            im += k[d] * vi[d].x;
        }
        vo[0] = mkc<C>(re, im);
    }
    __device__ void store2(int, int, int, size_t gi, const C* v) const { out[gi] = v[0]; }
    // register round trip (k_zpass_rr)
    struct State {
        C o;
    };
    __device__ void rr_mid(int ix, int iy, int iz, size_t gi, const C* w, State& st) const { mid(ix, iy, iz, gi, w, &st.o); }
    __device__ C rr_out(int, int, int, int, const State& st) const { return st.o; }
    __device__ void rr_store(int, size_t gi, C v) const { out[gi] = v; }
};

template <typename T> static fipi_status div_t(fipi_ctx* ctx, const double* v, double* out) {
    const Geom& g = ctx->g;
    T* tmp = (T*)ctx->fb.ureal;
    fipi_status st = upload<T>(ctx, v, tmp, (size_t)g.V * 3);
    if (st != FIPI_OK) return st;
    OpR2CN<T, 3> op{{tmp, tmp + g.V, tmp + 2 * g.V}, {F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2)}, g.nx, g.ny};
    launch_x<T, 0, 3, false>(ctx, "X forward", 3, NoAcc<OpR2CN<T, 3>>{op});
    void* s3[3] = {ctx->fb.S[0], ctx->fb.S[1], ctx->fb.S[2]};
    launch_y<T>(ctx, 3, s3, s3, -1);
    ZOpDivRt<T> zd{{F<T>::S(ctx, 0), F<T>::S(ctx, 1), F<T>::S(ctx, 2)}, F<T>::S(ctx, 3), F<T>::ktabs(ctx), g.m,
                   g.ny / 2, g.nz / 2};
    launch_zrt<T, 3, 1, -1, 16 / (sizeof(T) / 4), false>(ctx, "Z forward + div + inverse", 4, zd);
    void* s1[1] = {ctx->fb.S[3]};
    launch_y<T>(ctx, 1, s1, s1, +1);
    OpC2RStore<T, 1> oc{{F<T>::S(ctx, 3)}, {tmp}, g.nx, g.ny};
    launch_x<T, 1, 0, false>(ctx, "X inverse store", 1, NoAcc<OpC2RStore<T, 1>>{oc});
    FIPI_CUDA(ctx, cudaGetLastError());
    return download<T>(ctx, tmp, out, (size_t)g.V);
}

fipi_status fields_div(fipi_ctx* ctx, const double* v, double* out) {
    return ctx->prec == FIPI_MIXED ? div_t<float>(ctx, v, out) : div_t<double>(ctx, v, out);
}

const void* fields_real_c(fipi_ctx* ctx) { return ctx->fb.c; }
const void* fields_real_grad(fipi_ctx* ctx, int d) { return ctx->fb.g[d]; }

}  // namespace fipi
