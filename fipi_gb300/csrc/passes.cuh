// Pass machinery shared by the forward step (fields.cu) and its adjoint
// (adjoint.cu): step constants, wave-number tables, the fused X pass
// kernel, the Z-pass operations both sides use, and the launchers of the
// X / Y / Z passes of the 3-pass R2C/C2R transforms.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <type_traits>

#include "ctx.hpp"

namespace fipi {

// ------------------------------------------------------------ constants
template <typename T> struct StepConsts {
    T lam_eps;    // lambda/sqr(epsilon)              main.cpp:81
    T lam;        // lambda
    T dt;
    T s1, s2;     // t = 0: dt*M, dt*M*lambda          main.cpp:106-113
    T s4, s2m;    // t > 0: 4 dt M, 2 dt M             main.cpp:118-119
    T s4c, s2c;   // 4 dt, 2 dt                        main.cpp:123-124
    T s3;         // 2 dt M lambda                     main.cpp:127
    T mu;
    T rho1, rho2, gravity;
    int ny2, nz2, m;  // Nyquist indices
};

template <typename T> StepConsts<T> make_consts(const fipi_ctx* ctx) {
    const fipi_params& P = ctx->P;
    StepConsts<T> k;
    const double dt = P.dt, M = P.mobility, lam = P.lambda;
    k.lam_eps = T(P.lambda / (P.epsilon * P.epsilon));
    k.lam = T(lam);
    k.dt = T(dt);
    k.s1 = T(dt * M);
    k.s2 = T(dt * M * lam);
    k.s4 = T(4.0 * dt * M);
    k.s2m = T(2.0 * dt * M);
    k.s4c = T(4.0 * dt);
    k.s2c = T(2.0 * dt);
    k.s3 = T(2.0 * dt * M * lam);
    k.mu = T(P.mu);
    k.rho1 = T(P.rho1);
    k.rho2 = T(P.rho2);
    k.gravity = T(P.gravity);
    k.ny2 = P.ny / 2;
    k.nz2 = P.nz / 2;
    k.m = P.nx / 2;
    return k;
}

template <typename T> struct KTabs {
    const T* kx;
    const T* ky;
    const T* kz;
    __device__ __forceinline__ T k2(int ix, int iy, int iz) const {
        const T a = kx[ix], b = ky[iy], c = kz[iz];
        T s = a * a;
        s += b * b;
        s += c * c;
        return s;
    }
};

// ------------------------------------------------------------ block reduce
__device__ __forceinline__ double block_sum(double v) {
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        s = lane < nw ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    }
    return s;  // valid in thread 0
}

// X-pass tiles: rows of M complex pairs with one pad slot per 2^kXPad
// elements, the X_M slot at the end, an odd pitch (the transposed
// tile loads and stores walk rows).
constexpr int kXPad = 4;
struct IdxX {
    int pitch;
    __device__ __forceinline__ int operator()(int row, int e) const { return row * pitch + e + (e >> kXPad); }
};
__host__ __device__ inline int xpass_pitch(int M) {
    const int p = M + (M >> kXPad) + 1;
    return (p & 1) ? p : p + 1;
}

// C2R of NIN fields into real arrays dst[f].
template <typename T, int NIN> struct OpC2RStore {
    using C = cplx<T>;
    const C* src[NIN];
    T* dst[NIN];
    int nx, ny;
    __device__ const C* in(int f) const { return src[f]; }
    __device__ C* out(int) const { return nullptr; }
    __device__ void point(int z, int y, int n, C* v) const {
#pragma unroll
        for (int f = 0; f < NIN; ++f) reinterpret_cast<C*>(dst[f] + ((size_t)z * ny + y) * nx)[n] = v[f];
    }
};

// op.in(f) / op.out(f) for a run-time f through a chain of compile-time
// indices: indexing a kernel parameter's pointer array with a run-time
// value would copy the whole parameter to local memory.
template <int NF, class Op> __device__ __forceinline__ auto in_sel(const Op& op, int f) {
    auto p = op.in(0);
#pragma unroll
    for (int k = 1; k < NF; ++k)
        if (f == k) p = op.in(k);
    return p;
}
template <int NF, class Op> __device__ __forceinline__ auto out_sel(const Op& op, int f) {
    auto p = op.out(0);
#pragma unroll
    for (int k = 1; k < NF; ++k)
        if (f == k) p = op.out(k);
    return p;
}

// R2C of NF real fields.
template <typename T, int NF> struct OpR2CN {
    using C = cplx<T>;
    const T* src[NF];
    C* o[NF];
    int nx, ny;
    __device__ C* out(int f) const { return o[f]; }
    __device__ const C* in(int) const { return nullptr; }
    __device__ void point(int z, int y, int n, C* v) const {
        const size_t row = ((size_t)z * ny + y) * nx;
#pragma unroll
        for (int f = 0; f < NF; ++f) v[f] = reinterpret_cast<const C*>(src[f] + row)[n];
    }
};

// Adapter giving point() an accumulator when the op does not take one.
template <class Op> struct NoAcc {
    Op op;
    __device__ const auto* in(int f) const { return op.in(f); }
    __device__ auto* out(int f) const { return op.out(f); }
    template <class C, class A> __device__ void point(int z, int y, int n, C* v, A&) const { op.point(z, y, n, v); }
};

// The same access to the real inputs read straight from global memory.
// The rows are read-only for the whole launch, so they are read through the
// non-coherent path: the compiler may then issue a later point's loads
// ahead of an earlier point's global stores (which it would otherwise have
// to assume alias them).
template <typename T, int NRF> struct XGlobalRow {
    const T* p[NRF];
    size_t row;  // element offset of the row
    __device__ __forceinline__ cplx<T> get(int f, int n) const {
        return __ldg(reinterpret_cast<const cplx<T>*>(p[f] + row) + n);
    }
};

// Split processing of the half-length complex transforms of the X pass
// (N = 2M real points as M complex pairs), W_k = twx[k] = exp(-2 pi i k / N).
// Each thread keeps one k (its twiddles in registers) and walks rows; the
// self-paired k = M/2 of every row follows, one row per thread.
// C2R pre-processing: Z_k = (X_k + conj X_{M-k}) + i conj(W_k) (X_k - conj X_{M-k});
// only the real parts of X_0 and X_M enter.
template <typename T, int M, int ROWS, int NT, class Idx>
__device__ __forceinline__ void c2r_pre(cplx<T>* s, const Idx& idx, const cplx<T>* __restrict__ twx, int tid) {
    using C = cplx<T>;
    constexpr int HM = M / 2;
    constexpr int L = HM < NT ? HM : NT;  // lanes per row
    constexpr int RG = NT / L;            // rows in flight
    const int lane = tid % L, rg = tid / L;
    auto pair = [&](int row, int k, const C Wk, const C Wm) {
        const int km = M - k;
        const C Xk = s[idx(row, k)], Xm = s[idx(row, km)];
        const C A = cadd(Xk, cconj(Xm)), B = csub(Xk, cconj(Xm));
        const C A2 = cadd(Xm, cconj(Xk)), B2 = csub(Xm, cconj(Xk));
        s[idx(row, k)] = cadd(A, cmul_i(cmul(B, cconj(Wk)), +1));
        if (km != k) s[idx(row, km)] = cadd(A2, cmul_i(cmul(B2, cconj(Wm)), +1));
    };
    for (int k = lane; k < HM; k += L) {
        const C Wk = twx[k], Wm = twx[M - k];
        for (int row = rg; row < ROWS; row += RG) {
            if (k == 0) {
                const T a = s[idx(row, 0)].x, c = s[idx(row, M)].x;
                s[idx(row, 0)] = mkc<C>(a + c, a - c);
            } else {
                pair(row, k, Wk, Wm);
            }
        }
    }
    const C Wh = twx[HM];
    for (int row = tid; row < ROWS; row += NT) pair(row, HM, Wh, Wh);
}

// R2C post-processing: X_k = (E - i W_k D) / 2 with E = Z_k + conj Z_{M-k},
// D = Z_k - conj Z_{M-k}; X_0 and X_M from Z_0; X_M lands at index M.
template <typename T, int M, int ROWS, int NT, class Idx>
__device__ __forceinline__ void r2c_post(cplx<T>* s, const Idx& idx, const cplx<T>* __restrict__ twx, int tid) {
    using C = cplx<T>;
    constexpr int HM = M / 2;
    constexpr int L = HM < NT ? HM : NT;
    constexpr int RG = NT / L;
    const int lane = tid % L, rg = tid / L;
    auto pair = [&](int row, int k, const C Wk, const C Wm) {
        const int km = M - k;
        const C Zk = s[idx(row, k)], Zm = s[idx(row, km)];
        const C E1 = cadd(Zk, cconj(Zm)), D1 = csub(Zk, cconj(Zm));
        const C E2 = cadd(Zm, cconj(Zk)), D2 = csub(Zm, cconj(Zk));
        s[idx(row, k)] = cscale(csub(E1, cmul_i(cmul(Wk, D1), +1)), T(0.5));
        if (km != k) s[idx(row, km)] = cscale(csub(E2, cmul_i(cmul(Wm, D2), +1)), T(0.5));
    };
    for (int k = lane; k < HM; k += L) {
        const C Wk = twx[k], Wm = twx[M - k];
        for (int row = rg; row < ROWS; row += RG) {
            if (k == 0) {
                const C Z0 = s[idx(row, 0)];
                s[idx(row, 0)] = mkc<C>(Z0.x + Z0.y, T(0));
                s[idx(row, M)] = mkc<C>(Z0.x - Z0.y, T(0));
            } else {
                pair(row, k, Wk, Wm);
            }
        }
    }
    const C Wh = twx[HM];
    for (int row = tid; row < ROWS; row += NT) pair(row, HM, Wh, Wh);
}

template <int I, int N, class F> __device__ __forceinline__ void static_for(F&& f) {
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        static_for<I + 1, N>(f);
    }
}

// exp(-2 pi i j / (2E)) for j < E/2 (E = 4 or 8): an eighth of a turn or
// less, from the sixteenth-turn cosines (the product with j = 0 is exact).
template <typename T, int E> __device__ __forceinline__ cplx<T> xsplit_rot(int j) {
    static_assert(E == 4 || E == 8, "X-pass split twiddles: E = 4 or 8");
    const int e = j * (8 / E);
    const T c = e == 0 ? T(1) : e == 1 ? T(cos16(1)) : e == 2 ? T(cos16(2)) : T(cos16(3));
    const T sn = e == 0 ? T(0) : e == 1 ? T(cos16(3)) : e == 2 ? T(cos16(2)) : T(cos16(1));
    return mkc<cplx<T>>(c, -sn);
}
// The C2R split pre-processing of c2r_pre for one row by the Tn = M / E
// threads that transform it, in place in the tile (thread t takes the pairs
// k = t + Tn j, j < E/2, and thread 0 also the self-paired k = M/2), so a
// warp that owns whole rows needs no block barrier around it; used where
// the register form below does not fit the register budget (the streamed
// pass with three inputs).  Wt = twx[t]; the other twiddles follow by one
// rotation each: W_{t + Tn j} = W_t exp(-2 pi i j / (2E)) and
// W_{M-k} = -conj(W_k).
template <typename T, int M, int E, class Idx>
__device__ __forceinline__ void c2r_pre_row(cplx<T>* s, const Idx& idx, int row, int t, cplx<T> Wt) {
    using C = cplx<T>;
    constexpr int Tn = M / E, HM = M / 2;
    auto pair = [&](int k, const C Wk, const C Wm) {
        const int km = M - k;
        const C Xk = s[idx(row, k)], Xm = s[idx(row, km)];
        const C A = cadd(Xk, cconj(Xm)), B = csub(Xk, cconj(Xm));
        const C A2 = cadd(Xm, cconj(Xk)), B2 = csub(Xm, cconj(Xk));
        s[idx(row, k)] = cadd(A, cmul_i(cmul(B, cconj(Wk)), +1));
        if (km != k) s[idx(row, km)] = cadd(A2, cmul_i(cmul(B2, cconj(Wm)), +1));
    };
#pragma unroll 1
    for (int j = 0; j < E / 2; ++j) {
        const int k = t + Tn * j;
        const C Wk = cmul(Wt, xsplit_rot<T, E>(j));
        if (k == 0) {
            const T a = s[idx(row, 0)].x, c = s[idx(row, M)].x;
            s[idx(row, 0)] = mkc<C>(a + c, a - c);
        } else {
            pair(k, Wk, mkc<C>(-Wk.x, Wk.y));
        }
    }
    if (t == 0) pair(HM, mkc<C>(T(0), T(-1)), mkc<C>(T(0), T(-1)));
}
// Split processing between the tile and a row's FFT registers, for rows
// owned by the Tn = M / E lanes of one warp.  Lane t holds the modes
// k = t + Tn j (j < E): the input set of the inverse transform's first
// stage and the output set of the forward transform's last stage.
// Twiddles: W_{t + Tn j} = W_t exp(-2 pi i j / (2E)) from Wt = twx[t].
template <typename T> __device__ __forceinline__ cplx<T> shfl_c(cplx<T> v, int src) {
    return mkc<cplx<T>>(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
// slot of mode t + Tn j in a stage's register order (first stage of radix R:
// slot = q R + m holds t + Tn q + m M / R)
template <int E, int R> constexpr int xslot_of_j(int j) {
    return (j % (E / R)) * R + j / (E / R);
}
// C2R pre-processing straight into v (the inverse plan's first-stage
// order): Z_k = (X_k + conj X_{M-k}) + i conj(W_k) (X_k - conj X_{M-k}),
// both modes read from the tile (M - k = M for k = 0: the X_M slot); Z_0
// from the real parts of X_0 and X_M.  Reads the tile only.
template <typename T, int M, int E, class Idx>
__device__ __forceinline__ void c2r_pre_regs(const cplx<T>* s, const Idx& idx, int row, int t, cplx<T> Wt,
                                             cplx<T>* v) {
    using C = cplx<T>;
    constexpr int Tn = M / E;
    constexpr int R0 = FftPlan<M, E>::radix(0, +1);
    static_for<0, E>([&](auto JC) {
        constexpr int j = decltype(JC)::value;
        const int k = t + Tn * j;
        const C xk = s[idx(row, k)], xm = s[idx(row, M - k)];
        const C Wk = tw16<-1, (8 * j) / E>(Wt);
        const C A = cadd(xk, cconj(xm)), B = csub(xk, cconj(xm));
        C z = cadd(A, cmul_i(cmul(B, cconj(Wk)), +1));
        if constexpr (j == 0)
            if (t == 0) z = mkc<C>(xk.x + xm.x, xk.x - xm.x);
        v[xslot_of_j<E, R0>(j)] = z;
    });
}
// R2C post-processing from v (the forward plan's last-stage order) into the
// tile: X_k = (E - i W_k D) / 2 with E = Z_k + conj Z_{M-k}, D = Z_k - conj
// Z_{M-k}; X_0 and X_M from Z_0.  The partner mode M - k = (Tn - t) +
// Tn (E - 1 - j) is held by lane (Tn - t) mod Tn of the same row and arrives
// by shuffle; lane 0 pairs k = Tn j with its own j' = E - j.  The warp's
// lanes finish reading the tile (the last FFT stage) before any writes.
template <typename T, int M, int E, class Idx>
__device__ __forceinline__ void r2c_post_regs(cplx<T>* s, const Idx& idx, int row, int t, cplx<T> Wt,
                                              const cplx<T>* v) {
    using C = cplx<T>;
    constexpr int Tn = M / E;
    constexpr int RL = FftPlan<M, E>::radix(FftPlan<M, E>::NS - 1, -1);
    const int lane = threadIdx.x & 31;
    const int src = (lane & ~(Tn - 1)) | ((Tn - t) & (Tn - 1));
    __syncwarp();
    static_for<0, E>([&](auto JC) {
        constexpr int j = decltype(JC)::value;
        const C zk = v[xslot_of_j<E, RL>(j)];
        C zm = shfl_c<T>(v[xslot_of_j<E, RL>(E - 1 - j)], src);
        if constexpr (j > 0)
            if (t == 0) zm = v[xslot_of_j<E, RL>(E - j)];
        const C Wk = tw16<-1, (8 * j) / E>(Wt);
        const C Ev = cadd(zk, cconj(zm)), D = csub(zk, cconj(zm));
        C x = cscale(csub(Ev, cmul_i(cmul(Wk, D), +1)), T(0.5));
        if constexpr (j == 0)
            if (t == 0) {
                x = mkc<C>(zk.x + zk.y, T(0));
                s[idx(row, M)] = mkc<C>(zk.x - zk.y, T(0));
            }
        s[idx(row, t + Tn * j)] = x;
    });
}

// X pass: one block = TY consecutive rows y0..y0+TY-1 of plane z, NIN
// spectral inputs (transposed runs of TY along y, C2R) and NOUT spectral
// outputs (R2C, transposed store); point() does the fused real-space work
// and may accumulate an FP64 per-block sum.  Rows of M = nx/2 complex pairs
// live in shared memory with one pad slot per 16 (pitch odd, so the
// transposed column accesses are conflict-free); X_M sits at index M.
// Blocks per SM the register budget is set for: FP32 4 (3 with four
// fields), FP64 3 (2).  512-thread blocks measured slower.
// Rows per X-pass tile: 16 FP32 rows (8 FP64) keep 128-byte runs along y;
// FP32 rows of 512 points take 8 so that the tile of four fields fits
// three blocks per SM.
__host__ __device__ constexpr int x_rows_of(int elem_bytes, int m) {
    return elem_bytes == 4 ? (m >= 256 ? 8 : 16) : 8;
}
template <typename T, int M> constexpr int x_rows = x_rows_of(sizeof(T), M);

// The FFT rows of an X pass lie within one warp each (Tn = M / E <= 32
// threads per row, rows of consecutive threads), so the stages between the
// split processing steps synchronise the warp only; the block synchronises
// where the thread mapping changes (tile loads, split processing, point
// loop, tile stores).
constexpr bool kXWarpSync = true;

// Elements per thread (radix of the register codelets) of the X pass.
template <typename T, int NIN, int NOUT> constexpr int x_elems = FftE<T>::value;

template <typename T, int NF, int NT> struct XMinBlocks {
    static constexpr int value = sizeof(T) == 4 ? (NF <= 3 ? 4 : 3) : (NF <= 3 ? 3 : 2);
};

// op.prefetch_rows(z, y0, rows): L2 prefetches of the real rows the point
// operation reads, issued by one thread with the tile loads.
template <class O, class = void> struct HasRowPrefetch : std::false_type {};
template <class O>
struct HasRowPrefetch<O, std::void_t<decltype(std::declval<const O&>().prefetch_rows(0, 0, 0))>> : std::true_type {};

template <typename T, int NIN, int NOUT, bool REDUCE, int M, class Op, int NT = kThreads>
__global__ void __launch_bounds__(NT, XMinBlocks<T, (NIN > NOUT ? NIN : NOUT), NT>::value)
    k_xpass_acc(Geom g, const cplx<T>* __restrict__ twx, Op op, double* partials) {
    using C = cplx<T>;
    constexpr int TY = x_rows<T, M>;
    constexpr int NF = NIN > NOUT ? NIN : NOUT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    constexpr int H = M + 1;
    const IdxX idx{xpass_pitch(M)};
    const int z = blockIdx.y, y0 = blockIdx.x * TY;
    const int tid = threadIdx.x;
    constexpr int EM = x_elems<T, NIN, NOUT>;
    constexpr int Tn = FftPlan<M, EM>::Tn;
    constexpr int rpr = NT / Tn;  // row FFTs per round
    // WL: one round covers the TY rows of a field, so every row of every
    // field belongs to one warp from the split processing through the
    // point loop; the block synchronises only after each field's tile
    // load and before the tile stores
    constexpr bool WL = kXWarpSync && TY * Tn == NT && M >= 32;
    // Loads and stores walk the tile field by field with ty fastest (a
    // run of TY along y per kx): each thread keeps one ty and steps kx.
    constexpr int KS = NT / TY;
    const int tyl = tid % TY, kx0 = tid / TY;
    const size_t gbase = (size_t)z * H * g.ny + y0 + tyl;
    const int rrow = tid / Tn, rt = tid % Tn;  // WL: the row of a field this thread transforms
    C Wt{};
    if constexpr (WL) Wt = twx[rt];
    if constexpr (NIN > 0) {
        // every element of the tile is requested before any is waited for,
        // one cp.async group per field
#pragma unroll
        for (int f = 0; f < NIN; ++f) {
            const C* src = op.in(f) + gbase;
            for (int kx = kx0; kx < H; kx += KS) cp_async<sizeof(C)>(&s[idx(f * TY + tyl, kx)], src + (size_t)kx * g.ny);
            cp_async_commit();
        }
        if constexpr (HasRowPrefetch<Op>::value)
            if (tid == 0) op.prefetch_rows(z, y0, TY);
        if constexpr (WL) {
#pragma unroll
            for (int f = 0; f < NIN; ++f) {
                cp_async_wait_pending(NIN - 1 - f);
                __syncthreads();
                C* sf = s + (size_t)f * TY * idx.pitch;
                C v[EM];
                c2r_pre_regs<T, M, EM>(sf, idx, rrow, rt, Wt, v);
                __syncwarp();  // the row is read before the first stage writes it
                smem_fft2<T, +1, M, true, false, EM, true>(sf, idx, rrow, rt, true, twx, 2, v);
            }
        } else if constexpr (TY % rpr == 0) {
            // FFT rounds align with fields: field f is pre-processed and
            // transformed while the later fields are still in flight
#pragma unroll
            for (int f = 0; f < NIN; ++f) {
                cp_async_wait_pending(NIN - 1 - f);
                __syncthreads();
                C* sf = s + (size_t)f * TY * idx.pitch;
                c2r_pre<T, M, TY, NT>(sf, idx, twx, tid);
                __syncthreads();
                for (int r0 = 0; r0 < TY; r0 += rpr)
                    smem_fft2<T, +1, M, EM, kXWarpSync>(sf, idx, r0 + tid / Tn, tid % Tn, true, twx, 2);
            }
        } else {
            cp_async_wait_all();
            __syncthreads();
            c2r_pre<T, M, NIN * TY, NT>(s, idx, twx, tid);
            __syncthreads();
            for (int r0 = 0; r0 < NIN * TY; r0 += rpr) {
                const int row = r0 + tid / Tn;
                smem_fft2<T, +1, M, EM, kXWarpSync>(s, idx, row, tid % Tn, row < NIN * TY, twx, 2);
            }
        }
        if constexpr (kXWarpSync && !WL) __syncthreads();  // the point loop walks rows across warps
    }
    const T invV = T(1) / T(g.V);
    T acc = T(0);  // per-thread partial sum in the arithmetic type (FP64 only per block)
    auto point = [&](int ty, int n) {
        C v[NF];
#pragma unroll
        for (int f = 0; f < NIN; ++f) v[f] = cscale(s[idx(f * TY + ty, n)], invV);
        op.point(z, y0 + ty, n, v, acc);
#pragma unroll
        for (int f = 0; f < NOUT; ++f) s[idx(f * TY + ty, n)] = v[f];
    };
    if constexpr (WL) {
        // the warp's own rows, 32 consecutive x pairs per step (coalesced
        // global accesses of the point operation)
        constexpr int RPW = 32 / Tn;
        const int lane = tid & 31, w = tid >> 5;
#pragma unroll
        for (int r = 0; r < RPW; ++r)
#pragma unroll
            for (int n0 = 0; n0 < M; n0 += 32) point(w * RPW + r, n0 + lane);
    } else {
        for (int i = tid; i < TY * M; i += NT) point(i / M, i % M);
    }
    if constexpr (REDUCE) {
        const double bs = block_sum((double)acc);
        if (tid == 0) partials[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = bs;
    }
    if constexpr (WL) __syncwarp();
    else __syncthreads();
    if constexpr (NOUT > 0) {
        if constexpr (WL) {
#pragma unroll
            for (int f = 0; f < NOUT; ++f) {
                C v[EM];
                smem_fft2<T, -1, M, false, true, EM, true>(s, idx, f * TY + rrow, rt, true, twx, 2, v);
                r2c_post_regs<T, M, EM>(s, idx, f * TY + rrow, rt, Wt, v);
            }
        } else {
            for (int r0 = 0; r0 < NOUT * TY; r0 += rpr) {
                const int row = r0 + tid / Tn;
                smem_fft2<T, -1, M, EM, kXWarpSync>(s, idx, row, tid % Tn, row < NOUT * TY, twx, 2);
            }
            if constexpr (kXWarpSync) __syncthreads();  // the split post-processing walks rows across warps
            r2c_post<T, M, NOUT * TY, NT>(s, idx, twx, tid);
        }
        __syncthreads();
#pragma unroll
        for (int f = 0; f < NOUT; ++f) {
            C* dst = op.out(f) + gbase;
            for (int kx = kx0; kx < H; kx += KS) dst[(size_t)kx * g.ny] = s[idx(f * TY + tyl, kx)];
        }
    }
}

// X pass with the point operation on registers: one FFT round per field
// (TY rows x Tn threads = the block), the inverse transform of input f ends
// in registers (its last stage's modes), op.take<f> consumes them and, when
// op.emit_after(f) names an output d, returns that output's values, whose
// forward transform starts from the registers, exchanging through the tile
// of field d (already consumed).  Against k_xpass_acc this drops the point
// loop's shared-memory round trip and one exchange per field.  The op keeps
// a State per mode between the rounds; real-space rows it reads in take()
// come from global memory (op.prefetch_rows puts them in L2 at block start).
template <typename T, int M> struct XStreamShape {
    static constexpr int TY = x_rows<T, M>;
    static constexpr int E = FftPlan<M, FftE<T>::value>::E;
    static constexpr int Tn = FftPlan<M, FftE<T>::value>::Tn;
    static constexpr int NT = TY * Tn;
    // blocks per SM the register budget is set for: three (two in FP64)
    // 256-thread blocks' worth (the State of a mode stays live across
    // rounds); a single field five (48 registers) for rows of up to 128
    // pairs, four for longer rows (which spill at 48)
    template <int NF> static constexpr int minb() {
        const int b = (sizeof(T) == 4 ? (NF == 1 ? (M <= 128 ? 5 : 4) : 3) : 2) * 256 / NT;
        return b < 1 ? 1 : (b > 8 ? 8 : b);
    }
};

template <typename T, int NIN, int NOUT, bool REDUCE, int M, class Op>
__global__ void __launch_bounds__(XStreamShape<T, M>::NT,
                                  XStreamShape<T, M>::template minb<(NIN > NOUT ? NIN : NOUT)>())
    k_xpass_stream(Geom g, const cplx<T>* __restrict__ twx, Op op, double* partials) {
    using C = cplx<T>;
    using SH = XStreamShape<T, M>;
    constexpr int TY = SH::TY, E = SH::E, Tn = SH::Tn, NT = SH::NT;
    constexpr int NF = NIN > NOUT ? NIN : NOUT;
    constexpr int EM = FftE<T>::value;
    constexpr int H = M + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const IdxX idx{xpass_pitch(M)};
    const int z = blockIdx.y, y0 = blockIdx.x * TY;
    const int tid = threadIdx.x;
    {
        // one cp.async group per field; each round waits for its own field
        const int tyl = tid % TY, kx0 = tid / TY;
        const size_t gbase = (size_t)z * H * g.ny + y0 + tyl;
#pragma unroll
        for (int f = 0; f < NIN; ++f) {
            const C* src = op.in(f) + gbase;
            for (int kx = kx0; kx < H; kx += NT / TY) cp_async<sizeof(C)>(&s[idx(f * TY + tyl, kx)], src + (size_t)kx * g.ny);
            cp_async_commit();
        }
        if constexpr (HasRowPrefetch<Op>::value)
            if (tid == 0) op.prefetch_rows(z, y0, TY);
    }
    const int ty = tid / Tn, t = tid % Tn;
    using IO = FftIO<T, +1, M, EM>;
    // WL: a field's rows are pre-processed, transformed and post-processed
    // by the warp that owns them (no block barrier in between); rows of 512
    // points keep the block-wide split processing (the warp-local form
    // spills there at the three-blocks-per-SM register budget)
    constexpr bool WL = kXWarpSync && M >= 32 && M <= 128;
    // the pre-processing feeds the first FFT stage from registers for a
    // single input; with three inputs the State kept across rounds leaves no
    // room for it (it spills), so those rows are pre-processed in the tile
    constexpr bool PRE_REGS = WL && NIN == 1;
    const T invV = T(1) / T(g.V);
    T acc = T(0);
    typename Op::State st[E];
    static_for<0, NIN>([&](auto FC) {
        constexpr int f = decltype(FC)::value;
        C* sf = s + (size_t)f * TY * idx.pitch;
        cp_async_wait_pending(NIN - 1 - f);
        __syncthreads();
        C v[E];
        if constexpr (PRE_REGS) {
            c2r_pre_regs<T, M, EM>(sf, idx, ty, t, twx[t], v);  // twiddle read at use: no register held across rounds
            __syncwarp();  // the row is read before the first stage writes it
        } else if constexpr (WL) {
            c2r_pre_row<T, M, EM>(sf, idx, ty, t, twx[t]);
            __syncwarp();
        } else {
            c2r_pre<T, M, TY, NT>(sf, idx, twx, tid);
            __syncthreads();
        }
        smem_fft2<T, +1, M, PRE_REGS, true, EM, kXWarpSync>(s, idx, f * TY + ty, t, true, twx, 2, v);
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int n = IO::out_elem(t, i);
            v[i] = op.template take<f>(z, y0 + ty, n, cscale(v[i], invV), st[i], acc);
        }
        constexpr int d = Op::emit_after(f);
        if constexpr (d >= 0) {
            smem_fft2<T, -1, M, true, WL, EM, kXWarpSync>(s, idx, d * TY + ty, t, true, twx, 2, v);
            if constexpr (WL) r2c_post_regs<T, M, EM>(s, idx, d * TY + ty, t, twx[t], v);
        }
    });
    if constexpr (REDUCE) {
        const double bs = block_sum((double)acc);
        if (tid == 0) partials[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = bs;
    }
    __syncthreads();
    if constexpr (!WL) {
        r2c_post<T, M, NOUT * TY, NT>(s, idx, twx, tid);
        __syncthreads();
    }
    const int tyl = tid % TY, kx0 = tid / TY;
    const size_t gbase = (size_t)z * H * g.ny + y0 + tyl;
#pragma unroll
    for (int f = 0; f < NOUT; ++f) {
        C* dst = op.out(f) + gbase;
        for (int kx = kx0; kx < H; kx += NT / TY) dst[(size_t)kx * g.ny] = s[idx(f * TY + tyl, kx)];
    }
}

// Z forward with the Leray projection (main.cpp:177-178) fused:
// u_hat = (F - k (k.F)/k^2) / (mu k^2), 0 at k = 0.  At modes with a Nyquist
// index the reference's C2C inverse keeps only the real part of a
// non-Hermitian spectrum; that equals the inverse of the average of the
// projections with k and with the Nyquist components of k negated, which is
// what is stored here (a Hermitian half spectrum).
template <typename T> struct ZOpProj {
    using C = cplx<T>;
    const C* in[3];
    C* out[3];
    __device__ const C* src(int f) const { return in[f]; }
    KTabs<T> kt;
    T mu;
    int m, ny2, nz2;
    __device__ void load(int, int, int, size_t gi, C* v) const {
        v[0] = in[0][gi];
        v[1] = in[1][gi];
        v[2] = in[2][gi];
    }
    __device__ static void project(const T* kv, T k2, T mk2, const C* F, C* u) {
        T dre = T(0), dim = T(0);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            dre += kv[d] * F[d].x;
            dim += kv[d] * F[d].y;
        }
        if constexpr (sizeof(T) == sizeof(float)) {
            // mixed form: two reciprocals instead of twelve divisions
            const T r1 = T(1) / k2, r2 = T(1) / mk2;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const T qre = (kv[d] * dre) * r1, qim = (kv[d] * dim) * r1;
                u[d] = mkc<C>((F[d].x - qre) * r2, (F[d].y - qim) * r2);
            }
        } else {
            // FP64: the reference's evaluation order (main.cpp:177-178)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const T qre = (kv[d] * dre) / k2, qim = (kv[d] * dim) / k2;
                u[d] = mkc<C>((F[d].x - qre) / mk2, (F[d].y - qim) / mk2);
            }
        }
    }
    __device__ void store(int ix, int iy, int iz, size_t gi, const C* F) const {
        C u[3];
        compute(ix, iy, iz, F, u);
        out[0][gi] = u[0];
        out[1][gi] = u[1];
        out[2][gi] = u[2];
    }
    __device__ void compute(int ix, int iy, int iz, const C* F, C* u) const {
        const T kv[3] = {kt.kx[ix], kt.ky[iy], kt.kz[iz]};
        const T k2 = kt.k2(ix, iy, iz);
        if (k2 == T(0)) {
            u[0] = u[1] = u[2] = mkc<C>(T(0), T(0));
        } else {
            const T mk2 = k2 * mu;
            project(kv, k2, mk2, F, u);
            const bool nx_ = ix == m, ny_ = iy == ny2, nz_ = iz == nz2;
            if (nx_ || ny_ || nz_) {
                const T ks[3] = {nx_ ? -kv[0] : kv[0], ny_ ? -kv[1] : kv[1], nz_ ? -kv[2] : kv[2]};
                C u2[3];
                project(ks, k2, mk2, F, u2);
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    u[d] = mkc<C>(T(0.5) * (u[d].x + u2[d].x), T(0.5) * (u[d].y + u2[d].y));
            }
        }
    }
};

// Z forward plain store; in the mixed form the k = 0 entry of c_hat is held
// in FP64 and zeroed in the FP32 array.
template <typename T, int NF> struct ZOpStore {
    using C = cplx<T>;
    const C* in[NF];
    C* out[NF];
    int zero_k0_mask;
    __device__ const C* src(int f) const { return in[f]; }
    __device__ void load(int, int, int, size_t gi, C* v) const {
#pragma unroll
        for (int f = 0; f < NF; ++f) v[f] = in[f][gi];
    }
    __device__ void store(int, int, int, size_t gi, const C* v) const {
#pragma unroll
        for (int f = 0; f < NF; ++f)
            out[f][gi] = (gi == 0 && ((zero_k0_mask >> f) & 1)) ? mkc<C>(T(0), T(0)) : v[f];
    }
};

template <typename Tin, typename Tout>
__global__ void k_convert(const Tin* __restrict__ a, Tout* __restrict__ b, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = (Tout)a[i];
}

// ------------------------------------------------------------ launch glue
template <typename T> struct F {
    using C = cplx<T>;
    static C* S(fipi_ctx* ctx, int i) { return (C*)ctx->fb.S[i]; }
    static C* sp(void* p) { return (C*)p; }
    static T* re(void* p) { return (T*)p; }
    static const C* tw(void* p) { return (const C*)p; }
    static KTabs<T> ktabs(fipi_ctx* ctx) {
        return KTabs<T>{(const T*)ctx->fb.kx, (const T*)ctx->fb.ky, (const T*)ctx->fb.kz};
    }
};

// nreal: real (V-sized) arrays the fused point operation reads or writes.
// One block per tile of x_rows<T, M> rows; NT threads per block.
template <typename T, int NIN, int NOUT, bool REDUCE, class Op, int NT = kThreads>
void launch_x(fipi_ctx* ctx, const char* name, int nreal, const Op& op, double* partials = nullptr) {
    const Geom& g = ctx->g;
    LaunchScope ls(ctx, name,
                   (double)(NIN + NOUT) * g.SH * sizeof(cplx<T>) + (double)nreal * g.V * sizeof(T));
    constexpr int NF = NIN > NOUT ? NIN : NOUT;
    dispatch_pow2(g.m, [&](auto MC) {
        constexpr int M = decltype(MC)::value;
        constexpr int TY = x_rows<T, M>;
        const size_t smem = (size_t)NF * TY * xpass_pitch(g.m) * sizeof(cplx<T>);
        dim3 grid(g.ny / TY, g.nz);
        auto kern = k_xpass_acc<T, NIN, NOUT, REDUCE, M, Op, NT>;
        static size_t granted = 48 * 1024;
        ensure_smem(kern, smem, granted);
        kern<<<grid, NT, smem, ctx->stream>>>(g, (const cplx<T>*)ctx->fb.twx, op, partials);
    });
}

// FP32: k_xpass_stream (ops with take) for rows up to 256 points; otherwise
// and in FP64: k_xpass_acc.  The force pass stays on k_xpass_acc (measured
// faster there: its streamed form holds mu and the force inputs across rounds).
template <typename T, int NIN, int NOUT, bool REDUCE, class Op>
void launch_xs(fipi_ctx* ctx, const char* name, int nreal, const Op& op, double* partials = nullptr) {
    if constexpr (sizeof(T) != sizeof(float)) {
        launch_x<T, NIN, NOUT, REDUCE>(ctx, name, nreal, op, partials);
    } else {
        const Geom& g = ctx->g;
        LaunchScope ls(ctx, name,
                       (double)(NIN + NOUT) * g.SH * sizeof(cplx<T>) + (double)nreal * g.V * sizeof(T));
        constexpr int NF = NIN > NOUT ? NIN : NOUT;
        dispatch_pow2(g.m, [&](auto MC) {
            constexpr int M = decltype(MC)::value;
            constexpr int TY = x_rows<T, M>;
            const size_t smem = (size_t)NF * TY * xpass_pitch(g.m) * sizeof(cplx<T>);
            dim3 grid(g.ny / TY, g.nz);
            if constexpr (XStreamShape<T, M>::NT <= kThreads) {
                auto kern = k_xpass_stream<T, NIN, NOUT, REDUCE, M, Op>;
                static size_t granted = 48 * 1024;
                ensure_smem(kern, smem, granted);
                kern<<<grid, XStreamShape<T, M>::NT, smem, ctx->stream>>>(g, (const cplx<T>*)ctx->fb.twx, op,
                                                                            partials);
            } else {  // rows of more than 256 points: one round per field would need > 256 threads
                auto kern = k_xpass_acc<T, NIN, NOUT, REDUCE, M, Op>;
                static size_t granted = 48 * 1024;
                ensure_smem(kern, smem, granted);
                kern<<<grid, kThreads, smem, ctx->stream>>>(g, (const cplx<T>*)ctx->fb.twx, op, partials);
            }
        });
    }
}

template <typename T> void launch_y(fipi_ctx* ctx, int nf, void* const* in, void* const* out, int dir) {
    const Geom& g = ctx->g;
    static const char* names[9] = {"Y pass x0", "Y pass x1", "Y pass x2", "Y pass x3", "Y pass x4",
                                   "Y pass x5", "Y pass x6", "Y pass x7", "Y pass x8"};
    LaunchScope ls(ctx, names[nf], 2.0 * nf * g.SH * sizeof(cplx<T>));
    FieldPtrs<T> fp{};
    for (int f = 0; f < nf; ++f) {
        fp.in[f] = (cplx<T>*)in[f];
        fp.out[f] = (cplx<T>*)out[f];
    }
    // persistent, TMA double-buffered: a grid of resident blocks walks all tiles
    const size_t smem = ypass_tma_smem<T>(g);
    dispatch_pow2(g.ny, [&](auto NC) {
        constexpr int N = decltype(NC)::value;
        auto kern = (dir < 0) ? k_ypass_tma<T, -1, N> : k_ypass_tma<T, +1, N>;
        static size_t granted[2] = {48 * 1024, 48 * 1024};
        static int blocks_per_sm[2] = {0, 0};
        const int di = dir < 0 ? 0 : 1;
        ensure_smem(kern, smem, granted[di]);
        if (!blocks_per_sm[di]) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm[di], kern, kThreads, smem);
            if (blocks_per_sm[di] < 1) blocks_per_sm[di] = 1;
        }
        const int rb = ypass_tile_rows<T>(g.ny);
        const long long tiles = ((long long)g.nz * g.h + rb - 1) / rb * nf;
        long long grid = (long long)ctx->num_sms * blocks_per_sm[di];
        if (grid > tiles) grid = tiles;
        kern<<<(unsigned)grid, kThreads, smem, ctx->stream>>>(g, (const cplx<T>*)ctx->fb.twy, fp, nf, ctx->status,
                                                              ctx->debug_first_wait);
    });
}

// nspec: spectral arrays the pass and its fused operation read or write.
template <typename T, int NF, int DIR, class Op> void launch_z(fipi_ctx* ctx, const char* name, int nspec, const Op& op) {
    const Geom& g = ctx->g;
    LaunchScope ls(ctx, name, (double)nspec * g.SH * sizeof(cplx<T>));
    const size_t smem = zpass_smem<T, NF>(g);
    dim3 grid(g.h, g.ny / zpass_cols<T>(g.nz));
    const int threads = zpass_threads<T>(g.nz);
    dispatch_pow2(g.nz, [&](auto NC) {
        constexpr int N = decltype(NC)::value;
        auto kern = k_zpass<T, NF, DIR, N, Op>;
        static size_t granted = 48 * 1024;
        ensure_smem(kern, smem, granted);
        kern<<<grid, threads, smem, ctx->stream>>>(g, (const cplx<T>*)ctx->fb.twz, op);
    });
}

// FP32 round trips that run as k_zpass_rr (measured faster there than the
// shared-memory tiles of k_zpass_rt / k_zpass_rt_t).
template <int NF, int NB> constexpr bool zrt_in_registers = (NF == 1 && NB == 4);
// Elements per thread (radix of the register codelets) of the Z round trips:
// 16 in FP32 (N = 256 in two stages, one shared-memory exchange; measured
// 10 % faster than radix 8 for the one-field round trips), 8 in FP64.
template <typename T, int NF, int NB> constexpr int zrt_elems = sizeof(T) == 4 ? 16 : 8;

// Round-trip Z pass: NF fields in, NB fields out; WIDE: k_zpass_rt with
// tiles of COLS ky columns (COLS <= 16 for FP32, whose grids have
// ny >= 16, and <= 8 for FP64, ny >= 8), else k_zpass_rt_t.
template <typename T, int NF, int NB, int DIR, int COLS, bool WIDE, class Op>
void launch_zrt(fipi_ctx* ctx, const char* name, int nspec, const Op& op) {
    const Geom& g = ctx->g;
    LaunchScope ls(ctx, name, (double)nspec * g.SH * sizeof(cplx<T>));
    constexpr int EM = zrt_elems<T, NF, NB>;
    if constexpr (sizeof(T) == sizeof(float) && zrt_in_registers<NF, NB>) {
        // FP32: the round trip held in registers
        dispatch_pow2(g.nz, [&](auto NC) {
            constexpr int N = decltype(NC)::value;
            using SHP = ZRtShapeT<T, N, 16, EM>;
            const size_t smem = (size_t)(HasAux<Op>::value ? 2 : 1) * SHP::TZ * N * sizeof(cplx<T>);
            dim3 grid(g.h, g.ny / SHP::TZ);
            auto kern = k_zpass_rr<T, NF, NB, DIR, N, 16, Op, EM>;
            static size_t granted = 48 * 1024;
            ensure_smem(kern, smem, granted);
            kern<<<grid, SHP::TZ * SHP::Tn, smem, ctx->stream>>>(g, (const cplx<T>*)ctx->fb.twz, op);
        });
        return;
    }
    if constexpr (!WIDE) {
        dispatch_pow2(g.nz, [&](auto NC) {
            constexpr int N = decltype(NC)::value;
            using SHP = ZRtShapeT<T, N, COLS, EM>;
            constexpr int NS = NF > NB ? NF : NB;
            const size_t smem = (size_t)NS * SHP::TZ * N * sizeof(cplx<T>);
            dim3 grid(g.h, g.ny / SHP::TZ);
            auto kern = k_zpass_rt_t<T, NF, NB, DIR, N, COLS, Op, EM>;
            static size_t granted = 48 * 1024;
            ensure_smem(kern, smem, granted);
            kern<<<grid, SHP::TZ * SHP::Tn, smem, ctx->stream>>>(g, (const cplx<T>*)ctx->fb.twz, op);
        });
        return;
    } else
    dispatch_pow2(g.nz, [&](auto NC) {
        constexpr int N = decltype(NC)::value;
        constexpr int NS = NF > NB ? NF : NB;
        // columns of 512 modes with three or more fields: half the tile (two blocks per SM)
        constexpr int CW = (N >= 512 && NS >= 3 && COLS > 8) ? COLS / 2 : COLS;
        using SHP = ZRtShape<T, N, CW, EM>;
        const size_t smem = (size_t)NS * SHP::FSTRIDE * sizeof(cplx<T>);
        dim3 grid(g.h, g.ny / CW);
        auto kern = k_zpass_rt<T, NF, NB, DIR, N, CW, Op, EM>;
        static size_t granted = 48 * 1024;
        ensure_smem(kern, smem, granted);
        kern<<<grid, SHP::THREADS, smem, ctx->stream>>>(g, (const cplx<T>*)ctx->fb.twz, op);
    });
}

// ------------------------------------------------------------ state I/O
// Copies host doubles into a T device array through a staging buffer.
template <typename T> inline fipi_status upload(fipi_ctx* ctx, const double* h, T* d, size_t n) {
    if (sizeof(T) == sizeof(double)) {
        FIPI_CUDA(ctx, cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        return FIPI_OK;
    }
    double* stage = nullptr;
    FIPI_CUDA(ctx, cudaMallocAsync((void**)&stage, n * sizeof(double), ctx->stream));
    FIPI_CUDA(ctx, cudaMemcpyAsync(stage, h, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    { LaunchScope ls(ctx, "convert", 0.0); k_convert<double, T><<<1024, 256, 0, ctx->stream>>>(stage, d, n); }
    FIPI_CUDA(ctx, cudaFreeAsync(stage, ctx->stream));
    return FIPI_OK;
}

template <typename T> inline fipi_status download(fipi_ctx* ctx, const T* d, double* h, size_t n) {
    if (sizeof(T) == sizeof(double)) {
        FIPI_CUDA(ctx, cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return FIPI_OK;
    }
    double* stage = nullptr;
    FIPI_CUDA(ctx, cudaMallocAsync((void**)&stage, n * sizeof(double), ctx->stream));
    { LaunchScope ls(ctx, "convert", 0.0); k_convert<T, double><<<1024, 256, 0, ctx->stream>>>(d, stage, n); }
    FIPI_CUDA(ctx, cudaMemcpyAsync(h, stage, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    FIPI_CUDA(ctx, cudaFreeAsync(stage, ctx->stream));
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return FIPI_OK;
}

}  // namespace fipi
