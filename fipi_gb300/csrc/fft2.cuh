// Shared-memory row FFT with radix-16 register codelets (sm_103a).
//
// A row of N = 2^L complex values is transformed by Tn = N/E threads that
// hold E = min(EM, N) values each (EM = 16 or 8, chosen per pass: FftPlan,
// smem_fft2's EM parameter).  Stages follow the Stockham autosort
// recursion: with p the length of the sub-transforms already done, the
// group g of a stage of radix R reads x[g + m N/R] (m < R), multiplies by
// W_{Rp}^{m (g mod p)}, does a DFT-R in registers and writes
// y[(g - g mod p) R + g mod p + j p] (j < R).  Forward plans start with
// radix E and inverse plans end with it, so N = 256 takes two radix-16
// stages (one shared-memory exchange instead of the eight barriers of a
// radix-4 pass).  Where rows live in shared memory is given by an index
// functor, so each pass picks a bank-conflict-free layout.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace fipi {

// a * w, or a * conj(w) for the inverse direction
template <int DIR, typename C> __device__ __forceinline__ C mulw(C a, C w) {
    return DIR < 0 ? mkc<C>(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x)
                   : mkc<C>(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}

// cos(2 pi e / 16) for e in [0, 16)
__host__ __device__ constexpr double cos16(int e) {
    return e == 0 ? 1.0 : e == 1 ? 0.92387953251128675613 : e == 2 ? 0.70710678118654752440
         : e == 3 ? 0.38268343236508977173 : e == 4 ? 0.0 : e == 5 ? -0.38268343236508977173
         : e == 6 ? -0.70710678118654752440 : e == 7 ? -0.92387953251128675613 : e == 8 ? -1.0
         : e == 9 ? -0.92387953251128675613 : e == 10 ? -0.70710678118654752440
         : e == 11 ? -0.38268343236508977173 : e == 12 ? 0.0 : e == 13 ? 0.38268343236508977173
         : e == 14 ? 0.70710678118654752440 : 0.92387953251128675613;
}

// a * exp(DIR 2 pi i e / 16) for a compile-time e in [0, 16).
template <int DIR, int E16, typename C> __device__ __forceinline__ C tw16(C a) {
    using T = decltype(a.x);
    constexpr int e = E16 & 15;
    if constexpr (e == 0) return a;
    else if constexpr (e == 4) return cmul_i(a, DIR);
    else if constexpr (e == 8) return mkc<C>(-a.x, -a.y);
    else if constexpr (e == 12) return cmul_i(a, -DIR);
    else {
        // exp(DIR 2 pi i e/16): forward (DIR < 0) uses (cos, -sin)
        constexpr double cs = cos16(e), sn = cos16((e + 12) & 15);  // sin(x) = cos(x - pi/2)
        const T wr = (T)cs, wi = (T)(DIR < 0 ? -sn : sn);
        return mkc<C>(a.x * wr - a.y * wi, a.x * wi + a.y * wr);
    }
}

template <int DIR, typename C> __device__ __forceinline__ void dft2(C& a, C& b) {
    const C t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <int DIR, typename C> __device__ __forceinline__ void dft4(C& u0, C& u1, C& u2, C& u3) {
    const C a0 = cadd(u0, u2), a1 = csub(u0, u2), a2 = cadd(u1, u3);
    const C a3 = cmul_i(csub(u1, u3), DIR);
    u0 = cadd(a0, a2);
    u1 = cadd(a1, a3);
    u2 = csub(a0, a2);
    u3 = csub(a1, a3);
}

// natural order in and out
template <int DIR, typename C> __device__ __forceinline__ void dft8(C* v) {
    C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<DIR>(e0, e1, e2, e3);
    dft4<DIR>(o0, o1, o2, o3);
    o1 = tw16<DIR, 2>(o1);
    o2 = tw16<DIR, 4>(o2);
    o3 = tw16<DIR, 6>(o3);
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}

// 16 = 4 x 4: A[n1][k2] = DFT4_n2 x[n1 + 4 n2]; A *= W16^(n1 k2); X[k2 + 4 k1] = DFT4_n1 A[n1][k2]
template <int DIR, typename C> __device__ __forceinline__ void dft16(C* v) {
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) dft4<DIR>(v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]);
    // v[n1 + 4 k2] = A[n1][k2]
    v[1 + 4] = tw16<DIR, 1>(v[1 + 4]);
    v[1 + 8] = tw16<DIR, 2>(v[1 + 8]);
    v[1 + 12] = tw16<DIR, 3>(v[1 + 12]);
    v[2 + 4] = tw16<DIR, 2>(v[2 + 4]);
    v[2 + 8] = tw16<DIR, 4>(v[2 + 8]);
    v[2 + 12] = tw16<DIR, 6>(v[2 + 12]);
    v[3 + 4] = tw16<DIR, 3>(v[3 + 4]);
    v[3 + 8] = tw16<DIR, 6>(v[3 + 8]);
    v[3 + 12] = tw16<DIR, 9>(v[3 + 12]);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) dft4<DIR>(v[4 * k2], v[4 * k2 + 1], v[4 * k2 + 2], v[4 * k2 + 3]);
    // v[4 k2 + k1] = X[k2 + 4 k1]: transpose 4 x 4
    C o[16];
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2)
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) o[k2 + 4 * k1] = v[4 * k2 + k1];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = o[i];
}

template <int R, int DIR, typename C> __device__ __forceinline__ void dft_r(C* v) {
    if constexpr (R == 2) dft2<DIR>(v[0], v[1]);
    else if constexpr (R == 4) dft4<DIR>(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 8) dft8<DIR>(v);
    else dft16<DIR>(v);
}

// Row element -> shared-memory offset.
struct IdxPadded {  // rows contiguous, one pad slot per 16 elements
    int pitch;
    __device__ __forceinline__ int operator()(int row, int e) const { return row * pitch + e + (e >> 4); }
};
struct IdxColumns {  // element e of column `row` at e*cols + row (column index fastest)
    int cols;
    __device__ __forceinline__ int operator()(int row, int e) const { return e * cols + row; }
};
__host__ __device__ __forceinline__ int padded_len(int n) { return n + (n >> 4); }

// Default elements per thread (radix <= 8): keeps the pass kernels near 64
// registers, so several blocks share an SM; the FP32 Y and Z passes take 16
// (YE, zrt_elems).
template <typename T> struct FftE {
    static constexpr int value = 8;
};
template <typename T> __host__ __device__ inline int fft_threads_per_row(int n) {
    return n / (n < FftE<T>::value ? n : FftE<T>::value);
}

// Compile-time plan of an N-point transform with at most EM values per
// thread: forward radices are E = min(EM, N) first, then EM's, then the
// remainder; the inverse plan is the forward one reversed.
template <int N, int EM> struct FftPlan {
    static constexpr int E = N < EM ? N : EM;
    static constexpr int Tn = N / E;
    static constexpr int rfwd(int s) {
        if (s == 0) return E;
        int rest = N / E;
        for (int i = 1; i < s; ++i) rest /= (rest >= EM ? EM : rest);
        return rest >= EM ? EM : rest;
    }
    static constexpr int count() {
        int c = 1;
        for (int rest = N / E; rest > 1; rest /= (rest >= EM ? EM : rest)) ++c;
        return c;
    }
    static constexpr int NS = count();
    static constexpr int radix(int s, int dir) { return dir < 0 ? rfwd(s) : rfwd(NS - 1 - s); }
};

// One Stockham stage of radix R (compile-time N, p) for the row owned by
// (row, t); E/R groups per thread.  With IN the stage's inputs are already
// in v (slot q*R + m holds element g + m N/R, g = t + Tn q); with OUT its
// outputs stay in v (slot q*R + j holds element (g - k) R + k + j p).
// Barrier between the reads and the writes of a stage: the whole block, or
// only the warp when every row is owned by the lanes of one warp (WS).
template <bool WS> __device__ __forceinline__ void stage_sync() {
    if constexpr (WS) __syncwarp();
    else __syncthreads();
}

template <typename T, int R, int DIR, int N, int P, bool IN, bool OUT, int EM, bool WS, class Idx>
__device__ __forceinline__ void fft_stage(cplx<T>* s, const Idx& idx, int row, int t, bool act,
                                          const cplx<T>* __restrict__ tw, int ts, cplx<T>* v) {
    using PL = FftPlan<N, EM>;
    constexpr int G = PL::E / R;
    constexpr int NR = N / R;
    if constexpr (!IN) {
        if (act) {
#pragma unroll
            for (int q = 0; q < G; ++q) {
                const int g = t + PL::Tn * q;
#pragma unroll
                for (int m = 0; m < R; ++m) v[q * R + m] = s[idx(row, g + m * NR)];
            }
        }
        stage_sync<WS>();
    }
    if (act) {
#pragma unroll
        for (int q = 0; q < G; ++q) {
            const int g = t + PL::Tn * q;
            const int k = g & (P - 1);
            if constexpr (P > 1) {
                const int base = (NR / P) * k * ts;
#pragma unroll
                for (int m = 1; m < R; ++m) v[q * R + m] = mulw<DIR>(v[q * R + m], tw[m * base]);
            }
            dft_r<R, DIR>(&v[q * R]);
            if constexpr (!OUT) {
                const int o = (g - k) * R + k;
#pragma unroll
                for (int j = 0; j < R; ++j) s[idx(row, o + j * P)] = v[q * R + j];
            }
        }
    }
    if constexpr (!OUT) stage_sync<WS>();
}

template <typename T, int DIR, int N, int S, int P, bool IN, bool OUT, int EM, bool WS, class Idx>
__device__ __forceinline__ void fft_stages(cplx<T>* s, const Idx& idx, int row, int t, bool act,
                                           const cplx<T>* __restrict__ tw, int ts, cplx<T>* v) {
    using PL = FftPlan<N, EM>;
    if constexpr (S < PL::NS) {
        constexpr int R = PL::radix(S, DIR);
        fft_stage<T, R, DIR, N, P, IN && S == 0, OUT && S == PL::NS - 1, EM, WS>(s, idx, row, t, act, tw, ts, v);
        fft_stages<T, DIR, N, S + 1, P * R, IN, OUT, EM, WS>(s, idx, row, t, act, tw, ts, v);
    }
}

// Element indices of the register slots of the first stage (inputs) and
// of the last stage (outputs) for thread t of a row.
template <typename T, int DIR, int N, int EM = FftE<T>::value> struct FftIO {
    using PL = FftPlan<N, EM>;
    static constexpr int E = PL::E;
    static constexpr int R0 = PL::radix(0, DIR);
    static constexpr int RL = PL::radix(PL::NS - 1, DIR);
    __device__ static __forceinline__ int in_elem(int t, int slot) {
        return t + PL::Tn * (slot / R0) + (slot % R0) * (N / R0);
    }
    __device__ static __forceinline__ int out_elem(int t, int slot) {
        return t + PL::Tn * (slot / RL) + (slot % RL) * (N / RL);
    }
};

// In-place N-point FFT of one row per participating thread group, held in
// shared memory through `idx`.  tw[q*ts] = exp(-2 pi i q / N) for q < N.
// Every thread of the block must call it (it contains block barriers; with
// WS only warp barriers, for callers whose rows each lie within one warp,
// which then synchronise the block themselves where their own thread
// mapping changes).
// IN: the first stage's inputs are in v (FftIO::in_elem order) instead of
// shared memory; OUT: the results stay in v (FftIO::out_elem order).
template <typename T, int DIR, int N, bool IN = false, bool OUT = false, int EM = FftE<T>::value, bool WS = false,
          class Idx>
__device__ __forceinline__ void smem_fft2(cplx<T>* s, const Idx& idx, int row, int t, bool act,
                                          const cplx<T>* __restrict__ tw, int ts, cplx<T>* v) {
    fft_stages<T, DIR, N, 0, 1, IN, OUT, EM, WS>(s, idx, row, t, act, tw, ts, v);
}
template <typename T, int DIR, int N, int EM = FftE<T>::value, bool WS = false, class Idx>
__device__ __forceinline__ void smem_fft2(cplx<T>* s, const Idx& idx, int row, int t, bool act,
                                          const cplx<T>* __restrict__ tw, int ts) {
    cplx<T> v[FftPlan<N, EM>::E];
    fft_stages<T, DIR, N, 0, 1, false, false, EM, WS>(s, idx, row, t, act, tw, ts, v);
}

// Calls f(std::integral_constant<int, n>) for a power of two n in [8, 512].
template <class F> inline void dispatch_pow2(int n, F&& f) {
    switch (n) {
        case 4: f(std::integral_constant<int, 4>{}); break;
        case 8: f(std::integral_constant<int, 8>{}); break;
        case 16: f(std::integral_constant<int, 16>{}); break;
        case 32: f(std::integral_constant<int, 32>{}); break;
        case 64: f(std::integral_constant<int, 64>{}); break;
        case 128: f(std::integral_constant<int, 128>{}); break;
        case 256: f(std::integral_constant<int, 256>{}); break;
        default: f(std::integral_constant<int, 512>{}); break;
    }
}

}  // namespace fipi
