// 3-D real <-> half-spectrum FFT passes for sm_103a.
//
// Layouts (V = nz*ny*nx, H = nx/2 + 1, M = nx/2):
//   real field      R[z][y][x]        x fastest  (the reference's field layout,
//                                                 field.cpp:88-92)
//   spectral field  S[kz][kx][ky]     ky fastest, kx in [0, M]
//
// A forward transform is three passes, each one HBM read and one write of
// the array:
//   X (R2C along x, rows contiguous) -> writes S1[z][kx][y] through a
//       shared-memory transpose (runs of TY consecutive y per kx);
//   Y (C2C along contiguous rows of length ny);
//   Z (C2C along z for a tile of TZ consecutive ky at one kx).
// The inverse runs Z, Y, X(C2R).  Element-wise work is fused into the X
// passes (real space) and the Z passes (spectral space) through functors.
//
// The row FFT is an in-place radix-4 Stockham autosort in shared memory
// (one radix-2 stage first when log2 n is odd), four elements per thread
// per stage, twiddles from a table exp(-2 pi i q / n) computed on the host
// in extended precision.  An R2C row of length nx is a complex FFT of
// length M over (x[2n], x[2n+1]) pairs plus the standard split
// post-processing; C2R is the mirror image.  Unnormalised, like FFTW.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "fft2.cuh"
#include "tma.cuh"

namespace fipi {

struct Geom {
    int nx, ny, nz;
    int m, h;        // nx/2, nx/2 + 1
    int lm, ly, lz;  // log2 of m, ny, nz
    long long V;     // nx*ny*nz
    long long SH;    // nz*h*ny complex entries of a spectral field
};

constexpr int kThreads = 256;

// Tile sizes: 128-byte runs of the transposed dimension.
template <typename T> struct Tiles {
    static constexpr int TY = 128 / (2 * sizeof(T));  // 16 (fp32) / 8 (fp64)
    static constexpr int TZ = 128 / (2 * sizeof(T));
};

// A Z-pass operation that declares PreT and pre() has global reads in its
// mid operation that can be issued ahead (k_zpass_rt batches ZU modes; two
// measured fastest, more raise register pressure).
template <class O, class = void> struct HasPre : std::false_type {};
template <class O> struct HasPre<O, std::void_t<typename O::PreT>> : std::true_type {};
constexpr int ZU = 2;

// A register round trip (k_zpass_rr) whose mid operation reads one more
// spectral array declares aux() (that array); its tile is then staged in
// shared memory with cp.async and handed to rr_mid.
template <class O, class = void> struct HasAux : std::false_type {};
template <class O> struct HasAux<O, std::void_t<decltype(std::declval<const O&>().aux())>> : std::true_type {};

// A Z-pass operation whose load() only copies NF spectral arrays declares
// src(f) (the array of field f); its tiles are then fetched with cp.async.
template <class O, class = void> struct HasSrc : std::false_type {};
template <class O> struct HasSrc<O, std::void_t<decltype(std::declval<const O&>().src(0))>> : std::true_type {};

// ----------------------------------------------------------------- Y pass
template <typename T> struct FieldPtrs {
    cplx<T>* in[8];
    cplx<T>* out[8];
    // in[f] / out[f] for a run-time f without copying the parameter to local memory
    __device__ __forceinline__ cplx<T>* pick(cplx<T>* const (&a)[8], int f) const {
        cplx<T>* p = a[0];
#pragma unroll
        for (int k = 1; k < 8; ++k)
            if (f == k) p = a[k];
        return p;
    }
};

// Elements per thread of the Y pass: radix-16 register codelets in FP32
// (N = 256 in two stages, one shared-memory exchange), 8 in FP64.
template <typename T> struct YE {
    static constexpr int value = sizeof(T) == 4 ? 16 : 8;
};
// Rows per FFT round of a Y-pass block: 256 threads, N / min(N, YE) per row.
template <typename T> __host__ __device__ inline int ypass_rows(int ny) {
    return kThreads / (ny / (ny < YE<T>::value ? ny : YE<T>::value));
}

// Persistent Y pass: each block streams tiles of RB consecutive rows
// (RB * N contiguous complex values) into shared memory with one bulk TMA
// copy per tile through a ring of kYStages buffers, so kYStages - 1 tiles
// are in flight while one is transformed; the buffer a tile arrived in then
// serves as that tile's (padded) exchange buffer.  The first stage reads the
// tile, the last stage stores straight to global memory.  `fields` fields of
// rows are processed in one launch.
constexpr int kYStages = 2;  // 3 measured no faster on GB300 (more registers)
// FP32: three blocks per SM (<= 85 registers) measured 6 % faster than two
// with the radix-16 codelets; FP64 keeps two (its codelets need ~124).
// FFT rounds per Y tile (one: 16 FP32 or 8 FP64 rows of 256, 32 KB per copy).
template <typename T> struct YGroups {
    static constexpr int value = 1;
};

// first_wait: polls of the block's first copy wait (-1: the normal bound);
// a test hook that lets the bounded-wait error path run (fipi_set_debug).
template <typename T, int DIR, int N>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 3 : 2) k_ypass_tma(Geom g, const cplx<T>* __restrict__ twy, FieldPtrs<T> fp,
                                                       int fields, int* status, int first_wait) {
    using C = cplx<T>;
    constexpr int EM = YE<T>::value;
    using IO = FftIO<T, DIR, N, EM>;
    constexpr int S = kYStages;
    constexpr int Tn = FftPlan<N, EM>::Tn;
    constexpr int RG = kThreads / Tn;           // rows per FFT round (all threads)
    constexpr int G = YGroups<T>::value;        // rounds per tile: G * RG rows per bulk copy
    constexpr int RB = G * RG;
    constexpr int PITCH = (N + (N >> 4) + 15) & ~15;  // >= padded_len(N); 128-byte multiple for FP32/FP64
    constexpr int BUF = RB * PITCH;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* buf0 = reinterpret_cast<C*>(smem_raw);
    __shared__ __align__(8) uint64_t bar[S];
    __shared__ int abort_flag;
    const int tid = threadIdx.x;
    const long long rows_f = (long long)g.nz * g.h;
    const long long tiles_f = (rows_f + RB - 1) / RB;
    const long long ntiles = tiles_f * fields;
    const IdxPadded xidx{padded_len(N)};
    if (tid == 0) {
        for (int k = 0; k < S; ++k) mbar_init(&bar[k], 1);
        fence_mbar_init();
        abort_flag = 0;
    }
    __syncthreads();
    uint32_t inflight = 0;  // stages with a copy issued and not yet waited for (thread 0)
    auto issue = [&](long long tile, int b) {
        const int f = (int)(tile / tiles_f);
        const long long r0 = (tile - (long long)f * tiles_f) * RB;
        const int rows = (int)min((long long)RB, rows_f - r0);
        const uint32_t bytes = (uint32_t)(rows * N * sizeof(C));
        mbar_arrive_expect_tx(&bar[b], bytes);
        bulk_g2s(buf0 + b * BUF, fp.pick(fp.in, f) + r0 * N, bytes, &bar[b]);
        inflight |= 1u << b;
    };
    if (tid == 0)
        for (int k = 0; k < S - 1; ++k) {
            const long long tl = blockIdx.x + (long long)k * gridDim.x;
            if (tl < ntiles) issue(tl, k);
        }
    uint32_t parity = 0;  // bit k: parity of the next phase of stage k
    int b = 0;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int f = (int)(tile / tiles_f);
        const long long r0 = (tile - (long long)f * tiles_f) * RB;
        const int rows = (int)min((long long)RB, rows_f - r0);
        const int limit = (first_wait >= 0 && tile == blockIdx.x) ? first_wait : kSpinLimit;
        const bool ok = mbar_wait(&bar[b], (parity >> b) & 1u, limit);
        if (ok) {
            parity ^= 1u << b;
            inflight &= ~(1u << b);
        } else {
            abort_flag = 1;
        }
        C* in = buf0 + b * BUF;
        const int rl = tid / Tn, t = tid - rl * Tn;
        // generic-proxy accesses of the previous tile's buffer are ordered
        // before the bulk copy that will overwrite it
        fence_proxy_async_smem();
        __syncthreads();  // this tile has landed; the previous tile is finished
        if (abort_flag) {
            if (tid == 0) {
                atomicOr(status, ERR_TMA_TIMEOUT);
                for (int k = 0; k < S; ++k)  // bounded: let late copies land before the block exits
                    if ((inflight >> k) & 1u) mbar_wait(&bar[k], (parity >> k) & 1u);
            }
            return;
        }
        const long long next = tile + (long long)(S - 1) * gridDim.x;
        if (tid == 0 && next < ntiles) issue(next, (b + S - 1) % S);
        // rounds in descending order: round gr exchanges through padded rows
        // [gr RG, (gr + 1) RG), which lie past the natural rows of the rounds
        // still to come (PITCH >= N)
        for (int gr = G - 1; gr >= 0; --gr) {
            const int row = gr * RG + rl;
            const bool act = row < rows;
            C v[IO::E];
            if (act) {
#pragma unroll
                for (int i = 0; i < IO::E; ++i) v[i] = in[row * N + IO::in_elem(t, i)];
            }
            __syncthreads();  // the round's exchange rows overlap its natural rows
            smem_fft2<T, DIR, N, true, true, EM>(in + gr * RG * PITCH, xidx, rl, t, act, twy, 1, v);
            if (act) {
                C* out = fp.pick(fp.out, f) + (r0 + row) * N;
#pragma unroll
                for (int i = 0; i < IO::E; ++i) out[IO::out_elem(t, i)] = v[i];
            }
        }
        b = (b + 1) % S;
    }
}

template <typename T> inline size_t ypass_tma_smem(const Geom& g) {
    const int rb = YGroups<T>::value * ypass_rows<T>(g.ny);
    const int row = (g.ny + (g.ny >> 4) + 15) & ~15;
    return (size_t)kYStages * rb * row * sizeof(cplx<T>);
}
template <typename T> inline int ypass_tile_rows(int ny) { return YGroups<T>::value * ypass_rows<T>(ny); }

// ----------------------------------------------------------------- Z pass
// One block = kx = blockIdx.x, ky in [blockIdx.y*TZ, +TZ), all kz, NF fields
// (TZ = zpass_cols: 128-byte runs of ky).  kx fastest in the grid measured
// faster than ky-tile fastest on GB300.
// Threads: column c = tid % TZ (fastest, so global runs and shared-memory
// accesses are contiguous), t = tid / TZ; blockDim = TZ * nz/min(16, nz).
// Op provides
//   void load(int kx, int ky, int kz, size_t gi, cplx<T> v[NF])
//   void store(int kx, int ky, int kz, size_t gi, cplx<T> v[NF])
// with gi = (kz*H + kx)*ny + ky the spectral index of the mode.
// Columns per Z-pass block: 128-byte runs, fewer when nz needs > 256 threads.
template <typename T> __host__ __device__ inline int zpass_cols(int nz) {
    const int tn = fft_threads_per_row<T>(nz);
    return Tiles<T>::TZ * tn <= kThreads ? Tiles<T>::TZ : kThreads / tn;
}
template <typename T> __host__ __device__ inline int zpass_threads(int nz) {
    return zpass_cols<T>(nz) * fft_threads_per_row<T>(nz);
}

template <typename T, int NF, int DIR, int N, class Op>
__global__ void __launch_bounds__(kThreads) k_zpass(Geom g, const cplx<T>* __restrict__ twz, Op op) {
    using C = cplx<T>;
    constexpr int EM = FftE<T>::value;
    constexpr int E = N < EM ? N : EM;
    constexpr int Tn = N / E;
    constexpr int TZ = Tiles<T>::TZ * Tn <= kThreads ? Tiles<T>::TZ : kThreads / Tn;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const int kx = blockIdx.x, ky0 = blockIdx.y * TZ;
    const int c = threadIdx.x % TZ, t = threadIdx.x / TZ;
    const int ky = ky0 + c;
    const size_t zstride = (size_t)g.h * g.ny;
    const size_t base = (size_t)kx * g.ny + ky;
    const IdxColumns idx{TZ};
    constexpr size_t fstride = (size_t)N * TZ;
    if constexpr (NF == 1) {
        // the loaded modes are exactly the first stage's inputs
        using IO = FftIO<T, DIR, N>;
        C v[IO::E];
#pragma unroll
        for (int i = 0; i < IO::E; ++i) {
            const int z = IO::in_elem(t, i);
            C w[1];
            op.load(kx, ky, z, base + z * zstride, w);
            v[i] = w[0];
        }
        smem_fft2<T, DIR, N, true, false>(s, idx, c, t, true, twz, 1, v);
    } else if constexpr (HasSrc<Op>::value) {
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const C* src = op.src(f);
#pragma unroll
            for (int i = 0; i < E; ++i) {
                const int z = t + Tn * i;
                cp_async<sizeof(C)>(&s[f * fstride + idx(c, z)], src + base + z * zstride);
            }
        }
        cp_async_wait_all();
        __syncthreads();
#pragma unroll
        for (int f = 0; f < NF; ++f) smem_fft2<T, DIR, N>(s + f * fstride, idx, c, t, true, twz, 1);
    } else {
        // loads in chunks of CH modes per thread: CH * NF independent loads in flight
        constexpr int CH = 8 / NF >= 2 ? 8 / NF : 2;
#pragma unroll
        for (int i0 = 0; i0 < E; i0 += CH) {
            C v[CH][NF];
#pragma unroll
            for (int u = 0; u < CH; ++u)
                if (i0 + u < E) {
                    const int z = t + Tn * (i0 + u);
                    op.load(kx, ky, z, base + z * zstride, v[u]);
                }
#pragma unroll
            for (int u = 0; u < CH; ++u)
                if (i0 + u < E) {
                    const int z = t + Tn * (i0 + u);
#pragma unroll
                    for (int f = 0; f < NF; ++f) s[f * fstride + idx(c, z)] = v[u][f];
                }
        }
        __syncthreads();
#pragma unroll
        for (int f = 0; f < NF; ++f) smem_fft2<T, DIR, N>(s + f * fstride, idx, c, t, true, twz, 1);
    }
#pragma unroll 4
    for (int i = 0; i < E; ++i) {
        const int z = t + Tn * i;
        C v[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) v[f] = s[f * fstride + idx(c, z)];
        op.store(kx, ky, z, base + z * zstride, v);
    }
}

// Z pass with a round trip: the NF loaded fields are transformed along z
// in direction DIR; op.mid() maps each mode's NF values to NB values
// (writing whatever state it owns) that are transformed back in the other
// direction and stored output by output with op.rr_store(b, gi, v)
// (k_zpass_rt; k_zpass_rt_t hands a mode's NB values to op.store2()).  It
// replaces a forward Z pass and the
// inverse Z pass that read its output again (one write and one read of
// every intermediate spectrum less).  COLS ky columns per block (a run of
// COLS complex values per kz).
template <typename T, int N, int COLS, int EM = FftE<T>::value> struct ZRtShape {
    static constexpr int E = N < EM ? N : EM;
    static constexpr int Tn = N / E;                                      // threads per column FFT
    static constexpr int RC = COLS * Tn <= kThreads ? COLS : kThreads / Tn;  // columns per FFT round
    static constexpr int THREADS = RC * Tn;
    static constexpr int P = COLS + 1;  // shared-memory pitch of one kz row (odd: fewer bank conflicts)
    // WZ (FP32, one round of column FFTs of at most a warp each): the
    // forward transforms and the first stage of each inverse run on columns
    // owned by single warps; the tile then adds one pad slot per 16 kz rows
    // so that the strided writes of a column's first stage meet no bank
    // conflicts
    static constexpr bool WZ = sizeof(T) == 4 && RC == COLS && Tn <= 32 && FftPlan<N, EM>::NS >= 2;
    static constexpr int FSTRIDE = N * P + (WZ ? N / 16 : 0);  // complex entries per field tile
};
// Z round-trip tile index: mode e of column c, with the WZ pad slots.
template <bool PAD> struct IdxZ {
    int cols;
    __device__ __forceinline__ int operator()(int c, int e) const { return e * cols + c + (PAD ? (e >> 4) : 0); }
};

// The tile is COLS columns (a 128-byte run of ky per kz for FP32 and FP64)
// of all kz; the column FFTs run in rounds of RC columns, while loads and
// the mid operation walk the tile with ky fastest (full runs per warp).
// Tiles whose load() only copies arrays (src()) arrive by cp.async.
template <typename T, int NF, int NB, int DIR, int N, int COLS, class Op, int EM = FftE<T>::value>
__global__ void __launch_bounds__(kThreads) k_zpass_rt(Geom g, const cplx<T>* __restrict__ twz, Op op) {
    using C = cplx<T>;
    using SH = ZRtShape<T, N, COLS, EM>;
    constexpr int RC = SH::RC, P = SH::P, NT = SH::THREADS;
    constexpr int ELEMS = COLS * N;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const int kx = blockIdx.x, ky0 = blockIdx.y * COLS;
    const int tid = threadIdx.x;
    const size_t zstride = (size_t)g.h * g.ny;
    const size_t base = (size_t)kx * g.ny + ky0;
    constexpr bool WZ = SH::WZ;
    const IdxZ<WZ> idx{P};
    constexpr size_t fstride = SH::FSTRIDE;
    op.prologue();
    if constexpr (HasSrc<Op>::value) {
        // one cp.async group per field: the transform of field f starts once
        // its own tile has landed, while the later fields are still in flight
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const C* src = op.src(f);
            for (int e = tid; e < ELEMS; e += NT) {
                const int c = e % COLS, z = e / COLS;
                cp_async<sizeof(C)>(&s[f * fstride + idx(c, z)], src + base + c + z * zstride);
            }
            cp_async_commit();
        }
    } else {
        for (int e = tid; e < ELEMS; e += NT) {
            const int c = e % COLS, z = e / COLS;
            C v[NF];
            op.load(kx, ky0 + c, z, base + c + z * zstride, v);
#pragma unroll
            for (int f = 0; f < NF; ++f) s[f * fstride + idx(c, z)] = v[f];
        }
        __syncthreads();
    }
    const int cl = tid % RC, t = tid / RC;
    // WZ: the forward transforms (and the first stage of each inverse) run
    // on columns owned by single warps (wc = tid / Tn), synchronising only
    // the warp; the mid operation and the inverse's last stage keep the
    // column-fastest mapping (full 128-byte runs in global memory)
    using PLZ = FftPlan<N, EM>;
    const int wc = tid / PLZ::Tn, wt = tid % PLZ::Tn;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        if constexpr (HasSrc<Op>::value) {
            cp_async_wait_pending(NF - 1 - f);
            __syncthreads();
        }
        if constexpr (WZ) smem_fft2<T, DIR, N, EM, true>(s + f * fstride, idx, wc, wt, true, twz, 1);
        else
            for (int r = 0; r < COLS; r += RC) smem_fft2<T, DIR, N, EM>(s + f * fstride + r, idx, cl, t, true, twz, 1);
    }
    __syncthreads();
    if constexpr (HasPre<Op>::value) {
        // the mid operation's global reads of ZU modes are issued before any is used
        for (int e0 = tid; e0 < ELEMS; e0 += ZU * NT) {
            typename Op::PreT p[ZU];
#pragma unroll
            for (int u = 0; u < ZU; ++u) {
                const int e = e0 + u * NT;
                if (e < ELEMS) op.pre(kx, ky0 + e % COLS, e / COLS, base + e % COLS + (e / COLS) * zstride, p[u]);
            }
#pragma unroll
            for (int u = 0; u < ZU; ++u) {
                const int e = e0 + u * NT;
                if (e < ELEMS) {
                    const int c = e % COLS, z = e / COLS;
                    C vi[NF], vo[NB];
#pragma unroll
                    for (int f = 0; f < NF; ++f) vi[f] = s[f * fstride + idx(c, z)];
                    op.mid(kx, ky0 + c, z, base + c + z * zstride, vi, vo, p[u]);
#pragma unroll
                    for (int b = 0; b < NB; ++b) s[b * fstride + idx(c, z)] = vo[b];
                }
            }
        }
    } else {
        for (int e = tid; e < ELEMS; e += NT) {
            const int c = e % COLS, z = e / COLS;
            C vi[NF], vo[NB];
#pragma unroll
            for (int f = 0; f < NF; ++f) vi[f] = s[f * fstride + idx(c, z)];
            op.mid(kx, ky0 + c, z, base + c + z * zstride, vi, vo);
#pragma unroll
            for (int b = 0; b < NB; ++b) s[b * fstride + idx(c, z)] = vo[b];
        }
    }
    __syncthreads();
    // the inverse transforms' last stages store from registers: for each
    // slot a warp writes RC consecutive columns of Tn-strided modes (full
    // 128-byte runs), field by field while the next field is transformed
    using IO = FftIO<T, -DIR, N, EM>;
#pragma unroll
    for (int b = 0; b < NB; ++b)
        for (int r = 0; r < COLS; r += RC) {
            C v[SH::E];
            if constexpr (WZ) {
                constexpr int R0 = PLZ::radix(0, -DIR);
                fft_stage<T, R0, -DIR, N, 1, false, false, EM, true>(s + b * fstride, idx, wc, wt, true, twz, 1, v);
                __syncthreads();
                fft_stages<T, -DIR, N, 1, R0, false, true, EM, false>(s + b * fstride, idx, cl, t, true, twz, 1, v);
            } else {
                smem_fft2<T, -DIR, N, false, true, EM>(s + b * fstride + r, idx, cl, t, true, twz, 1, v);
            }
#pragma unroll
            for (int i = 0; i < SH::E; ++i) op.rr_store(b, base + r + cl + (size_t)IO::out_elem(t, i) * zstride, v[i]);
        }
}

// Round trip with the column-per-thread-group mapping of k_zpass: the tile
// is ZRtShapeT::TZ columns (one FFT round), loaded through registers, and
// each thread's mid and store work is on the modes its last FFT stage
// produced.  Measured faster than k_zpass_rt for three or more fields
// (smaller tiles, more blocks per SM); k_zpass_rt is faster for one.
template <typename T, int N, int COLS, int EM = FftE<T>::value> struct ZRtShapeT {
    static constexpr int E = N < EM ? N : EM;
    static constexpr int Tn = N / E;
    static constexpr int TZ = COLS * Tn <= kThreads ? COLS : kThreads / Tn;
};

template <typename T, int NF, int NB, int DIR, int N, int COLS, class Op, int EM = FftE<T>::value>
__global__ void __launch_bounds__(kThreads) k_zpass_rt_t(Geom g, const cplx<T>* __restrict__ twz, Op op) {
    using C = cplx<T>;
    using SH = ZRtShapeT<T, N, COLS, EM>;
    constexpr int E = SH::E, Tn = SH::Tn, TZ = SH::TZ;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const int kx = blockIdx.x, ky0 = blockIdx.y * TZ;
    const int c = threadIdx.x % TZ, t = threadIdx.x / TZ;
    const int ky = ky0 + c;
    const size_t zstride = (size_t)g.h * g.ny;
    const size_t base = (size_t)kx * g.ny + ky;
    const IdxColumns idx{TZ};
    constexpr size_t fstride = (size_t)N * TZ;
    op.prologue();
    {
        constexpr int CH = 8 / NF >= 2 ? 8 / NF : 2;
#pragma unroll
        for (int i0 = 0; i0 < E; i0 += CH) {
            C v[CH][NF];
#pragma unroll
            for (int u = 0; u < CH; ++u)
                if (i0 + u < E) {
                    const int z = t + Tn * (i0 + u);
                    op.load(kx, ky, z, base + z * zstride, v[u]);
                }
#pragma unroll
            for (int u = 0; u < CH; ++u)
                if (i0 + u < E) {
                    const int z = t + Tn * (i0 + u);
#pragma unroll
                    for (int f = 0; f < NF; ++f) s[f * fstride + idx(c, z)] = v[u][f];
                }
        }
    }
    __syncthreads();
#pragma unroll
    for (int f = 0; f < NF; ++f) smem_fft2<T, DIR, N, EM>(s + f * fstride, idx, c, t, true, twz, 1);
    // each thread's outputs of the last stage are the modes z = t + Tn i
#pragma unroll 2
    for (int i = 0; i < E; ++i) {
        const int z = t + Tn * i;
        C vi[NF], vo[NB];
#pragma unroll
        for (int f = 0; f < NF; ++f) vi[f] = s[f * fstride + idx(c, z)];
        op.mid(kx, ky, z, base + z * zstride, vi, vo);
#pragma unroll
        for (int b = 0; b < NB; ++b) s[b * fstride + idx(c, z)] = vo[b];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; ++b) smem_fft2<T, -DIR, N, EM>(s + b * fstride, idx, c, t, true, twz, 1);
#pragma unroll 4
    for (int i = 0; i < E; ++i) {
        const int z = t + Tn * i;
        C v[NB];
#pragma unroll
        for (int b = 0; b < NB; ++b) v[b] = s[b * fstride + idx(c, z)];
        op.store2(kx, ky, z, base + z * zstride, v);
    }
}

// Round trip held in registers (the FP32 passes): each thread loads its
// column's modes straight into the first FFT stage, the mid operation runs
// on the last stage's outputs (FftIO: the same modes the inverse's first
// stage takes), and every inverse transform is stored from registers.
// Shared memory only carries the exchanges between FFT stages, one field
// at a time through a single tile.  The op supplies State (what a mode
// keeps between the transforms), rr_mid (NF transformed values -> State),
// rr_out (output b of a State) and rr_store (output b at gi).
template <typename T, int NF, int NB, int DIR, int N, int COLS, class Op, int EM = FftE<T>::value>
__global__ void __launch_bounds__(kThreads, 2) k_zpass_rr(Geom g, const cplx<T>* __restrict__ twz, Op op) {
    using C = cplx<T>;
    using SH = ZRtShapeT<T, N, COLS, EM>;
    using IOF = FftIO<T, DIR, N, EM>;
    using IOI = FftIO<T, -DIR, N, EM>;
    constexpr int E = SH::E, TZ = SH::TZ;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const int kx = blockIdx.x, ky0 = blockIdx.y * TZ;
    const int c = threadIdx.x % TZ, t = threadIdx.x / TZ;
    const int ky = ky0 + c;
    const size_t zstride = (size_t)g.h * g.ny;
    const size_t base = (size_t)kx * g.ny + ky;
    const IdxColumns idx{TZ};
    op.prologue();
    // the mid operation's extra spectral input (op.aux()) is staged with
    // cp.async behind the exchange tile while the forward transform runs
    C* sa = s + (size_t)TZ * N;
    if constexpr (HasAux<Op>::value) {
        const C* aux = op.aux() + (size_t)kx * g.ny + ky0;
        for (int e = threadIdx.x; e < TZ * N; e += blockDim.x) {
            const int cc = e % TZ, z = e / TZ;
            cp_async<sizeof(C)>(&sa[(size_t)z * TZ + cc], aux + cc + z * zstride);
        }
    }
    typename Op::State st[E];
    {
        C v[NF][E];
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int z = IOF::in_elem(t, i);
            C w[NF];
            op.load(kx, ky, z, base + z * zstride, w);
#pragma unroll
            for (int f = 0; f < NF; ++f) v[f][i] = w[f];
        }
#pragma unroll
        for (int f = 0; f < NF; ++f) smem_fft2<T, DIR, N, true, true, EM>(s, idx, c, t, true, twz, 1, v[f]);
        if constexpr (HasAux<Op>::value) {
            cp_async_wait_all();
            __syncthreads();
        }
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int z = IOF::out_elem(t, i);
            C w[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) w[f] = v[f][i];
            if constexpr (HasAux<Op>::value) op.rr_mid(kx, ky, z, base + z * zstride, w, sa[(size_t)z * TZ + c], st[i]);
            else op.rr_mid(kx, ky, z, base + z * zstride, w, st[i]);
        }
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        C v[E];
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int z = IOF::out_elem(t, i);
            // the staged aux value is read again per output instead of being
            // kept in registers across the inverse transforms
            if constexpr (HasAux<Op>::value) v[i] = op.rr_out(b, kx, ky, z, st[i], sa[(size_t)z * TZ + c]);
            else v[i] = op.rr_out(b, kx, ky, z, st[i]);
        }
        smem_fft2<T, -DIR, N, true, true, EM>(s, idx, c, t, true, twz, 1, v);
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int z = IOI::out_elem(t, i);
            op.rr_store(b, base + z * zstride, v[i]);
        }
    }
}

template <typename T, int NF>
inline size_t zpass_smem(const Geom& g) {
    return (size_t)NF * zpass_cols<T>(g.nz) * g.nz * sizeof(cplx<T>);
}

}  // namespace fipi
