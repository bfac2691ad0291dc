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

#include "common.cuh"

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

// In-place FFT of `rows` rows of length n (power of two, 4 <= n <= 4*blockDim)
// held in shared memory at s[r*pitch + e].  tw[q*ts] = exp(-2 pi i q / n).
// dir = -1 forward, +1 backward (conjugated twiddles).  All threads of the
// block must call it.
template <typename T>
__device__ __forceinline__ void smem_fft(cplx<T>* s, int n, int log2n, int rows, int pitch,
                                         const cplx<T>* __restrict__ tw, int ts, int dir) {
    using C = cplx<T>;
    const int tid = threadIdx.x;
    const int q4 = n >> 2;
    int rpg = (4 * (int)blockDim.x) / n;
    if (rpg > rows) rpg = rows;
    const int active = rpg * q4;
    const int lrow = tid / q4;
    const int i0 = tid - lrow * q4;
    for (int r0 = 0; r0 < rows; r0 += rpg) {
        const bool act = (tid < active) && (r0 + lrow < rows);
        C* row = s + (size_t)(r0 + lrow) * pitch;
        int p = 1;
        if (log2n & 1) {  // radix-2 stage with p = 1 (no twiddles): tasks i0 and i0 + q4
            C u0, u1, u2, u3;
            const int half = n >> 1;
            if (act) {
                u0 = row[i0];
                u1 = row[i0 + half];
                u2 = row[i0 + q4];
                u3 = row[i0 + q4 + half];
            }
            __syncthreads();
            if (act) {
                row[2 * i0] = cadd(u0, u1);
                row[2 * i0 + 1] = csub(u0, u1);
                row[2 * (i0 + q4)] = cadd(u2, u3);
                row[2 * (i0 + q4) + 1] = csub(u2, u3);
            }
            __syncthreads();
            p = 2;
        }
        for (; p < n; p <<= 2) {
            C v0, v1, v2, v3;
            const int k = i0 & (p - 1);
            if (act) {
                C u0 = row[i0], u1 = row[i0 + q4], u2 = row[i0 + 2 * q4], u3 = row[i0 + 3 * q4];
                if (p > 1) {
                    const int step = (n / (4 * p)) * k * ts;
                    C w1 = tw[step], w2 = tw[2 * step], w3 = tw[3 * step];
                    if (dir > 0) {
                        w1.y = -w1.y;
                        w2.y = -w2.y;
                        w3.y = -w3.y;
                    }
                    u1 = cmul(u1, w1);
                    u2 = cmul(u2, w2);
                    u3 = cmul(u3, w3);
                }
                const C a0 = cadd(u0, u2), a1 = csub(u0, u2), a2 = cadd(u1, u3);
                const C a3 = cmul_i(csub(u1, u3), dir);
                v0 = cadd(a0, a2);
                v1 = cadd(a1, a3);
                v2 = csub(a0, a2);
                v3 = csub(a1, a3);
            }
            __syncthreads();
            if (act) {
                const int o = (i0 - k) * 4 + k;
                row[o] = v0;
                row[o + p] = v1;
                row[o + 2 * p] = v2;
                row[o + 3 * p] = v3;
            }
            __syncthreads();
        }
    }
}

// ----------------------------------------------------------------- Y pass
template <typename T> struct FieldPtrs {
    cplx<T>* in[8];
    cplx<T>* out[8];
};

// C2C along contiguous rows of length ny; blockIdx.y selects the field.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_ypass(Geom g, const cplx<T>* __restrict__ twy, int dir,
                                                   FieldPtrs<T> fp, int rows_per_block) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const long long total_rows = (long long)g.nz * g.h;
    const long long r0 = (long long)blockIdx.x * rows_per_block;
    int rows = rows_per_block;
    if (r0 + rows > total_rows) rows = (int)(total_rows - r0);
    const C* in = fp.in[blockIdx.y] + r0 * g.ny;
    C* out = fp.out[blockIdx.y] + r0 * g.ny;
    const int n = rows * g.ny;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = in[i];
    __syncthreads();
    smem_fft<T>(s, g.ny, g.ly, rows, g.ny, twy, 1, dir);
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = s[i];
}

// ----------------------------------------------------------------- Z pass
// One block = kx = blockIdx.x, ky in [blockIdx.y*TZ, +TZ), all kz, NF fields.
// Op provides
//   void load(int kx, int ky, int kz, size_t gi, cplx<T> v[NF])
//   void store(int kx, int ky, int kz, size_t gi, cplx<T> v[NF])
// with gi = (kz*H + kx)*ny + ky the spectral index of the mode.
template <typename T, int NF, class Op>
__global__ void __launch_bounds__(kThreads) k_zpass(Geom g, const cplx<T>* __restrict__ twz, int dir, Op op) {
    using C = cplx<T>;
    constexpr int TZ = Tiles<T>::TZ;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* s = reinterpret_cast<C*>(smem_raw);
    const int kx = blockIdx.x, ky0 = blockIdx.y * TZ;
    const int pitch = g.nz + 1;
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int idx = tid; idx < g.nz * TZ; idx += nthr) {
        const int kyl = idx % TZ;
        const int z = idx / TZ;
        const size_t gi = ((size_t)z * g.h + kx) * g.ny + ky0 + kyl;
        C v[NF];
        op.load(kx, ky0 + kyl, z, gi, v);
#pragma unroll
        for (int f = 0; f < NF; ++f) s[(f * TZ + kyl) * pitch + z] = v[f];
    }
    __syncthreads();
    smem_fft<T>(s, g.nz, g.lz, NF * TZ, pitch, twz, 1, dir);
    for (int idx = tid; idx < g.nz * TZ; idx += nthr) {
        const int kyl = idx % TZ;
        const int z = idx / TZ;
        const size_t gi = ((size_t)z * g.h + kx) * g.ny + ky0 + kyl;
        C v[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) v[f] = s[(f * TZ + kyl) * pitch + z];
        op.store(kx, ky0 + kyl, z, gi, v);
    }
}

template <typename T, int NF>
inline size_t zpass_smem(const Geom& g) {
    return (size_t)NF * Tiles<T>::TZ * (g.nz + 1) * sizeof(cplx<T>);
}

}  // namespace fipi
