// Y and X passes of one z plane fused over a thread-block cluster (FP32).
//
// The unfused step runs a Y pass (rows of ky for each (z, kx)), an X pass
// (rows of kx for each (z, y)) and another Y pass, each reading and writing
// its fields once in HBM.  A z plane of one FP32 half spectrum (nx/2 + 1
// rows of ny complex values: 264 KB at 256^3) does not fit one CTA, but it
// fits the distributed shared memory of a cluster of kPlaneCS CTAs, so one
// kernel can take a plane from the Z pass's output to the next Z pass's
// input with one HBM read and one HBM write per field:
//
//   A  each CTA loads its kx rows (kx = rank, rank + CS, ...) of every input
//      field and transforms them along y (Y inverse) in place;
//   B  (cluster barrier) each CTA gathers, for its ny/CS rows of y, every
//      kx from the CTAs that own them (ld.shared::cluster) into an X-pass
//      tile and runs the X pass on it: C2R, the fused point operation, R2C;
//   C  (cluster barrier: every gather is done) each CTA scatters its output
//      tile back to the owners of the kx rows (st.shared::cluster);
//   D  (cluster barrier) each CTA transforms its kx rows of every output
//      field along y (Y forward) and stores them.
//
// The transforms are the Y pass's (radix-16 register codelets, the same
// twiddles) and the X pass's (split pre/post-processing, radix-8 rows), so
// the arithmetic is that of the three separate passes.  Every CTA executes
// every barrier (no CTA leaves early); the barriers are the hardware's.
#pragma once

#include "passes.cuh"

namespace fipi {

constexpr int kPlaneCS = 16;  // CTAs per cluster (one z plane)

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Address of `p` (this CTA's shared memory) in the shared memory of CTA `rank`.
__device__ __forceinline__ uint32_t cluster_addr(const void* p, unsigned rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_addr(p)), "r"(rank));
    return r;
}
// No memory clobber: the loads of a gather are independent and issue back
// to back; the cluster barriers (which clobber memory) order them against
// the stores of the other phases.
__device__ __forceinline__ float2 ld_cluster(uint32_t a) {
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}
__device__ __forceinline__ void st_cluster(uint32_t a, float2 v) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}

template <int M, int NY> struct PlaneShape {
    static constexpr int CS = kPlaneCS;
    static constexpr int NT = 256;
    static constexpr int H = M + 1;                // kx rows of the half spectrum
    static constexpr int RMAX = (H + CS - 1) / CS;  // kx rows of a CTA at most
    static constexpr int TY = NY / CS;              // y rows of a CTA's X tile
    static constexpr int EY = YE<float>::value;     // Y codelet: values per thread
    static constexpr int TnY = NY / EY;             // threads per Y row
    static constexpr int YPITCH = (NY + (NY >> 4) + 15) & ~15;  // >= padded_len(NY) (exchange rows)
    static constexpr int YBUF = RMAX * YPITCH;      // complex values per field (rows at stride NY)
    static constexpr int EM = FftE<float>::value;   // X codelet
    static constexpr int TnX = M / EM;
    static_assert(NT / TnY >= RMAX, "the kx rows of a CTA are one Y round");
    static_assert(NT / TnX == TY, "the X tile is one FFT round");
    static constexpr size_t smem(int nf) {
        return (size_t)nf * (YBUF + (size_t)TY * (M + (M >> kXPad) + 2)) * sizeof(cplx<float>);
    }
};

// Y transform of the CTA's `rows` kx rows of one field, in place in `buf`
// (natural rows at stride NY, exchanges through padded rows as the Y pass).
template <int DIR, int NY, int M>
__device__ __forceinline__ void plane_y(cplx<float>* buf, int rows, const cplx<float>* __restrict__ twy,
                                        cplx<float>* gout, size_t gstride, unsigned rank) {
    using C = cplx<float>;
    using SH = PlaneShape<M, NY>;
    using IO = FftIO<float, DIR, NY, SH::EY>;
    const IdxPadded xidx{padded_len(NY)};
    const int rl = threadIdx.x / SH::TnY, t = threadIdx.x % SH::TnY;
    const bool act = rl < rows;
    C v[IO::E];
    if (act) {
#pragma unroll
        for (int i = 0; i < IO::E; ++i) v[i] = buf[rl * NY + IO::in_elem(t, i)];
    }
    __syncthreads();  // the exchange rows overlap the natural rows
    smem_fft2<float, DIR, NY, true, true, SH::EY>(buf, xidx, rl, t, act, twy, 1, v);
    if (gout) {  // Y forward: straight to global memory (kx = rank + CS * rl)
        if (act) {
            C* dst = gout + (size_t)(rank + SH::CS * rl) * gstride;
#pragma unroll
            for (int i = 0; i < IO::E; ++i) dst[IO::out_elem(t, i)] = v[i];
        }
    } else {
        __syncthreads();  // every thread has read the last exchange
        if (act) {
#pragma unroll
            for (int i = 0; i < IO::E; ++i) buf[rl * NY + IO::out_elem(t, i)] = v[i];
        }
    }
}

// One cluster per z plane (blockIdx.x = z * CS + rank).  Op: the X pass's
// op (in(f), out(f), point(z, y, n, v, acc)); in(f) / out(f) are the
// spectral arrays before the Y inverse / after the Y forward.  REDUCE: the
// FP64 sum of each CTA's point accumulator goes to partials[z * CS + rank]
// (the X pass's block index: plane z, tile of rows `rank`).
template <int NIN, int NOUT, bool REDUCE, int M, int NY, class Op>
__global__ void __launch_bounds__(256) k_plane_yx(Geom g, const cplx<float>* __restrict__ twx,
                                                  const cplx<float>* __restrict__ twy, Op op, double* partials) {
    using T = float;
    using C = cplx<T>;
    using SH = PlaneShape<M, NY>;
    constexpr int CS = SH::CS, NT = SH::NT, H = SH::H, TY = SH::TY;
    constexpr int NF = NIN > NOUT ? NIN : NOUT;
    static_assert(NOUT <= NIN, "outputs return through the input fields' row buffers");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* ybuf = reinterpret_cast<C*>(smem_raw);   // NIN fields x YBUF
    C* s = ybuf + (size_t)NIN * SH::YBUF;        // X tile: NF fields x TY rows
    const IdxX idx{xpass_pitch(M)};
    const unsigned rank = cluster_rank();
    const int z = blockIdx.x / CS;
    const int tid = threadIdx.x;
    const int rows = (H - (int)rank + CS - 1) / CS;  // kx rows owned: rank, rank + CS, ...
    const size_t plane = (size_t)z * H * NY;

    // A: load the owned kx rows of every input field, Y inverse in place
#pragma unroll
    for (int f = 0; f < NIN; ++f) {
        const C* src = op.in(f) + plane;
        C* buf = ybuf + (size_t)f * SH::YBUF;
        constexpr int CH = NY * (int)sizeof(C) / 16;  // 16-byte chunks per row
        for (int e = tid; e < rows * CH; e += NT) {
            const int j = e / CH, q = e - j * CH;
            cp_async<16>(reinterpret_cast<unsigned char*>(buf + j * NY) + 16 * q,
                         reinterpret_cast<const unsigned char*>(src + (size_t)(rank + CS * j) * NY) + 16 * q);
        }
        cp_async_commit();
    }
    cp_async_wait_all();
    __syncthreads();
#pragma unroll
    for (int f = 0; f < NIN; ++f) plane_y<+1, NY, M>(ybuf + (size_t)f * SH::YBUF, rows, twy, nullptr, 0, rank);
    cluster_sync_all();

    // B: gather this CTA's y rows (y0 = rank * TY) of every kx, X pass
    const int y0 = (int)rank * TY;
    // all of a thread's remote loads of a field are issued before any of
    // their values is stored
    constexpr int PER = (TY * H + NT - 1) / NT;
#pragma unroll
    for (int f = 0; f < NIN; ++f) {
        const C* buf = ybuf + (size_t)f * SH::YBUF;
        float2 r[PER];
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int e = tid + k * NT;
            if (e < TY * H) {
                const int yl = e % TY, kx = e / TY;
                r[k] = ld_cluster(cluster_addr(buf + (kx / CS) * NY + y0 + yl, (unsigned)(kx % CS)));
            }
        }
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int e = tid + k * NT;
            if (e < TY * H) s[idx(f * TY + e % TY, e / TY)] = mkc<C>(r[k].x, r[k].y);
        }
    }
    __syncthreads();
    constexpr int Tn = SH::TnX;
#pragma unroll
    for (int f = 0; f < NIN; ++f) {
        C* sf = s + (size_t)f * TY * idx.pitch;
        c2r_pre<T, M, TY, NT>(sf, idx, twx, tid);
        __syncthreads();
        smem_fft2<T, +1, M, SH::EM>(sf, idx, tid / Tn, tid % Tn, true, twx, 2);
    }
    const T invV = T(1) / T(g.V);
    T acc = T(0);
    for (int i = tid; i < TY * M; i += NT) {
        const int n = i % M, ty = i / M;
        C v[NF];
#pragma unroll
        for (int f = 0; f < NIN; ++f) v[f] = cscale(s[idx(f * TY + ty, n)], invV);
        op.point(z, y0 + ty, n, v, acc);
#pragma unroll
        for (int f = 0; f < NOUT; ++f) s[idx(f * TY + ty, n)] = v[f];
    }
    if constexpr (REDUCE) {
        const double bs = block_sum((double)acc);
        if (tid == 0) partials[(size_t)z * CS + rank] = bs;
    }
    __syncthreads();
#pragma unroll
    for (int f = 0; f < NOUT; ++f)
        smem_fft2<T, -1, M, SH::EM>(s + (size_t)f * TY * idx.pitch, idx, tid / Tn, tid % Tn, true, twx, 2);
    r2c_post<T, M, NOUT * TY, NT>(s, idx, twx, tid);
    __syncthreads();
    cluster_sync_all();  // every gather of phase B is done: the row buffers can be overwritten

    // C: scatter the output tile to the owners' row buffers
#pragma unroll
    for (int f = 0; f < NOUT; ++f) {
        C* buf = ybuf + (size_t)f * SH::YBUF;
        for (int e = tid; e < TY * H; e += NT) {
            const int yl = e % TY, kx = e / TY;
            const C v = s[idx(f * TY + yl, kx)];
            st_cluster(cluster_addr(buf + (kx / CS) * NY + y0 + yl, (unsigned)(kx % CS)), make_float2(v.x, v.y));
        }
    }
    cluster_sync_all();  // every scatter has landed; no remote access follows

    // D: Y forward of the owned rows, stored to the outputs
#pragma unroll
    for (int f = 0; f < NOUT; ++f) {
        __syncthreads();
        plane_y<-1, NY, M>(ybuf + (size_t)f * SH::YBUF, rows, twy, op.out(f) + plane, NY, rank);
    }
}

}  // namespace fipi
