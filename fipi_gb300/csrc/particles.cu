// Lagrangian side of the FIPI step on sm_103a (main.cpp:186-219 and
// cluster.cpp / element.cpp of the reference).
//
//  - cell list: key = i + j n + k n^2 with i = floor(p/d_cell + margin/d_cell)
//    (cluster.cpp:140-165), a stable LSD radix sort of (key, particle id) and
//    offsets by binary search; ids inside a cell are ascending, which is the
//    order the reference's linked lists hold them in (linked_list.cpp:30-43);
//  - contact forces one warp per home cell (cluster.cpp:174-275): each lane
//    owns one particle of the cell and walks the 27 neighbour cells in the
//    reference's (k, j, i) order; every pair is evaluated from the lower id's
//    side exactly as the reference does and the result is applied with the
//    reference's sign, so forces are deterministic and atomic-free;
//  - interpolation, attachment force, Heun advection and periodic wrap per
//    particle (field.cpp:223-248, element.cpp:55-185);
//  - spreading (cluster.cpp:344-410) as a sorted segmented reduction: the
//    8 corner records of every particle are radix-sorted by grid node,
//    stable in particle id, and each node sums its records in ascending id,
//    the order in which the reference's loop adds them.
//
// Positions are FP64 in every form.  This file is compiled with
// -fmad=false so its FP64 expressions round exactly as the reference's.
// TA is the arithmetic type of interpolation, contact forces and spreading
// weights: double in the plain form, float in the mixed form.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "ctx.hpp"
#include "fixed_point.cuh"

namespace fipi {

// Threads per block of the per-particle kernels of the step: 20,000
// particles in 64-thread blocks reach every SM (256-thread blocks would
// leave half of the 152 SMs idle).
constexpr int kPT = 64;

struct PC {
    int n;
    int nc[3];
    double dc[3];
    double margin;
    double L[3];
    double r_eq, k_n, r_p, A, sigma, epsilon, pi, mu, dt;
    double dx, dy, dz;
    int N[3];
    double tanh2;  // tanh(2.0), element.cpp:84
    // Constants of the mixed form's particle arithmetic.  GB300 issues FP64
    // at about 1/70 of the FP32 rate, so the mixed form multiplies by
    // reciprocals instead of dividing, forms f_pi in FP32 and converts its
    // fixed-point sums with integer operations; positions stay FP64.
    double inv_d[3];   // 1/dx, 1/dy, 1/dz
    double inv_dc[3];  // 1/d_cell
    double mdc[3];     // margin/d_cell
    double drag;       // 6 pi mu: the Stokes drag is drag * r
    float f_req, f_req2, f_kn, f_dc[3], f_inv_vol, f_tanh2, f_dscale, f_apisig;
};

static PC make_pc(const fipi_ctx* ctx) {
    const fipi_params& P = ctx->P;
    PC c;
    c.n = P.n_p;
    for (int a = 0; a < 3; ++a) {
        c.nc[a] = ctx->pb.ncell[a];
        c.dc[a] = ctx->pb.dcell[a];
    }
    c.margin = P.margin;
    c.L[0] = P.lx;
    c.L[1] = P.ly;
    c.L[2] = P.lz;
    c.r_eq = P.r_eq;
    c.k_n = P.k_n;
    c.r_p = P.r_p;
    c.A = P.A;
    c.sigma = P.sigma;
    c.epsilon = P.epsilon;
    c.pi = P.pi;
    c.mu = P.mu;
    c.dt = P.dt;
    c.dx = P.lx / P.nx;
    c.dy = P.ly / P.ny;
    c.dz = P.lz / P.nz;
    c.N[0] = P.nx;
    c.N[1] = P.ny;
    c.N[2] = P.nz;
    c.tanh2 = std::tanh(2.0);
    const double d[3] = {c.dx, c.dy, c.dz};
    for (int a = 0; a < 3; ++a) {
        c.inv_d[a] = 1.0 / d[a];
        c.inv_dc[a] = 1.0 / c.dc[a];
        c.mdc[a] = c.margin / c.dc[a];
        c.f_dc[a] = (float)c.dc[a];
    }
    c.drag = 6.0 * c.pi * c.mu;
    c.f_req = (float)c.r_eq;
    c.f_req2 = c.f_req * c.f_req;
    c.f_kn = (float)c.k_n;
    c.f_inv_vol = (float)(1.0 / (c.dx * c.dy * c.dz));
    c.f_tanh2 = (float)c.tanh2;
    c.f_dscale = (float)(0.5 * 1.4142135623730951 * c.epsilon);
    c.f_apisig = (float)(c.A * c.pi * c.sigma);
    return c;
}

// ramp (primitive.cpp:122-129)
static double ramp(double t, double thr) {
    if (t < 0) return 0.0;
    if (t >= 0 && t < thr) return t / thr;
    return 1.0;
}

// ------------------------------------------------------------ radix sort
// Stable LSD radix sort of (key, value) pairs, 8-bit digits.
constexpr int RS_T = 256;
constexpr int RS_TILE = 2048;

__global__ void k_rs_hist(const unsigned* __restrict__ keys, int n, int shift, unsigned* hist, int nblk) {
    __shared__ unsigned cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RS_TILE;
    for (int i = threadIdx.x; i < RS_TILE; i += RS_T) {
        const int s = base + i;
        if (s < n) atomicAdd(&cnt[(keys[s] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblk + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of `total` entries in one block of 1024 threads.
__global__ void k_scan_excl(unsigned* a, int total) {
    __shared__ unsigned part[1024];
    const int t = threadIdx.x;
    const int chunk = (total + 1023) / 1024;
    const int b = t * chunk, e = min(total, b + chunk);
    unsigned s = 0;
    for (int i = b; i < e; ++i) s += a[i];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        unsigned v = (t >= off) ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    unsigned run = part[t] - s;
    for (int i = b; i < e; ++i) {
        const unsigned x = a[i];
        a[i] = run;
        run += x;
    }
}

__global__ void k_rs_scatter(const unsigned* __restrict__ kin, const unsigned* __restrict__ vin,
                             unsigned* __restrict__ kout, unsigned* __restrict__ vout, int n, int shift,
                             const unsigned* __restrict__ hist, int nblk) {
    __shared__ unsigned base[256];
    __shared__ unsigned wcnt[RS_T / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base[tid] = hist[tid * nblk + blockIdx.x];
    for (int w = 0; w < RS_T / 32; ++w) wcnt[w][tid] = 0;
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < RS_TILE; r += RS_T) {
        const int s = blockIdx.x * RS_TILE + r + tid;
        const bool valid = s < n;
        unsigned key = 0, val = 0, d = 256;
        if (valid) {
            key = kin[s];
            val = vin[s];
            d = (key >> shift) & 255u;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned rank = __popc(peers & lt);
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            unsigned run = base[tid];
            for (int w = 0; w < RS_T / 32; ++w) {
                const unsigned c = wcnt[w][tid];
                wcnt[w][tid] = run;
                run += c;
            }
            base[tid] = run;
        }
        __syncthreads();
        if (valid) {
            const unsigned pos = wcnt[warp][d] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        for (int w = 0; w < RS_T / 32; ++w) wcnt[w][tid] = 0;
        __syncthreads();
    }
}

// Sorts (k, v) by the low `bits` bits of k; results end in (k, v).
static void radix_sort(fipi_ctx* ctx, unsigned*& k, unsigned*& v, unsigned*& k2, unsigned*& v2, int n, int bits) {
    if (n <= 0) return;
    const int nblk = (n + RS_TILE - 1) / RS_TILE;
    for (int shift = 0; shift < bits; shift += 8) {
        { LaunchScope ls_(ctx, "radix sort hist", 0.0); k_rs_hist<<<nblk, RS_T, 0, ctx->stream>>>(k, n, shift, ctx->pb.hist, nblk); }
        { LaunchScope ls_(ctx, "radix sort scan", 0.0); k_scan_excl<<<1, 1024, 0, ctx->stream>>>(ctx->pb.hist, 256 * nblk); }
        { LaunchScope ls_(ctx, "radix sort scatter", 0.0); k_rs_scatter<<<nblk, RS_T, 0, ctx->stream>>>(k, v, k2, v2, n, shift, ctx->pb.hist, nblk); }
        std::swap(k, k2);
        std::swap(v, v2);
    }
}

static int bits_for(long long maxval) {
    int b = 1;
    while ((1ll << b) <= maxval) ++b;
    return b;
}

// ------------------------------------------------------------ cell list
__device__ __forceinline__ int cell_coord(double x, double dcell, double margin) {
    return (int)floor(x / dcell + margin / dcell);  // cluster.cpp:140-142
}

// x != 0.0 on the bits (true for NaN, false for -0.0), integer operations only
__device__ __forceinline__ bool nonzero_bits(double x) {
    return (__double_as_longlong(x) << 1) != 0;
}

// isfinite(x) from the exponent bits (integer operations only)
__device__ __forceinline__ bool finite_bits(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}

// Cell key of one position (cluster.cpp:140-163); out-of-range or
// non-finite positions are clamped and reported through the error word.
// FAST (mixed form): floor(x (1/d_cell) + margin/d_cell), one product
// instead of two divisions; a position within rounding of a cell face may
// land in the neighbouring cell, which changes no pair (the cells are
// wider than r_eq by more than that).
template <bool FAST = false>
__device__ __forceinline__ unsigned cell_key(const PC& pc, double x, double y, double z, int* status) {
    const double xs[3] = {x, y, z};
    int c[3];
    for (int a = 0; a < 3; ++a)
        c[a] = FAST ? (int)floor(fma(xs[a], pc.inv_dc[a], pc.mdc[a])) : cell_coord(xs[a], pc.dc[a], pc.margin);
    const bool fin = finite_bits(x) && finite_bits(y) && finite_bits(z);
    bool bad = !fin;
    for (int a = 0; a < 3; ++a) {
        if (c[a] < 0 || c[a] >= pc.nc[a]) {
            bad = true;
            c[a] = c[a] < 0 ? 0 : pc.nc[a] - 1;
        }
    }
    if (bad) atomicOr(status, fin ? ERR_OUT_OF_RANGE : ERR_NONFINITE);
    return (unsigned)(c[0] + c[1] * pc.nc[0] + c[2] * pc.nc[0] * pc.nc[1]);
}

__global__ void k_cell_keys(PC pc, const double* __restrict__ p, unsigned* keys, unsigned* ids, int* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pc.n) return;
    keys[i] = cell_key(pc, p[i], p[pc.n + i], p[2 * pc.n + i], status);
    ids[i] = (unsigned)i;
}

// off[c] = first sorted position whose key >= c, c in [0, ncells].
__global__ void k_cell_offsets(const unsigned* __restrict__ keys, int n, int* off, int ncells) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > ncells) return;
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int)keys[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    off[c] = lo;
}

// Cell list in four small kernels: keys and per-cell counts (the arrival
// slot from atomicAdd is arbitrary), an exclusive scan of the counts (the
// offsets), placement at offset + slot, then one warp per cell ranks its
// ids so each cell lists its particles in ascending id — the order of the
// stable sort of cluster::sorting (cluster.cpp:116-169).  The result does
// not depend on the order of the atomics.  With `ymax` the same kernels
// find it_mark of cluster.cpp:128-138 (the first id with the largest
// p_y > 0; unchanged when there is none).
template <bool FAST>
__global__ void k_cells_count(PC pc, const double* __restrict__ p, unsigned* keys, unsigned* slot, int* cnt,
                              unsigned long long* ymax, int* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    unsigned long long yb = 0;
    if (i < n) {
        const double y = p[n + i];
        const unsigned key = cell_key<FAST>(pc, p[i], y, p[2 * n + i], status);
        keys[i] = key;
        slot[i] = (unsigned)atomicAdd(&cnt[key], 1);
        // y > 0.0 on the bits: positive, at most +inf (NaN and -0.0 excluded)
        const long long b = __double_as_longlong(y);
        yb = (b > 0 && b <= 0x7ff0000000000000ll) ? (unsigned long long)b : 0ull;
    }
    if (ymax) {
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long x = __shfl_down_sync(0xffffffffu, yb, o);
            yb = x > yb ? x : yb;
        }
        if ((threadIdx.x & 31) == 0 && yb) atomicMax(&ymax[0], yb);
    }
}

// Exclusive scan of ncells counts into off[0..ncells] (one block).
__global__ void k_cells_scan(const int* __restrict__ cnt, int ncells, int* off) {
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int chunk = (ncells + 1023) / 1024;
    const int b = t * chunk, e = min(ncells, b + chunk);
    int s = 0;
    for (int i = b; i < e; ++i) s += cnt[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int v = (t >= o) ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - s;
    for (int i = b; i < e; ++i) {
        off[i] = run;
        run += cnt[i];
    }
    if (t == 1023) off[ncells] = part[1023];
}

__global__ void k_cells_place(PC pc, const double* __restrict__ p, const unsigned* __restrict__ keys,
                              const unsigned* __restrict__ slot, const int* __restrict__ off, unsigned* tmp,
                              unsigned long long* ymax) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (i >= n) return;
    tmp[off[keys[i]] + slot[i]] = (unsigned)i;
    if (ymax) {
        const unsigned long long best = ymax[0];
        if (best != 0ull && (unsigned long long)__double_as_longlong(p[n + i]) == best)
            atomicMin(&ymax[1], (unsigned long long)i);
    }
}

// One warp per cell: rank of each id among the cell's ids.  With spos the
// sorted cell-relative FP32 positions of the mixed-form contact forces are
// written as well (what k_sorted_pos computes).
__global__ void k_cells_order(PC pc, const double* __restrict__ p, const int* __restrict__ off, int ncells,
                              const unsigned* __restrict__ tmp, unsigned* ids, unsigned* skeys,
                              unsigned long long* ymax, int* it_mark, float4* spos) {
    const int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (ymax && blockIdx.x == 0 && threadIdx.x == 0) {
        if (ymax[0] != 0ull) *it_mark = (int)ymax[1];
        ymax[0] = 0ull;
        ymax[1] = ~0ull;
    }
    if (cell >= ncells) return;
    const int beg = off[cell], end = off[cell + 1];
    const int cx = cell % pc.nc[0], cy = (cell / pc.nc[0]) % pc.nc[1], cz = cell / (pc.nc[0] * pc.nc[1]);
    const int n = pc.n;
    for (int e = beg + lane; e < end; e += 32) {
        const unsigned id = tmp[e];
        int r = 0;
        for (int j = beg; j < end; ++j) r += tmp[j] < id;
        ids[beg + r] = id;
        skeys[beg + r] = (unsigned)cell;
        if (spos) {  // mixed form only: one fused multiply-add per axis
            float4 v;
            v.x = (float)fma((double)-cx, pc.dc[0], p[id]);
            v.y = (float)fma((double)-cy, pc.dc[1], p[n + id]);
            v.z = (float)fma((double)-cz, pc.dc[2], p[2 * n + id]);
            v.w = __int_as_float((int)id);
            spos[beg + r] = v;
        }
    }
}

// Returns true when it also computed it_mark (asked for by `want_it_mark`).
// With spos the sorted FP32 positions of the mixed-form contact forces too;
// `fast` takes the mixed form's cell keys (cell_key<true>).
static bool build_cells(fipi_ctx* ctx, const double* p_dev, bool want_it_mark = false, float4* spos = nullptr,
                        bool fast = false) {
    ParticleBufs& b = ctx->pb;
    const PC pc = make_pc(ctx);
    const int n = b.n;
    if (n <= 0) return false;
    const int nb = (n + kPT - 1) / kPT;
    unsigned long long* ym = want_it_mark ? b.ymax : nullptr;
    // keys_alt holds the per-particle keys (by id), ids_alt the arrival slots, then the placed ids
    cudaMemsetAsync(b.cell_cnt, 0, sizeof(int) * (b.ncells + 1), ctx->stream);
    {
        LaunchScope ls_(ctx, "cell keys + counts", 0.0);
        auto kern = fast ? k_cells_count<true> : k_cells_count<false>;
        kern<<<nb, kPT, 0, ctx->stream>>>(pc, p_dev, b.keys_alt, b.ids_alt, b.cell_cnt, ym, ctx->status);
    }
    { LaunchScope ls_(ctx, "cell offsets", 0.0); k_cells_scan<<<1, 1024, 0, ctx->stream>>>(b.cell_cnt, b.ncells, b.cell_off); }
    { LaunchScope ls_(ctx, "cell placement", 0.0); k_cells_place<<<nb, kPT, 0, ctx->stream>>>(pc, p_dev, b.keys_alt, b.ids_alt, b.cell_off, b.keys, ym); }
    { LaunchScope ls_(ctx, "cell order", 0.0); k_cells_order<<<(b.ncells * 32 + 255) / 256, 256, 0, ctx->stream>>>(pc, p_dev, b.cell_off, b.ncells, b.keys, b.ids, b.keys_alt, ym, b.it_mark, spos); }
    std::swap(b.keys, b.keys_alt);  // sorted keys now in keys
    return want_it_mark;
}

// ------------------------------------------------------------ contact forces
// Separation of exactly coincident particles: the reference draws
// rand()%1000/1e3*2 r_p - r_p per component (cluster.cpp:234-242); here the
// same 1e-3 lattice is drawn from a hash of the pair (lower id first).
__device__ __forceinline__ void coincident_d(int a, int b, double r_p, double d[3]) {
    unsigned long long h = ((unsigned long long)(unsigned)a << 32) ^ (unsigned long long)(unsigned)b;
    for (int k = 0; k < 3; ++k) {
        h += 0x9E3779B97F4A7C15ull;
        unsigned long long z = h;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        d[k] = (double)(z % 1000ull) / 1e3 * 2.0 * r_p - r_p;
    }
}

// MODE 0: forces (+ packing-energy terms); 1: count pairs (lower id side);
// 2: write pairs at pair_off[i].
template <typename TA, int MODE>
__global__ void k_f_pp(PC pc, const double* __restrict__ p, const unsigned* __restrict__ ids,
                       const int* __restrict__ off, const double* __restrict__ rmp_p, const double* __restrict__ f_pi,
                       const int* __restrict__ it_mark, double* f_pp, double* tau_part, int* pair_cnt,
                       const int* __restrict__ pair_off, int* pairs) {
    const int lane = threadIdx.x & 31;
    const int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int ncells = pc.nc[0] * pc.nc[1] * pc.nc[2];
    if (cell >= ncells) return;
    const int n = pc.n;
    const int ci = cell % pc.nc[0], cj = (cell / pc.nc[0]) % pc.nc[1], ck = cell / (pc.nc[0] * pc.nc[1]);
    const int beg = off[cell], end = off[cell + 1];
    const double rmp = rmp_p ? *rmp_p : 1.0;
    const double T0 = pc.dc[0] * (pc.nc[0] - 2), T1 = pc.dc[1] * (pc.nc[1] - 2), T2 = pc.dc[2] * (pc.nc[2] - 2);
    bool mark_ok = false;
    if (MODE == 0 && f_pi != nullptr) {
        const int m = *it_mark;
        if (m >= 0) {
            const double a = f_pi[m], b = f_pi[n + m], c = f_pi[2 * n + m];
            mark_ok = sqrt(a * a + b * b + c * c) != 0.0;
        }
    }
    for (int base = beg; base < end; base += 32) {
        const int s = base + lane;
        const bool active = s < end;
        const int i = active ? (int)ids[s] : 0;
        const double xi = p[i], yi = p[n + i], zi = p[2 * n + i];
        bool own_ok = false;
        if (MODE == 0 && f_pi != nullptr && active) {
            const double a = f_pi[i], b = f_pi[n + i], c = f_pi[2 * n + i];
            own_ok = sqrt(a * a + b * b + c * c) != 0.0;
        }
        TA ax = TA(0), ay = TA(0), az = TA(0);
        double tau = 0.0;
        int cnt = 0;
        int wpos = (MODE == 2 && active) ? pair_off[i] : 0;
        for (int dk = -1; dk <= 1; ++dk)
            for (int dj = -1; dj <= 1; ++dj)
                for (int di = -1; di <= 1; ++di) {
                    const int co = (ci + di + pc.nc[0]) % pc.nc[0] + (cj + dj + pc.nc[1]) % pc.nc[1] * pc.nc[0] +
                                   (ck + dk + pc.nc[2]) % pc.nc[2] * pc.nc[0] * pc.nc[1];
                    const int qe = off[co + 1];
                    for (int q = off[co]; q < qe; ++q) {
                        const int j = (int)ids[q];
                        const double xj = p[j], yj = p[n + j], zj = p[2 * n + j];
                        if (!active || j == i) continue;
                        const bool lo_side = i < j;  // the reference evaluates (it, id) with it < id
                        double d[3];
                        if (lo_side) {
                            d[0] = xi - xj;
                            d[1] = yi - yj;
                            d[2] = zi - zj;
                        } else {
                            d[0] = xj - xi;
                            d[1] = yj - yi;
                            d[2] = zj - zi;
                        }
                        // cluster.cpp:225-232
                        if (d[0] > T0) d[0] = d[0] - pc.L[0];
                        else if (d[0] < -T0) d[0] = d[0] + pc.L[0];
                        if (d[1] > T1) d[1] = d[1] - pc.L[1];
                        else if (d[1] < -T1) d[1] = d[1] + pc.L[1];
                        if (d[2] > T2) d[2] = d[2] - pc.L[2];
                        else if (d[2] < -T2) d[2] = d[2] + pc.L[2];
                        if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0)
                            coincident_d(lo_side ? i : j, lo_side ? j : i, pc.r_p, d);
                        const TA dx = (TA)d[0], dy = (TA)d[1], dz = (TA)d[2];
                        const TA dn = sqrt(dx * dx + dy * dy + dz * dz);
                        if (!(dn < (TA)pc.r_eq)) continue;
                        if (MODE == 1) {
                            if (lo_side) ++cnt;
                            continue;
                        }
                        if (MODE == 2) {
                            if (lo_side) {
                                pairs[2 * wpos] = i;
                                pairs[2 * wpos + 1] = j;
                                ++wpos;
                            }
                            continue;
                        }
                        const TA sc = ((TA)pc.r_eq - dn) * (TA)rmp * (TA)pc.k_n;
                        const TA fx = (dx / dn) * sc, fy = (dy / dn) * sc, fz = (dz / dn) * sc;
                        if (lo_side) {
                            ax = ax + fx;
                            ay = ay + fy;
                            az = az + fz;
                            if (own_ok && mark_ok) {
                                const double h0 = (double)fx * 0.5, h1 = (double)fy * 0.5, h2 = (double)fz * 0.5;
                                tau += h0 * d[0] + h1 * d[1] + h2 * d[2];
                            }
                        } else {
                            ax = ax - fx;
                            ay = ay - fy;
                            az = az - fz;
                        }
                    }
                }
        if (active) {
            if (MODE == 0) {
                f_pp[i] = (double)ax;
                f_pp[n + i] = (double)ay;
                f_pp[2 * n + i] = (double)az;
                if (tau_part) tau_part[i] = tau;
            } else if (MODE == 1) {
                pair_cnt[i] = cnt;
            }
        }
    }
}

// Mixed-form contact forces when every axis has at least 4 cells.  Then
// the reference's minimum-image rule (shift d by L when |d| exceeds
// d_cell (n_cell - 2), cluster.cpp:225-232) shifts exactly the pairs whose
// neighbour cell was reached through the periodic wrap, so d can be formed
// from cell-relative FP32 coordinates plus the neighbour cell's offset
// (di, dj, dk) d_cell, with no per-pair test.  A warp owns a home cell;
// candidates are read 32 at a time (coalesced float4: x, y, z relative to
// their cell, id) and broadcast by shuffles.  The force on the home
// particle from a pair is (d/|d|) s with d = p_i - p_j for either id
// order (exactly the reference's sign rule), summed in the reference's
// cell order.
__global__ void k_sorted_pos(PC pc, const double* __restrict__ p, const unsigned* __restrict__ keys,
                             const unsigned* __restrict__ ids, float4* __restrict__ spos) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= pc.n) return;
    const unsigned key = keys[s];
    const int i = (int)ids[s];
    const int cx = key % pc.nc[0], cy = (key / pc.nc[0]) % pc.nc[1], cz = key / (pc.nc[0] * pc.nc[1]);
    const int n = pc.n;
    float4 v;
    v.x = (float)(p[i] - cx * pc.dc[0]);
    v.y = (float)(p[n + i] - cy * pc.dc[1]);
    v.z = (float)(p[2 * n + i] - cz * pc.dc[2]);
    v.w = __int_as_float(i);
    spos[s] = v;
}

// One block per home cell, one warp per (dk, dj) neighbour row of three
// cells (9 warps); the nine partial forces of each home particle are then
// added in the reference's (k, j) cell order, so the result is
// deterministic.  Lanes own the home cell's particles, 32 at a time.
constexpr int kFppRows = 9;

__global__ void __launch_bounds__(32 * kFppRows) k_f_pp_fast(PC pc, const float4* __restrict__ spos,
                                                             const int* __restrict__ off,
                                                             const double* __restrict__ rmp_p,
                                                             const double* __restrict__ f_pi,
                                                             const int* __restrict__ it_mark, double* f_pp,
                                                             double* tau_part) {
    __shared__ float4 stage[kFppRows][3][32];  // per row warp: a chunk of each of its three cells
    __shared__ float part[kFppRows][4][32];    // fx, fy, fz, tau per row warp and lane
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int cell = blockIdx.x;
    const int n = pc.n;
    const int ci = cell % pc.nc[0], cj = (cell / pc.nc[0]) % pc.nc[1], ck = cell / (pc.nc[0] * pc.nc[1]);
    const int dk = w / 3 - 1, dj = w % 3 - 1;
    const int rowbase = (cj + dj + pc.nc[1]) % pc.nc[1] * pc.nc[0] + (ck + dk + pc.nc[2]) % pc.nc[2] * pc.nc[0] * pc.nc[1];
    // The home range and the ranges of the row's three cells are loaded
    // together (lanes 0-2 the starts, 3-5 the ends), then the first 32
    // candidates of each of the three cells: two dependent loads before the
    // pair loop instead of two per cell.
    const int cw = (ci + (lane % 3) - 1 + pc.nc[0]) % pc.nc[0] + rowbase;
    const int r6 = lane < 6 ? off[cw + (lane >= 3 ? 1 : 0)] : 0;
    const int beg = off[cell], end = off[cell + 1];
    int qb[3], qe[3], held[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        qb[c] = __shfl_sync(0xffffffffu, r6, c);
        qe[c] = __shfl_sync(0xffffffffu, r6, c + 3);
        held[c] = qb[c];  // first candidate of the chunk staged for cell c
    }
    {
        float4 v[3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (lane < qe[c] - qb[c]) v[c] = spos[qb[c] + lane];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            if (lane < qe[c] - qb[c]) stage[w][c][lane] = v[c];
    }
    // FP32 constants from the host; the ramp is converted once per warp
    const float req = pc.f_req, req2 = pc.f_req2, kn = pc.f_kn;
    float rmp = 0.f;
    if (lane == 0) rmp = (float)*rmp_p;
    rmp = __shfl_sync(0xffffffffu, rmp, 0);
    const float dcx = pc.f_dc[0], dcy = pc.f_dc[1], dcz = pc.f_dc[2];
    bool mark_ok = false;
    if (f_pi != nullptr) {
        const int m = *it_mark;
        if (m >= 0) mark_ok = nonzero_bits(f_pi[m]) || nonzero_bits(f_pi[n + m]) || nonzero_bits(f_pi[2 * n + m]);
    }
    __syncwarp();
    // L lanes per home particle when the cell holds few (L = 1, 2 or 4): the
    // L lanes take every L-th candidate and their sums meet by shuffles in a
    // fixed order (deterministic)
    const int cnt_home = end - beg;
    const int L = cnt_home <= 8 ? 4 : (cnt_home <= 16 ? 2 : 1);
    const int P = 32 / L;
    const int hl = lane / L, sub = lane % L;
    for (int base = beg; base < end; base += P) {
        const int s = base + hl;
        const bool active = s < end;
        const float4 h = active ? spos[s] : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        const int i = __float_as_int(h.w);
        bool own_ok = false;
        if (f_pi != nullptr && active)
            own_ok = nonzero_bits(f_pi[i]) || nonzero_bits(f_pi[n + i]) || nonzero_bits(f_pi[2 * n + i]);
        float ax = 0.f, ay = 0.f, az = 0.f, tau = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int di = c - 1;
            // home particle relative to the neighbour cell's origin (home frame)
            const float hx = h.x - di * dcx, hy = h.y - dj * dcy, hz = h.z - dk * dcz;
            for (int q0 = qb[c]; q0 < qe[c]; q0 += 32) {
                if (q0 != held[c]) {  // a cell of more than 32 particles: stage its next chunk
                    __syncwarp();
                    if (q0 + lane < qe[c]) stage[w][c][lane] = spos[q0 + lane];
                    held[c] = q0;
                    __syncwarp();
                }
                const int cnt = min(32, qe[c] - q0);
                if (!active) continue;
                for (int q = sub; q < cnt; q += L) {
                    const float4 cd = stage[w][c][q];
                    const int j = __float_as_int(cd.w);
                    float dx = hx - cd.x, dy = hy - cd.y, dz = hz - cd.z;
                    float d2 = dx * dx + dy * dy + dz * dz;
                    if (!(d2 < req2) || j == i) continue;
                    if (d2 == 0.f) {  // coincident in FP32: the hashed separation of the FP64 path
                        double d[3];
                        coincident_d(min(i, j), max(i, j), pc.r_p, d);
                        const float sg = i < j ? 1.f : -1.f;
                        dx = sg * (float)d[0];
                        dy = sg * (float)d[1];
                        dz = sg * (float)d[2];
                        d2 = dx * dx + dy * dy + dz * dz;
                        if (!(d2 < req2)) continue;
                    }
                    // (r_eq - |d|) ramp k_n d/|d|  =  (r_eq/|d| - 1) ramp k_n d
                    const float sc = (req * rsqrtf(d2) - 1.f) * rmp * kn;
                    const float fx = dx * sc, fy = dy * sc, fz = dz * sc;
                    ax += fx;
                    ay += fy;
                    az += fz;
                    if (own_ok && mark_ok && i < j) tau += (fx * 0.5f) * dx + (fy * 0.5f) * dy + (fz * 0.5f) * dz;
                }
            }
        }
        for (int o = 1; o < L; o <<= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, o);
            ay += __shfl_xor_sync(0xffffffffu, ay, o);
            az += __shfl_xor_sync(0xffffffffu, az, o);
            tau += __shfl_xor_sync(0xffffffffu, tau, o);
        }
        if (sub == 0) {
            part[w][0][hl] = ax;
            part[w][1][hl] = ay;
            part[w][2][hl] = az;
            part[w][3][hl] = tau;
        }
        __syncthreads();
        if (w == 0 && active && sub == 0) {
            float sx = 0.f, sy = 0.f, sz = 0.f, st = 0.f;
#pragma unroll
            for (int r = 0; r < kFppRows; ++r) {
                sx += part[r][0][hl];
                sy += part[r][1][hl];
                sz += part[r][2][hl];
                st += part[r][3][hl];
            }
            f_pp[i] = (double)sx;
            f_pp[n + i] = (double)sy;
            f_pp[2 * n + i] = (double)sz;
            if (tau_part) tau_part[i] = (double)st;
        }
        __syncthreads();
    }
}

// it_mark of cluster::sorting (cluster.cpp:128-138): the first index of
// the largest p_y, kept from the previous call when no p_y > 0.  For
// non-negative doubles the bit pattern orders like the value, so the
// maximum is an integer atomicMax and the first index an atomicMin.
// mk[0] = max bits, mk[1] = first index (as unsigned long long).
__global__ void k_ymax(const double* __restrict__ py, int n, unsigned long long* mk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long b = 0;
    if (i < n) {
        const double y = py[i];
        b = (y > 0.0) ? (unsigned long long)__double_as_longlong(y) : 0ull;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long x = __shfl_down_sync(0xffffffffu, b, o);
        b = x > b ? x : b;
    }
    if ((threadIdx.x & 31) == 0 && b) atomicMax(&mk[0], b);
}

__global__ void k_ymax_index(const double* __restrict__ py, int n, unsigned long long* mk, int* it_mark) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long best = mk[0];
    if (i < n && best != 0ull && (unsigned long long)__double_as_longlong(py[i]) == best)
        atomicMin(&mk[1], (unsigned long long)i);
}

__global__ void k_ymax_resolve(unsigned long long* mk, int* it_mark) {
    if (mk[0] != 0ull) *it_mark = (int)mk[1];
    mk[0] = 0ull;
    mk[1] = ~0ull;
}

// Sum of the per-particle packing-energy terms in a fixed order.
__global__ void k_sum_tau(const double* __restrict__ part, int n, double* out) {
    __shared__ double s[1024];
    double a = 0.0;
    const int chunk = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * chunk, e = min(n, b + chunk);
    for (int i = b; i < e; ++i) a += part[i];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) s[threadIdx.x] += s[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

// ------------------------------------------------------------ per-particle stage
// field::interpolate (field.cpp:223-248) of one real field.
template <typename TF, typename TA>
__device__ __forceinline__ TA interp(const TF* __restrict__ v, int i, int j, int k, int i1, int j1, int k1, TA m, TA nn,
                                     TA o, int Nx, int Ny) {
    const size_t sxy = (size_t)Nx * Ny;
    TA val = (TA(1) - m) * (TA(1) - nn) * (TA(1) - o) * (TA)v[i + (size_t)j * Nx + k * sxy];
    val += (TA(1) - m) * nn * (TA(1) - o) * (TA)v[i + (size_t)j1 * Nx + k * sxy];
    val += m * (TA(1) - nn) * (TA(1) - o) * (TA)v[i1 + (size_t)j * Nx + k * sxy];
    val += m * nn * (TA(1) - o) * (TA)v[i1 + (size_t)j1 * Nx + k * sxy];
    val += (TA(1) - m) * (TA(1) - nn) * o * (TA)v[i + (size_t)j * Nx + k1 * sxy];
    val += (TA(1) - m) * nn * o * (TA)v[i + (size_t)j1 * Nx + k1 * sxy];
    val += m * (TA(1) - nn) * o * (TA)v[i1 + (size_t)j * Nx + k1 * sxy];
    val += m * nn * o * (TA)v[i1 + (size_t)j1 * Nx + k1 * sxy];
    return val;
}

__device__ __forceinline__ int wrapi(int i, int n) {
    i %= n;
    return i < 0 ? i + n : i;
}

// Interpolate nf fields at particle i -> out[0..nf).
template <typename TF, typename TA>
__device__ __forceinline__ void interp_fields(const PC& pc, double x, double y, double z, const TF* const* f, int nf,
                                              TA* out) {
    const double fx = floor(x / pc.dx), fy = floor(y / pc.dy), fz = floor(z / pc.dz);
    const int i = wrapi((int)fx, pc.N[0]), j = wrapi((int)fy, pc.N[1]), k = wrapi((int)fz, pc.N[2]);
    const TA m = (TA)(x / pc.dx - fx), nn = (TA)(y / pc.dy - fy), o = (TA)(z / pc.dz - fz);
    const int i1 = (i + 1) % pc.N[0], j1 = (j + 1) % pc.N[1], k1 = (k + 1) % pc.N[2];
    for (int q = 0; q < nf; ++q) out[q] = interp<TF, TA>(f[q], i, j, k, i1, j1, k1, m, nn, o, pc.N[0], pc.N[1]);
}

// Node index (wrapped into [0, n)) and FP32 fraction of a coordinate, x (1/dx)
// split by floor: the mixed form's cell_and_frac / interpolation index.
__device__ __forceinline__ void node_frac_fast(double x, double inv, int n, int& i, float& fr) {
    const double q = x * inv;
    const double fq = floor(q);
    i = wrapi((int)fq, n);
    fr = (float)(q - fq);
}

// Mixed form: interp_fields with the index arithmetic of node_frac_fast.
template <typename TF>
__device__ __forceinline__ void interp_fields_fast(const PC& pc, double x, double y, double z, const TF* const* f,
                                                   int nf, float* out) {
    int i, j, k;
    float m, nn, o;
    node_frac_fast(x, pc.inv_d[0], pc.N[0], i, m);
    node_frac_fast(y, pc.inv_d[1], pc.N[1], j, nn);
    node_frac_fast(z, pc.inv_d[2], pc.N[2], k, o);
    const int i1 = i + 1 == pc.N[0] ? 0 : i + 1, j1 = j + 1 == pc.N[1] ? 0 : j + 1, k1 = k + 1 == pc.N[2] ? 0 : k + 1;
    for (int q = 0; q < nf; ++q) out[q] = interp<TF, float>(f[q], i, j, k, i1, j1, k1, m, nn, o, pc.N[0], pc.N[1]);
}

// element::get_f_pi (element.cpp:75-97) with f_mag = -A pi (d - r cos_theta) sigma.
__device__ __forceinline__ void f_pi_of(const PC& pc, double phi, double gx, double gy, double gz, double r, double ct,
                                        double* f) {
    const double gn = sqrt(gx * gx + gy * gy + gz * gz);
    if (fabs(phi) <= pc.tanh2 && gn != 0.0) {
        const double d = 0.5 * log((1.0 + phi) / (1.0 - phi)) * 1.4142135623730951 * pc.epsilon;
        double f_mag;
        if (fabs(d) < r) f_mag = -pc.A * pc.pi * (d - r * ct) * pc.sigma;
        else f_mag = 0.0;
        f[0] = gx / gn * f_mag;
        f[1] = gy / gn * f_mag;
        f[2] = gz / gn * f_mag;
    } else {
        f[0] = f[1] = f[2] = 0.0;
    }
}

// Mixed form: get_f_pi in FP32 from the FP32 interpolated phi and grad phi
// (d = 0.5 ln((1+phi)/(1-phi)) sqrt(2) eps, f_mag = -A pi sigma (d - r cos_theta)),
// stored as FP64 for the FP64 advection.
__device__ __forceinline__ void f_pi_fast(const PC& pc, float phi, float gx, float gy, float gz, double r_d,
                                          double ct_d, double* f) {
    const float gn = sqrtf(gx * gx + gy * gy + gz * gz);
    if (fabsf(phi) <= pc.f_tanh2 && gn != 0.f) {
        const float r = (float)r_d, ct = (float)ct_d;
        const float d = logf((1.f + phi) / (1.f - phi)) * pc.f_dscale;
        const float f_mag = fabsf(d) < r ? -pc.f_apisig * (d - r * ct) : 0.f;
        const float sc = f_mag / gn;
        f[0] = (double)(gx * sc);
        f[1] = (double)(gy * sc);
        f[2] = (double)(gz * sc);
    } else {
        f[0] = f[1] = f[2] = 0.0;
    }
}

// ------------------------------------------------------------ extensions
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011): ten rounds of two 32x32 -> 64-bit products
// with a Weyl-sequence key schedule.
__host__ __device__ inline void philox4x32(const unsigned ctr_in[4], unsigned k0, unsigned k1, unsigned out[4]) {
    unsigned c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const unsigned long long p0 = 0xD2511F53ull * c0, p1 = 0xCD9E8D57ull * c2;
        const unsigned hi0 = (unsigned)(p0 >> 32), lo0 = (unsigned)p0;
        const unsigned hi1 = (unsigned)(p1 >> 32), lo1 = (unsigned)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// Three standard normals the way element::get_f_rand draws them
// (element.cpp:109-144): Box-Muller on uniforms (k mod 1000)/1000, redrawn
// while |g| > 5 (only r1 = 0 is), here from the Philox stream of
// (particle, step) instead of rand(); at most 64 draws per normal (then 0).
__host__ __device__ inline void brownian_normals(unsigned long long seed, unsigned id, unsigned t, double pi,
                                                 double g[3]) {
    unsigned buf[4];
    int used = 4;
    unsigned blk = 0;
    auto next = [&]() -> unsigned {
        if (used == 4) {
            const unsigned ctr[4] = {id, t, blk++, 0u};
            philox4x32(ctr, (unsigned)seed, (unsigned)(seed >> 32), buf);
            used = 0;
        }
        return buf[used++];
    };
    for (int a = 0; a < 3; ++a) {
        double v = 0.0;
        for (int k = 0; k < 64; ++k) {
            const double r1 = double(next() % 1000u) / 1000;
            const double r2 = double(next() % 1000u) / 1000;
            v = sqrt(-2 * log(r1)) * cos(2 * pi * r2);
            if (fabs(v) <= 5.0) break;
            v = 0.0;
        }
        g[a] = v;
    }
}

// Per-step extension inputs of the stage kernels (all off: the reference's step).
struct PExt {
    const void* u[3];           // real fluid velocity (T), or NULL: uf = 0
    double* uf;                 // 3 x n: uf of the current stage
    double* f_rand;             // 3 x n: f_rand of the step, or NULL
    const int* d_t;             // step index (Philox counter)
    unsigned long long seed;
    double kt;
};

// fmod(x + L, L) (enforce_bc, element.cpp:177-185), bit for bit, without
// the FP64 remainder loop where x + L lies in [0, 2L): there the result is
// x + L or (x + L) - L, and the subtraction is exact (Sterbenz: L <= q <= 2L).
// The range tests compare bit patterns (non-negative doubles order like
// their bits).
__device__ __forceinline__ double wrap_exact(double x, double L) {
    const double q = x + L;
    const long long qb = __double_as_longlong(q), lb = __double_as_longlong(L);
    const long long l2b = lb + (1ll << 52);  // 2L: the exponent field plus one (L > 0 and normal)
    if (qb >= 0 && qb < lb) return q;
    if (qb >= lb && qb < l2b) return q - L;
    return fmod(q, L);
}

// element::advect (element.cpp:156-173) and enforce_bc (element.cpp:177-185)
// for one particle; f_ext = 0 as in the reference, uf = 0 unless fluid
// coupling is on, and f_rand only with a Brownian force.
__device__ __forceinline__ void advect_one(const PC& pc, int stage, const double* fpi, const double* fpp, double r,
                                           double* p, double* po, double* uo, const double* uf = nullptr,
                                           const double* fr = nullptr) {
    double v[3];
    for (int a = 0; a < 3; ++a) {
        double F = fpi[a] + 0.0;
        F = F + fpp[a];
        if (fr) F = F + fr[a];
        v[a] = (uf ? uf[a] : 0.0) + F / 6.0 / pc.pi / pc.mu / r;
    }
    if (stage == 1) {
        for (int a = 0; a < 3; ++a) {
            uo[a] = v[a];
            po[a] = p[a];
            p[a] = p[a] + v[a] * pc.dt;
        }
    } else {
        const double hdt = 0.5 * pc.dt;
        for (int a = 0; a < 3; ++a) p[a] = po[a] + (uo[a] + v[a]) * hdt;
    }
    for (int a = 0; a < 3; ++a) p[a] = wrap_exact(p[a], pc.L[a]);
}

// Mixed form: the same update with the drag as one reciprocal,
// v = F / (6 pi mu r), instead of four divisions per component.
__device__ __forceinline__ void advect_fast(const PC& pc, int stage, const double* fpi, const double* fpp, double r,
                                            double* p, double* po, double* uo, const double* uf = nullptr,
                                            const double* fr = nullptr) {
    const double mob = 1.0 / (pc.drag * r);
    double v[3];
    for (int a = 0; a < 3; ++a) {
        double F = fpi[a] + fpp[a];
        if (fr) F = F + fr[a];
        v[a] = uf ? fma(F, mob, uf[a]) : F * mob;
    }
    if (stage == 1) {
        for (int a = 0; a < 3; ++a) {
            uo[a] = v[a];
            po[a] = p[a];
            p[a] = fma(v[a], pc.dt, p[a]);
        }
    } else {
        const double hdt = 0.5 * pc.dt;
        for (int a = 0; a < 3; ++a) p[a] = fma(uo[a] + v[a], hdt, po[a]);
    }
    for (int a = 0; a < 3; ++a) p[a] = wrap_exact(p[a], pc.L[a]);
}

// Extension work of a stage for particle i at (x, y, z): uf from the fluid
// velocity (get_local_u with its interpolation, element.cpp:38-52) and, at
// the first stage of a step, the step's Brownian force
// sqrt(12 pi r mu kt / dt) g (element.cpp:138-143 with the particle's radius).
template <typename TF, typename TA>
__device__ __forceinline__ void stage_ext(const PC& pc, const PExt& ex, int i, double x, double y, double z, double r,
                                          bool first) {
    const int n = pc.n;
    if (ex.u[0]) {
        const TF* fl[3] = {(const TF*)ex.u[0], (const TF*)ex.u[1], (const TF*)ex.u[2]};
        TA uv[3];
        interp_fields<TF, TA>(pc, x, y, z, fl, 3, uv);
        for (int a = 0; a < 3; ++a) ex.uf[a * n + i] = (double)uv[a];
    }
    if (first && ex.f_rand) {
        double g[3];
        brownian_normals(ex.seed, (unsigned)i, (unsigned)*ex.d_t, pc.pi, g);
        const double s = sqrt(12.0 * pc.pi * r * pc.mu * ex.kt / pc.dt);
        for (int a = 0; a < 3; ++a) ex.f_rand[a * n + i] = s * g[a];
    }
}

__device__ __forceinline__ void ext_load(const PExt& ex, int n, int i, double* uf, double* fr, const double*& puf,
                                         const double*& pfr) {
    puf = nullptr;
    pfr = nullptr;
    if (ex.u[0]) {
        for (int a = 0; a < 3; ++a) uf[a] = ex.uf[a * n + i];
        puf = uf;
    }
    if (ex.f_rand) {
        for (int a = 0; a < 3; ++a) fr[a] = ex.f_rand[a * n + i];
        pfr = fr;
    }
}

// Stage part 1: interpolate c, grad c at the stage-start positions and form
// f_pi (cluster::interpolate_local_variables + compute_f_pi).
template <typename TF, typename TA>
__global__ void k_stage_fpi(PC pc, const TF* __restrict__ c, const TF* __restrict__ g0, const TF* __restrict__ g1,
                            const TF* __restrict__ g2, const double* __restrict__ p, double* f_pi,
                            const double* __restrict__ r, const double* __restrict__ cth, PExt ex) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (i >= n) return;
    const TF* fl[4] = {c, g0, g1, g2};
    TA vals[4];
    double fpi[3];
    if constexpr (std::is_same<TA, float>::value) {  // mixed form
        interp_fields_fast<TF>(pc, p[i], p[n + i], p[2 * n + i], fl, 4, vals);
        f_pi_fast(pc, vals[0], vals[1], vals[2], vals[3], r[i], cth[i], fpi);
    } else {
        interp_fields<TF, TA>(pc, p[i], p[n + i], p[2 * n + i], fl, 4, vals);
        f_pi_of(pc, (double)vals[0], (double)vals[1], (double)vals[2], (double)vals[3], r[i], cth[i], fpi);
    }
    for (int a = 0; a < 3; ++a) f_pi[a * n + i] = fpi[a];
    stage_ext<TF, TA>(pc, ex, i, p[i], p[n + i], p[2 * n + i], r[i], true);
}

// Stage 1's advection and wrap followed, for the same particle, by stage 2's
// interpolation of c, grad c and f_pi at the new position (k_stage_advect
// with stage = 1, then k_stage_fpi).
template <typename TF, typename TA>
__global__ void k_stage_advect1_fpi2(PC pc, double* p, double* p_old, double* u_old, double* f_pi,
                                     const double* __restrict__ f_pp, const double* __restrict__ r,
                                     const double* __restrict__ cth, const TF* __restrict__ c,
                                     const TF* __restrict__ g0, const TF* __restrict__ g1,
                                     const TF* __restrict__ g2, int* status, PExt ex) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (i >= n) return;
    double pp[3] = {p[i], p[n + i], p[2 * n + i]};
    double po[3], uo[3];
    const double fpi[3] = {f_pi[i], f_pi[n + i], f_pi[2 * n + i]};
    const double fpp[3] = {f_pp[i], f_pp[n + i], f_pp[2 * n + i]};
    double ufv[3], frv[3];
    const double *puf, *pfr;
    ext_load(ex, n, i, ufv, frv, puf, pfr);
    constexpr bool FAST = std::is_same<TA, float>::value;  // mixed form
    if constexpr (FAST) advect_fast(pc, 1, fpi, fpp, r[i], pp, po, uo, puf, pfr);
    else advect_one(pc, 1, fpi, fpp, r[i], pp, po, uo, puf, pfr);
    for (int a = 0; a < 3; ++a) {
        p[a * n + i] = pp[a];
        p_old[a * n + i] = po[a];
        u_old[a * n + i] = uo[a];
    }
    if (!(finite_bits(pp[0]) && finite_bits(pp[1]) && finite_bits(pp[2]))) {
        atomicOr(status, ERR_NONFINITE);
        return;
    }
    const TF* fl[4] = {c, g0, g1, g2};
    TA vals[4];
    double f2[3];
    if constexpr (FAST) {
        interp_fields_fast<TF>(pc, pp[0], pp[1], pp[2], fl, 4, vals);
        f_pi_fast(pc, vals[0], vals[1], vals[2], vals[3], r[i], cth[i], f2);
    } else {
        interp_fields<TF, TA>(pc, pp[0], pp[1], pp[2], fl, 4, vals);
        f_pi_of(pc, (double)vals[0], (double)vals[1], (double)vals[2], (double)vals[3], r[i], cth[i], f2);
    }
    for (int a = 0; a < 3; ++a) f_pi[a * n + i] = f2[a];
    stage_ext<TF, TA>(pc, ex, i, pp[0], pp[1], pp[2], r[i], false);
}

// Stage part 2: advect with this stage's f_pi + f_pp, then wrap (FAST: the
// mixed form's advect_fast).  With d_t the first thread also ends the step
// (k_step_tick's update; no thread of this kernel reads d_t or d_rmp).
template <bool FAST>
__global__ void k_stage_advect(PC pc, int stage, double* p, double* p_old, double* u_old,
                               const double* __restrict__ f_pi, const double* __restrict__ f_pp,
                               const double* __restrict__ r, int* status, PExt ex, int* d_t, double* d_rmp,
                               double thr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (d_t && i == 0) {
        const int t = ++(*d_t);
        const double x = (double)(t + 1);
        *d_rmp = (x < 0) ? 0.0 : (x < thr ? x / thr : 1.0);
    }
    if (i >= n) return;
    double pp[3] = {p[i], p[n + i], p[2 * n + i]};
    double po[3] = {p_old[i], p_old[n + i], p_old[2 * n + i]};
    double uo[3] = {u_old[i], u_old[n + i], u_old[2 * n + i]};
    const double fpi[3] = {f_pi[i], f_pi[n + i], f_pi[2 * n + i]};
    const double fpp[3] = {f_pp[i], f_pp[n + i], f_pp[2 * n + i]};
    double ufv[3], frv[3];
    const double *puf, *pfr;
    ext_load(ex, n, i, ufv, frv, puf, pfr);
    if constexpr (FAST) advect_fast(pc, stage, fpi, fpp, r[i], pp, po, uo, puf, pfr);
    else advect_one(pc, stage, fpi, fpp, r[i], pp, po, uo, puf, pfr);
    for (int a = 0; a < 3; ++a) {
        p[a * n + i] = pp[a];
        p_old[a * n + i] = po[a];
        u_old[a * n + i] = uo[a];
    }
    if (!(finite_bits(pp[0]) && finite_bits(pp[1]) && finite_bits(pp[2]))) atomicOr(status, ERR_NONFINITE);
}

// ------------------------------------------------------------ spreading
// Corner order of cluster.cpp:368-406: (0,0,0) (1,0,0) (1,1,0) (1,0,1) (1,1,1) (0,0,1) (0,1,0) (0,1,1).
__constant__ int c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {1, 0, 1}, {1, 1, 1}, {0, 0, 1}, {0, 1, 0}, {0, 1, 1}};

__device__ __forceinline__ void cell_and_frac(const PC& pc, double X, double Y, double Z, int* ix, double* fr) {
    const double fx = floor(X / pc.dx), fy = floor(Y / pc.dy), fz = floor(Z / pc.dz);
    ix[0] = wrapi((int)fx, pc.N[0]);
    ix[1] = wrapi((int)fy, pc.N[1]);
    ix[2] = wrapi((int)fz, pc.N[2]);
    fr[0] = X / pc.dx - fx;
    fr[1] = Y / pc.dy - fy;
    fr[2] = Z / pc.dz - fz;
}

// Per particle: the 8 corner records (node, particle*8 + corner), the force
// density f = (f_pp + f_ext)/dx/dy/dz and the fractions (o, p, q) of
// cluster.cpp:358-366, computed once here instead of once per record.
template <typename TA>
__global__ void k_spread_records(PC pc, const double* __restrict__ p, const double* __restrict__ f_pp,
                                 unsigned* keys, unsigned* vals, TA* __restrict__ fw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (i >= n) return;
    int ix[3];
    double fr[3];
    cell_and_frac(pc, p[i], p[n + i], p[2 * n + i], ix, fr);
    for (int c = 0; c < 8; ++c) {
        const int x = (ix[0] + c_corner[c][0]) % pc.N[0];
        const int y = (ix[1] + c_corner[c][1]) % pc.N[1];
        const int z = (ix[2] + c_corner[c][2]) % pc.N[2];
        keys[8 * i + c] = (unsigned)(x + (size_t)y * pc.N[0] + (size_t)z * pc.N[0] * pc.N[1]);
        vals[8 * i + c] = (unsigned)(8 * i + c);
    }
    for (int a = 0; a < 3; ++a) {
        fw[a * n + i] = (TA)((f_pp[a * n + i] + 0.0) / pc.dx / pc.dy / pc.dz);
        fw[(3 + a) * n + i] = (TA)fr[a];
    }
}

template <typename TF>
__global__ void k_spread_clear(const unsigned* __restrict__ nodes, int m, TF* f0, TF* f1, TF* f2) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    const unsigned nd = nodes[s];
    f0[nd] = TF(0);
    f1[nd] = TF(0);
    f2[nd] = TF(0);
}

// Weight products of cluster.cpp:369-406 for corner c, left to right from f.
template <typename TA>
__device__ __forceinline__ TA corner_value(TA f, int c, TA o, TA pp, TA q) {
    switch (c) {
        case 0: return f * (TA(1) - o) * (TA(1) - pp) * (TA(1) - q);
        case 1: return f * o * (TA(1) - pp) * (TA(1) - q);
        case 2: return f * o * pp * (TA(1) - q);
        case 3: return f * o * (TA(1) - pp) * q;
        case 4: return f * o * pp * q;
        case 5: return f * (TA(1) - o) * (TA(1) - pp) * q;
        case 6: return f * (TA(1) - o) * pp * (TA(1) - q);
        default: return f * (TA(1) - o) * pp * q;
    }
}

template <typename TF, typename TA>
__global__ void k_spread_reduce(PC pc, const unsigned* __restrict__ keys, const unsigned* __restrict__ vals, int m,
                                const TA* __restrict__ fw, TF* f0, TF* f1, TF* f2) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    const unsigned node = keys[s];
    if (s > 0 && keys[s - 1] == node) return;
    const int n = pc.n;
    TA acc[3] = {TA(0), TA(0), TA(0)};
    for (int q = s; q < m && keys[q] == node; ++q) {
        const unsigned rec = vals[q];
        const int i = (int)(rec >> 3), c = (int)(rec & 7u);
        const TA o = fw[3 * n + i], pp = fw[4 * n + i], qq = fw[5 * n + i];
#pragma unroll
        for (int a = 0; a < 3; ++a) acc[a] += corner_value<TA>(fw[a * n + i], c, o, pp, qq);
    }
    f0[node] = (TF)acc[0];
    f1[node] = (TF)acc[1];
    f2[node] = (TF)acc[2];
}

// ------------------------------------------------------------ orchestration
// `step_grid`: the target is the step's persistent spread grid, which only
// the nodes written by the previous spread need clearing in (the whole grid
// after a fine-grained call reused the record buffers).
template <typename T>
static void spread_t(fipi_ctx* ctx, const double* p, const double* f_pp, T* const f3[3], bool step_grid) {
    ParticleBufs& b = ctx->pb;
    const PC pc = make_pc(ctx);
    const int n = b.n, m = 8 * n;
    if (step_grid) {
        if (b.sp_prev_valid) {
            { LaunchScope ls_(ctx, "spread clear", 0.0); k_spread_clear<T><<<(m + 255) / 256, 256, 0, ctx->stream>>>(b.sp_prev, m, f3[0], f3[1], f3[2]); }
        } else {
            for (int a = 0; a < 3; ++a) cudaMemsetAsync(f3[a], 0, sizeof(T) * (size_t)ctx->g.V, ctx->stream);
        }
    }
    { LaunchScope ls_(ctx, "spread records", 0.0); k_spread_records<T><<<(n + 255) / 256, 256, 0, ctx->stream>>>(pc, p, f_pp, b.sp_keys, b.sp_vals, (T*)b.sp_fw); }
    radix_sort(ctx, b.sp_keys, b.sp_vals, b.sp_keys_alt, b.sp_vals_alt, m, bits_for(ctx->g.V - 1));
    { LaunchScope ls_(ctx, "spread segmented reduce", 0.0); k_spread_reduce<T, T><<<(m + 255) / 256, 256, 0, ctx->stream>>>(pc, b.sp_keys, b.sp_vals, m, (const T*)b.sp_fw, f3[0], f3[1], f3[2]); }
    if (step_grid) {
        cudaMemcpyAsync(b.sp_prev, b.sp_keys, sizeof(unsigned) * m, cudaMemcpyDeviceToDevice, ctx->stream);
        b.sp_prev_valid = 1;
    }
}

// Mixed-form spreading of the step: the 8 FP32 corner contributions of each
// particle (the weight products of cluster.cpp:369-406) are added as 64-bit
// fixed-point integers (units of 2^-32) with atomics.  Integer addition is
// associative, so the sums do not depend on the order of the atomics (the
// result is deterministic) and no sort is needed; the touched nodes are
// then converted to FP32.  The FP64 form keeps the sorted reduction in
// ascending particle id, bit-identical to the reference.
//
// Between steps the accumulators are zero everywhere and the force grids are
// zero except at the 8n nodes of the previous spread (nodes[]): the atomics
// kernel first zeroes the grids at its particle's previous nodes, and the
// store kernel takes each node's sum with an exchange against zero, so the
// first of a node's duplicate slots writes the grid and the others read 0.

// Range of the fixed-point sums: a node's running sums must stay inside the
// signed 64-bit accumulators, |sum| < 2^31 units.  Each node also sums the
// magnitudes of its contributions (|v_x| + |v_y| + |v_z|, FP32, a fire-and-
// forget atomic like the sums), which bounds every running sum of every
// component; the store kernel reports ERR_SPREAD_RANGE when that bound
// reaches kFxMaxNodeMagnitude (2^31 less a margin for the FP32 rounding of
// the bound), and a single contribution of 2^30 units or more (or NaN) is
// reported and left out at once.
constexpr float kFxMaxContribution = 1073741824.0f;   // 2^30
constexpr float kFxMaxNodeMagnitude = 2.1e9f;         // < 2^31 = 2.147e9


// One thread per (particle, corner), the eight corners of a particle on
// eight consecutive lanes (its position and force are loaded once per
// warp): a launch of 8 n threads instead of n keeps every SM busy.  Corner c
// is (c_corner[c][0..2]) as bit c of 0x1E, 0xD4 and 0xB8, and its weight
// is the product of corner_value (x factor, then y, then z) with each factor
// selected instead of switched on, so the lanes do not diverge.
__global__ void k_spread_fx(PC pc, const double* __restrict__ p, const double* __restrict__ f_pp,
                            unsigned long long* acc, unsigned* nodes, int clear_prev, float* f0, float* f1,
                            float* f2, int* status) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gid >> 3, c = gid & 7;
    const int n = pc.n;
    if (i >= n) return;
    if (clear_prev) {
        const unsigned nd = nodes[8 * i + c];
        f0[nd] = 0.f;
        f1[nd] = 0.f;
        f2[nd] = 0.f;
    }
    // the weights' fractions as in cell_and_frac, the force density in FP32
    int ix[3];
    float o, pp, q;
    node_frac_fast(p[i], pc.inv_d[0], pc.N[0], ix[0], o);
    node_frac_fast(p[n + i], pc.inv_d[1], pc.N[1], ix[1], pp);
    node_frac_fast(p[2 * n + i], pc.inv_d[2], pc.N[2], ix[2], q);
    const int cx = (0x1E >> c) & 1, cy = (0xD4 >> c) & 1, cz = (0xB8 >> c) & 1;
    const int x = (ix[0] + cx) % pc.N[0];
    const int y = (ix[1] + cy) % pc.N[1];
    const int z = (ix[2] + cz) % pc.N[2];
    const unsigned node = (unsigned)(x + (size_t)y * pc.N[0] + (size_t)z * pc.N[0] * pc.N[1]);
    nodes[8 * i + c] = node;
    const float wx = cx ? o : 1.f - o, wy = cy ? pp : 1.f - pp, wz = cz ? q : 1.f - q;
    unsigned long long* slot = acc + 4 * (size_t)node;
    float m = 0.f;
    for (int a = 0; a < 3; ++a) {
        const float v = (((float)f_pp[a * n + i] * pc.f_inv_vol) * wx * wy) * wz;
        if (!(fabsf(v) < kFxMaxContribution)) {  // also NaN
            atomicOr(status, ERR_SPREAD_RANGE);
            continue;
        }
        m += fabsf(v);
        atomicAdd(slot + a, (unsigned long long)fx_units(v));
    }
    if (m != 0.f) atomicAdd(reinterpret_cast<float*>(slot + 3), m);
}

__global__ void k_spread_fx_store(const unsigned* __restrict__ nodes, int m, unsigned long long* acc, float* f0,
                                  float* f1, float* f2, int* status) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    const unsigned nd = nodes[s];
    unsigned long long* slot = acc + 4 * (size_t)nd;
    if (atomicExch(reinterpret_cast<float*>(slot + 3), 0.f) >= kFxMaxNodeMagnitude) atomicOr(status, ERR_SPREAD_RANGE);
    float* fa[3] = {f0, f1, f2};
    for (int a = 0; a < 3; ++a) {
        const unsigned long long v = atomicExch(slot + a, 0ull);
        if (v != 0ull) fa[a][nd] = fx_to_float((long long)v);
    }
}

static void spread_fx(fipi_ctx* ctx) {
    ParticleBufs& b = ctx->pb;
    const PC pc = make_pc(ctx);
    const int n = b.n, m = 8 * n;
    const size_t V = (size_t)ctx->g.V;
    float* f0 = (float*)ctx->fb.fsp[0];
    float* f1 = (float*)ctx->fb.fsp[1];
    float* f2 = (float*)ctx->fb.fsp[2];
    if (!b.sp_prev_valid) {
        cudaMemsetAsync(b.sp_acc, 0, sizeof(unsigned long long) * 4 * V, ctx->stream);
        for (int a = 0; a < 3; ++a) cudaMemsetAsync(ctx->fb.fsp[a], 0, sizeof(float) * V, ctx->stream);
    }
    {
        LaunchScope ls_(ctx, "spread fixed-point atomics", 0.0);
        k_spread_fx<<<(m + 255) / 256, 256, 0, ctx->stream>>>(pc, b.p, b.f_pp, b.sp_acc, b.sp_prev, b.sp_prev_valid,
                                                              f0, f1, f2, ctx->status);
    }
    { LaunchScope ls_(ctx, "spread store", 0.0); k_spread_fx_store<<<(m + 255) / 256, 256, 0, ctx->stream>>>(b.sp_prev, m, b.sp_acc, f0, f1, f2,
                                                                                                     ctx->status); }
    b.sp_prev_valid = 1;
}

void particles_spread(fipi_ctx* ctx) {
    if (ctx->pb.n <= 0 || !ctx->P.switch_particle) return;
    if (ctx->prec == FIPI_MIXED) {
        spread_fx(ctx);
    } else {
        double* f3[3] = {(double*)ctx->fb.fsp[0], (double*)ctx->fb.fsp[1], (double*)ctx->fb.fsp[2]};
        spread_t<double>(ctx, ctx->pb.p, ctx->pb.f_pp, f3, true);
    }
}

// compute_f_pp; with `tau` the packing energy of cluster.cpp:256-259 is
// accumulated per particle and summed in a fixed order.  TA = float with
// at least 4 cells per axis takes the FP32 cell-relative path.
// it_mark for the packing energy: the first index of the largest p_y.
static void it_mark_launch(fipi_ctx* ctx, const double* p) {
    ParticleBufs& b = ctx->pb;
    const int nb = (b.n + 255) / 256;
    { LaunchScope ls_(ctx, "it_mark argmax", 0.0); k_ymax<<<nb, 256, 0, ctx->stream>>>(p + b.n, b.n, b.ymax); }
    { LaunchScope ls_(ctx, "it_mark argmax", 0.0); k_ymax_index<<<nb, 256, 0, ctx->stream>>>(p + b.n, b.n, b.ymax, b.it_mark); }
    { LaunchScope ls_(ctx, "it_mark argmax", 0.0); k_ymax_resolve<<<1, 1, 0, ctx->stream>>>(b.ymax, b.it_mark); }
}

// compute_f_pp; with `tau` the packing energy of cluster.cpp:256-259 is
// accumulated per particle (tau_part) and summed when it is asked for.
// TA = float with at least 4 cells per axis takes the FP32 cell-relative path.
static bool f_pp_fast_path(const fipi_ctx* ctx, bool fp32) {
    const ParticleBufs& b = ctx->pb;
    return fp32 && b.ncell[0] >= 4 && b.ncell[1] >= 4 && b.ncell[2] >= 4;
}

template <typename TA>
static void f_pp_launch(fipi_ctx* ctx, const double* p, const double* rmp, const double* f_pi, double* f_pp, bool tau,
                        bool have_it_mark = false, bool have_spos = false) {
    ParticleBufs& b = ctx->pb;
    const PC pc = make_pc(ctx);
    const int warps = b.ncells;
    const int blocks = (warps * 32 + 255) / 256;
    if (tau && !have_it_mark) it_mark_launch(ctx, p);
    const bool fast = f_pp_fast_path(ctx, sizeof(TA) == sizeof(float));
    if (fast) {
        if (!have_spos) { LaunchScope ls_(ctx, "sorted FP32 positions", 0.0); k_sorted_pos<<<(b.n + kPT - 1) / kPT, kPT, 0, ctx->stream>>>(pc, p, b.keys, b.ids, b.spos); }
        { LaunchScope ls_(ctx, "contact forces (warp per cell)", 0.0); k_f_pp_fast<<<b.ncells, 32 * kFppRows, 0, ctx->stream>>>(pc, b.spos, b.cell_off, rmp, tau ? f_pi : nullptr, b.it_mark, f_pp, b.tau_part); }
    } else {
        { LaunchScope ls_(ctx, "contact forces (warp per cell)", 0.0); k_f_pp<TA, 0><<<blocks, 256, 0, ctx->stream>>>(pc, p, b.ids, b.cell_off, rmp, tau ? f_pi : nullptr, b.it_mark,
                                                  f_pp, b.tau_part, nullptr, nullptr, nullptr); }
    }
    b.tau_valid = tau;
}

// The packing energy of the last contact-force evaluation (fixed-order sum).
fipi_status particles_packing_tau(fipi_ctx* ctx, double* out) {
    ParticleBufs& b = ctx->pb;
    if (!b.tau_valid || b.n == 0) {
        *out = 0.0;
        return FIPI_OK;
    }
    { LaunchScope ls_(ctx, "packing energy sum", 0.0); k_sum_tau<<<1, 1024, 0, ctx->stream>>>(b.tau_part, b.n, b.tau); }
    FIPI_CUDA(ctx, d2h(ctx, out, b.tau, sizeof(double)));
    return FIPI_OK;
}

static PExt particle_ext(const fipi_ctx* ctx) {
    PExt ex{};
    if (ctx->couple_u) {
        const size_t es = ctx->prec == FIPI_MIXED ? sizeof(float) : sizeof(double);
        for (int a = 0; a < 3; ++a) ex.u[a] = (const char*)ctx->fb.ureal + a * (size_t)ctx->g.V * es;
        ex.uf = ctx->pb.uf;
    }
    if (ctx->brown_kt > 0.0) {
        ex.f_rand = ctx->pb.f_rand;
        ex.kt = ctx->brown_kt;
        ex.seed = ctx->noise_seed;
    }
    ex.d_t = ctx->d_t;
    return ex;
}

// Buffers of the extensions, allocated when one is switched on.
fipi_status particles_ext_alloc(fipi_ctx* ctx) {
    ParticleBufs& b = ctx->pb;
    const size_t bytes = sizeof(double) * 3 * (size_t)(b.n > 0 ? b.n : 1);
    if ((ctx->couple_u || ctx->brown_kt > 0.0) && !b.uf) {
        FIPI_CUDA(ctx, cudaMalloc((void**)&b.uf, bytes));
        FIPI_CUDA(ctx, cudaMalloc((void**)&b.f_rand, bytes));
        FIPI_CUDA(ctx, cudaMemset(b.uf, 0, bytes));
        FIPI_CUDA(ctx, cudaMemset(b.f_rand, 0, bytes));
    }
    return FIPI_OK;
}

template <typename T> static void step_t(fipi_ctx* ctx) {
    constexpr bool FAST = sizeof(T) == sizeof(float);  // mixed form
    ParticleBufs& b = ctx->pb;
    const PC pc = make_pc(ctx);
    const int n = b.n;
    const int nb = (n + kPT - 1) / kPT;
    const T* c = (const T*)ctx->fb.c;
    const T* g0 = (const T*)ctx->fb.g[0];
    const T* g1 = (const T*)ctx->fb.g[1];
    const T* g2 = (const T*)ctx->fb.g[2];
    float4* spos = f_pp_fast_path(ctx, FAST) ? b.spos : nullptr;
    // per stage: interpolate_local_variables, sorting, compute_f_pi,
    // compute_f_pp(t+1), compute_f_ext (zero), advect, enforce_bc
    // (main.cpp:198-217); the ramp(t+1, 0.2 t_end) factor is kept on the
    // device: the last advection kernel advances it with t (step_tick's
    // update).  Stage 1's advection and stage 2's interpolation run in one
    // kernel.
    const PExt ex = particle_ext(ctx);
    { LaunchScope ls_(ctx, "stage interpolate + f_pi", 0.0); k_stage_fpi<T, T><<<nb, kPT, 0, ctx->stream>>>(pc, c, g0, g1, g2, b.p, b.f_pi, b.r, b.cth, ex); }
    for (int stage = 1; stage <= 2; ++stage) {
        const bool im = build_cells(ctx, b.p, ctx->track_tau, spos, FAST);
        f_pp_launch<T>(ctx, b.p, ctx->d_rmp, b.f_pi, b.f_pp, ctx->track_tau, im, spos != nullptr);
        if (stage == 1) {
            LaunchScope ls_(ctx, "stage advect + interpolate + f_pi", 0.0);
            k_stage_advect1_fpi2<T, T><<<nb, kPT, 0, ctx->stream>>>(pc, b.p, b.p_old, b.u_old, b.f_pi, b.f_pp, b.r,
                                                                     b.cth, c, g0, g1, g2, ctx->status, ex);
        } else {
            LaunchScope ls_(ctx, "stage advect + wrap", 0.0);
            k_stage_advect<FAST><<<nb, kPT, 0, ctx->stream>>>(pc, 2, b.p, b.p_old, b.u_old, b.f_pi, b.f_pp, b.r,
                                                              ctx->status, ex, ctx->d_t, ctx->d_rmp,
                                                              0.2 * ctx->P.t_end);
        }
    }
}

bool particles_step(fipi_ctx* ctx) {
    if (ctx->pb.n <= 0 || !ctx->P.switch_particle) return false;
    if (ctx->couple_u) fields_velocity_real(ctx);  // u^{n+1} at the particles (get_local_u)
    if (ctx->prec == FIPI_MIXED) step_t<float>(ctx);
    else step_t<double>(ctx);
    return true;
}

// End of a step: t += 1 and the next step's ramp(t + 1, 0.2 t_end)
// (compute_f_pp(t+1), main.cpp:202; primitive.cpp:122-129).
__global__ void k_step_tick(int* d_t, double* d_rmp, double thr) {
    const int t = ++(*d_t);
    const double x = (double)(t + 1);
    *d_rmp = (x < 0) ? 0.0 : (x < thr ? x / thr : 1.0);
}

void step_tick(fipi_ctx* ctx) {
    LaunchScope ls_(ctx, "step tick", 0.0);
    k_step_tick<<<1, 1, 0, ctx->stream>>>(ctx->d_t, ctx->d_rmp, 0.2 * ctx->P.t_end);
}

// ------------------------------------------------------------ allocation
fipi_status particles_alloc(fipi_ctx* ctx) {
    ParticleBufs& b = ctx->pb;
    const fipi_params& P = ctx->P;
    b.n = P.n_p;
    fipi_cell_geometry(&P, b.ncell, b.dcell);
    b.ncells = b.ncell[0] * b.ncell[1] * b.ncell[2];
    const int n = b.n > 0 ? b.n : 1;
    auto A = [&](void** ptr, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(ptr, bytes);
        if (e == cudaSuccess) {
            ctx->device_bytes += bytes;
            e = cudaMemsetAsync(*ptr, 0, bytes, ctx->stream);
        }
        return e;
    };
    FIPI_CUDA(ctx, A((void**)&b.p, sizeof(double) * 3 * n));
    FIPI_CUDA(ctx, A((void**)&b.p_old, sizeof(double) * 3 * n));
    FIPI_CUDA(ctx, A((void**)&b.u_old, sizeof(double) * 3 * n));
    FIPI_CUDA(ctx, A((void**)&b.f_pp, sizeof(double) * 3 * n));
    FIPI_CUDA(ctx, A((void**)&b.f_pi, sizeof(double) * 3 * n));
    FIPI_CUDA(ctx, A((void**)&b.r, sizeof(double) * n));
    FIPI_CUDA(ctx, A((void**)&b.cth, sizeof(double) * n));
    FIPI_CUDA(ctx, A((void**)&b.keys, sizeof(unsigned) * n));
    FIPI_CUDA(ctx, A((void**)&b.keys_alt, sizeof(unsigned) * n));
    FIPI_CUDA(ctx, A((void**)&b.ids, sizeof(unsigned) * n));
    FIPI_CUDA(ctx, A((void**)&b.ids_alt, sizeof(unsigned) * n));
    FIPI_CUDA(ctx, A((void**)&b.cell_off, sizeof(int) * (b.ncells + 1)));
    FIPI_CUDA(ctx, A((void**)&b.cell_cnt, sizeof(int) * (b.ncells + 1)));
    FIPI_CUDA(ctx, A((void**)&b.sp_keys, sizeof(unsigned) * 8 * n));
    FIPI_CUDA(ctx, A((void**)&b.sp_keys_alt, sizeof(unsigned) * 8 * n));
    FIPI_CUDA(ctx, A((void**)&b.sp_vals, sizeof(unsigned) * 8 * n));
    FIPI_CUDA(ctx, A((void**)&b.sp_vals_alt, sizeof(unsigned) * 8 * n));
    FIPI_CUDA(ctx, A((void**)&b.sp_prev, sizeof(unsigned) * 8 * n));
    if (ctx->prec == FIPI_MIXED && b.n > 0) {
        FIPI_CUDA(ctx, A((void**)&b.sp_acc, sizeof(unsigned long long) * 4 * (size_t)P.nx * P.ny * P.nz));
    }
    b.hist_cap = 256 * ((16 * n + RS_TILE - 1) / RS_TILE + 1);  // up to 16 records per particle (adjoint)
    FIPI_CUDA(ctx, A((void**)&b.hist, sizeof(unsigned) * b.hist_cap));
    FIPI_CUDA(ctx, A((void**)&b.tau_part, sizeof(double) * n));
    FIPI_CUDA(ctx, A((void**)&b.spos, sizeof(float4) * n));
    FIPI_CUDA(ctx, A((void**)&b.sp_fw, sizeof(double) * 6 * n));
    FIPI_CUDA(ctx, A((void**)&b.ymax, sizeof(unsigned long long) * 2));
    {
        const unsigned long long init[2] = {0ull, ~0ull};
        FIPI_CUDA(ctx, h2d(ctx, b.ymax, init, sizeof(init)));
    }
    FIPI_CUDA(ctx, A((void**)&b.it_mark, sizeof(int)));
    FIPI_CUDA(ctx, cudaMemsetAsync(b.it_mark, 0xff, sizeof(int), ctx->stream));
    FIPI_CUDA(ctx, A((void**)&b.tau, sizeof(double)));
    b.sp_prev_valid = 0;
    return FIPI_OK;
}

void particles_free(fipi_ctx* ctx) {
    ParticleBufs& b = ctx->pb;
    void* all[] = {b.p, b.p_old, b.u_old, b.f_pp, b.f_pi, b.r, b.cth, b.keys, b.keys_alt, b.ids, b.ids_alt,
                   b.cell_off, b.cell_cnt, b.sp_keys, b.sp_keys_alt, b.sp_vals, b.sp_vals_alt, b.sp_prev,
                   b.hist, b.tau_part, b.it_mark, b.tau, b.spos, b.sp_fw, b.ymax, b.sp_acc, b.uf, b.f_rand};
    for (void* p : all)
        if (p) cudaFree(p);
    b = ParticleBufs{};
}

// ------------------------------------------------------------ fine-grained entry points
// Host AoS (n x 3) <-> device SoA (3 x n) staging.
static fipi_status to_dev_soa(fipi_ctx* ctx, const double* h, double* d, int n) {
    std::vector<double> s((size_t)3 * n);
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) s[(size_t)a * n + i] = h[3 * i + a];
    FIPI_CUDA(ctx, h2d(ctx, d, s.data(), sizeof(double) * 3 * n));
    return FIPI_OK;
}

static fipi_status from_dev_soa(fipi_ctx* ctx, const double* d, double* h, int n) {
    std::vector<double> s((size_t)3 * n);
    FIPI_CUDA(ctx, d2h(ctx, s.data(), d, sizeof(double) * 3 * n));
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) h[3 * i + a] = s[(size_t)a * n + i];
    return FIPI_OK;
}

struct DevScratch {
    fipi_ctx* ctx;
    std::vector<void*> ptrs;
    template <typename X> X* get(size_t count) {
        void* p = nullptr;
        if (cudaMalloc(&p, sizeof(X) * (count ? count : 1)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return (X*)p;
    }
    ~DevScratch() {
        for (void* p : ptrs) cudaFree(p);
    }
};

static fipi_status read_status(fipi_ctx* ctx) {
    int st = 0;
    FIPI_CUDA(ctx, d2h(ctx, &st, ctx->status, sizeof(int)));
    FIPI_CUDA(ctx, cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->stream));
    if (st & ERR_NONFINITE) return set_error(ctx, FIPI_ERR_NONFINITE, "non-finite particle position");
    if (st & ERR_OUT_OF_RANGE)
        return set_error(ctx, FIPI_ERR_OUT_OF_RANGE, "particle out of sorting range (cluster.cpp:144-163)");
    return FIPI_OK;
}

__global__ void k_wrap_many(PC pc, double* p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pc.n) return;
    for (int a = 0; a < 3; ++a) p[3 * i + a] = wrap_exact(p[3 * i + a], pc.L[a]);  // element.cpp:177-185
}

fipi_status particles_wrap(fipi_ctx* ctx, double* p_host) {
    const int n = ctx->pb.n;
    if (n == 0) return FIPI_OK;
    DevScratch ds{ctx};
    double* pd = ds.get<double>(3 * (size_t)n);
    if (!pd) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    FIPI_CUDA(ctx, h2d(ctx, pd, p_host, sizeof(double) * 3 * n));
    const PC pc = make_pc(ctx);
    { LaunchScope ls_(ctx, "wrap", 0.0); k_wrap_many<<<(n + kPT - 1) / kPT, kPT, 0, ctx->stream>>>(pc, pd); }
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    FIPI_CUDA(ctx, d2h(ctx, p_host, pd, sizeof(double) * 3 * n));
    return FIPI_OK;
}

fipi_status particles_get_radii(fipi_ctx* ctx, double* r_host) {
    FIPI_CUDA(ctx, d2h(ctx, r_host, ctx->pb.r, sizeof(double) * ctx->pb.n));
    return FIPI_OK;
}

fipi_status particles_cells_build(fipi_ctx* ctx, const double* p, int* keys, int* sorted, int* offsets) {
    ParticleBufs& b = ctx->pb;
    const int n = b.n;
    DevScratch ds{ctx};
    double* pd = ds.get<double>(3 * (size_t)n);
    if (!pd) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    fipi_status st = to_dev_soa(ctx, p, pd, n);
    if (st != FIPI_OK) return st;
    build_cells(ctx, pd);
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    st = read_status(ctx);
    if (st != FIPI_OK) return st;
    // keys are needed per particle id: the sorted keys follow the sorted ids
    std::vector<unsigned> k(n), id(n);
    FIPI_CUDA(ctx, d2h(ctx, k.data(), b.keys, sizeof(unsigned) * n));
    FIPI_CUDA(ctx, d2h(ctx, id.data(), b.ids, sizeof(unsigned) * n));
    if (keys)
        for (int s = 0; s < n; ++s) keys[id[s]] = (int)k[s];
    if (sorted)
        for (int s = 0; s < n; ++s) sorted[s] = (int)id[s];
    if (offsets) FIPI_CUDA(ctx, d2h(ctx, offsets, b.cell_off, sizeof(int) * (b.ncells + 1)));
    return FIPI_OK;
}

fipi_status particles_f_pp(fipi_ctx* ctx, const double* p, int t, const double* f_pi, double* f_pp, double* tau) {
    ParticleBufs& b = ctx->pb;
    const int n = b.n;
    DevScratch ds{ctx};
    double* pd = ds.get<double>(3 * (size_t)n);
    double* fpid = ds.get<double>(3 * (size_t)n);
    double* fpp = ds.get<double>(3 * (size_t)n);
    if (!pd || !fpid || !fpp) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    fipi_status st = to_dev_soa(ctx, p, pd, n);
    if (st != FIPI_OK) return st;
    if (f_pi) {
        st = to_dev_soa(ctx, f_pi, fpid, n);
        if (st != FIPI_OK) return st;
    }
    build_cells(ctx, pd);
    const double rmp = ramp((double)t, 0.2 * ctx->P.t_end);
    double* rmpd = ds.get<double>(1);
    if (!rmpd) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    FIPI_CUDA(ctx, h2d(ctx, rmpd, &rmp, sizeof(double)));
    if (f_pi) FIPI_CUDA(ctx, cudaMemsetAsync(b.it_mark, 0xff, sizeof(int), ctx->stream));
    if (ctx->prec == FIPI_MIXED) f_pp_launch<float>(ctx, pd, rmpd, f_pi ? fpid : nullptr, fpp, f_pi != nullptr);
    else f_pp_launch<double>(ctx, pd, rmpd, f_pi ? fpid : nullptr, fpp, f_pi != nullptr);
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    st = read_status(ctx);
    if (st != FIPI_OK) return st;
    if (f_pp) {
        st = from_dev_soa(ctx, fpp, f_pp, n);
        if (st != FIPI_OK) return st;
    }
    if (tau) {
        if (f_pi) {
            st = particles_packing_tau(ctx, tau);
            if (st != FIPI_OK) return st;
        } else {
            *tau = 0.0;
        }
    }
    return FIPI_OK;
}

fipi_status particles_pairs(fipi_ctx* ctx, const double* p, int* pairs, int max_pairs, int* n_pairs) {
    ParticleBufs& b = ctx->pb;
    const int n = b.n;
    DevScratch ds{ctx};
    double* pd = ds.get<double>(3 * (size_t)n);
    int* cnt = ds.get<int>(n);
    int* offd = ds.get<int>(n);
    if (!pd || !cnt || !offd) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    fipi_status st = to_dev_soa(ctx, p, pd, n);
    if (st != FIPI_OK) return st;
    build_cells(ctx, pd);
    const PC pc = make_pc(ctx);
    const int blocks = (b.ncells * 32 + 255) / 256;
    { LaunchScope ls_(ctx, "contact forces (warp per cell)", 0.0); k_f_pp<double, 1><<<blocks, 256, 0, ctx->stream>>>(pc, pd, b.ids, b.cell_off, nullptr, nullptr, nullptr, nullptr,
                                                      nullptr, cnt, nullptr, nullptr); }
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    st = read_status(ctx);
    if (st != FIPI_OK) return st;
    std::vector<int> hc(n), ho(n);
    FIPI_CUDA(ctx, d2h(ctx, hc.data(), cnt, sizeof(int) * n));
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        ho[i] = (int)total;
        total += hc[i];
    }
    *n_pairs = (int)total;
    if (!pairs || total == 0) return FIPI_OK;
    int* pr = ds.get<int>(2 * (size_t)total);
    if (!pr) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    FIPI_CUDA(ctx, h2d(ctx, offd, ho.data(), sizeof(int) * n));
    { LaunchScope ls_(ctx, "contact forces (warp per cell)", 0.0); k_f_pp<double, 2><<<blocks, 256, 0, ctx->stream>>>(pc, pd, b.ids, b.cell_off, nullptr, nullptr, nullptr, nullptr,
                                                      nullptr, nullptr, offd, pr); }
    std::vector<int> hp(2 * (size_t)total);
    FIPI_CUDA(ctx, d2h(ctx, hp.data(), pr, sizeof(int) * 2 * total));
    std::vector<std::pair<int, int>> v((size_t)total);
    for (long long q = 0; q < total; ++q) v[q] = {hp[2 * q], hp[2 * q + 1]};
    std::sort(v.begin(), v.end());
    for (long long q = 0; q < total && q < max_pairs; ++q) {
        pairs[2 * q] = v[q].first;
        pairs[2 * q + 1] = v[q].second;
    }
    return FIPI_OK;
}

// field::interpolate2 (field.cpp:250-281): the trilinear products on the
// fractions m/3 + 1/3 of a size-3 stencil whose corners are the nodes i + 1
// and i + 2 (periodic), dead code in the reference's loop.
template <typename TF, typename TA>
__device__ __forceinline__ TA interp2(const PC& pc, double x, double y, double z, const TF* __restrict__ v) {
    const int size = 3;
    const double fx = floor(x / pc.dx), fy = floor(y / pc.dy), fz = floor(z / pc.dz);
    const int i = (int)fx, j = (int)fy, k = (int)fz;
    TA m = (TA)(x / pc.dx - fx), nn = (TA)(y / pc.dy - fy), o = (TA)(z / pc.dz - fz);
    m = m / size + TA(1.0) / size;
    nn = nn / size + TA(1.0) / size;
    o = o / size + TA(1.0) / size;
    const int Nx = pc.N[0], Ny = pc.N[1], Nz = pc.N[2];
    const int i0 = wrapi(i + 1 + Nx, Nx), i1 = wrapi(i + 2, Nx);
    const int j0 = wrapi(j + 1 + Ny, Ny), j1 = wrapi(j + 2, Ny);
    const int k0 = wrapi(k + 1 + Nz, Nz), k1 = wrapi(k + 2, Nz);
    return interp<TF, TA>(v, i0, j0, k0, i1, j1, k1, m, nn, o, Nx, Ny);
}

template <typename T, bool WIDE>
__global__ void k_interp_many(PC pc, const T* __restrict__ fields, int nf, size_t V, const double* __restrict__ p,
                              double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pc.n) return;
    const double x = p[i], y = p[pc.n + i], z = p[2 * pc.n + i];
    for (int f = 0; f < nf; ++f) {
        const T* fl[1] = {fields + (size_t)f * V};
        T v;
        if (WIDE) v = interp2<T, T>(pc, x, y, z, fl[0]);
        else interp_fields<T, T>(pc, x, y, z, fl, 1, &v);
        out[(size_t)i * nf + f] = (double)v;
    }
}

static fipi_status interpolate_impl(fipi_ctx* ctx, const double* fields, int nfields, const double* p, double* out,
                                    bool wide);

fipi_status particles_interpolate(fipi_ctx* ctx, const double* fields, int nfields, const double* p, double* out) {
    return interpolate_impl(ctx, fields, nfields, p, out, false);
}

fipi_status particles_interpolate2(fipi_ctx* ctx, const double* fields, int nfields, const double* p, double* out) {
    return interpolate_impl(ctx, fields, nfields, p, out, true);
}

static fipi_status interpolate_impl(fipi_ctx* ctx, const double* fields, int nfields, const double* p, double* out,
                                    bool wide) {
    const int n = ctx->pb.n;
    const size_t V = (size_t)ctx->g.V;
    DevScratch ds{ctx};
    double* pd = ds.get<double>(3 * (size_t)n);
    double* od = ds.get<double>((size_t)n * nfields);
    if (!pd || !od) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    fipi_status st = to_dev_soa(ctx, p, pd, n);
    if (st != FIPI_OK) return st;
    const PC pc = make_pc(ctx);
    if (ctx->prec == FIPI_MIXED) {
        std::vector<float> hf(V * nfields);
        for (size_t i = 0; i < V * nfields; ++i) hf[i] = (float)fields[i];
        float* fd = ds.get<float>(V * nfields);
        if (!fd) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
        FIPI_CUDA(ctx, h2d(ctx, fd, hf.data(), sizeof(float) * V * nfields));
        { LaunchScope ls_(ctx, "interpolate", 0.0);
          if (wide) k_interp_many<float, true><<<(n + 255) / 256, 256, 0, ctx->stream>>>(pc, fd, nfields, V, pd, od);
          else k_interp_many<float, false><<<(n + 255) / 256, 256, 0, ctx->stream>>>(pc, fd, nfields, V, pd, od); }
    } else {
        double* fd = ds.get<double>(V * nfields);
        if (!fd) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
        FIPI_CUDA(ctx, h2d(ctx, fd, fields, sizeof(double) * V * nfields));
        { LaunchScope ls_(ctx, "interpolate", 0.0);
          if (wide) k_interp_many<double, true><<<(n + 255) / 256, 256, 0, ctx->stream>>>(pc, fd, nfields, V, pd, od);
          else k_interp_many<double, false><<<(n + 255) / 256, 256, 0, ctx->stream>>>(pc, fd, nfields, V, pd, od); }
    }
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    FIPI_CUDA(ctx, d2h(ctx, out, od, sizeof(double) * n * nfields));
    return FIPI_OK;
}

__global__ void k_f_pi_many(PC pc, const double* __restrict__ c_loc, const double* __restrict__ dcdx,
                            const double* __restrict__ r, const double* __restrict__ cth, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pc.n) return;
    double f[3];
    f_pi_of(pc, c_loc[i], dcdx[3 * i], dcdx[3 * i + 1], dcdx[3 * i + 2], r ? r[i] : pc.r_p, cth ? cth[i] : 0.0, f);
    for (int a = 0; a < 3; ++a) out[3 * i + a] = f[a];
}

fipi_status particles_f_pi(fipi_ctx* ctx, const double* c_loc, const double* dcdx, const double* r, const double* cth,
                           double* f_pi) {
    const int n = ctx->pb.n;
    DevScratch ds{ctx};
    double* cd = ds.get<double>(n);
    double* gd = ds.get<double>(3 * (size_t)n);
    double* rd = r ? ds.get<double>(n) : nullptr;
    double* td = cth ? ds.get<double>(n) : nullptr;
    double* od = ds.get<double>(3 * (size_t)n);
    if (!cd || !gd || !od) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    FIPI_CUDA(ctx, h2d(ctx, cd, c_loc, sizeof(double) * n));
    FIPI_CUDA(ctx, h2d(ctx, gd, dcdx, sizeof(double) * 3 * n));
    if (rd) FIPI_CUDA(ctx, h2d(ctx, rd, r, sizeof(double) * n));
    if (td) FIPI_CUDA(ctx, h2d(ctx, td, cth, sizeof(double) * n));
    const PC pc = make_pc(ctx);
    { LaunchScope ls_(ctx, "f_pi", 0.0); k_f_pi_many<<<(n + 255) / 256, 256, 0, ctx->stream>>>(pc, cd, gd, rd, td, od); }
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    FIPI_CUDA(ctx, d2h(ctx, f_pi, od, sizeof(double) * 3 * n));
    return FIPI_OK;
}

__global__ void k_advect_many(PC pc, int stage, const double* __restrict__ fpi, const double* __restrict__ fpp,
                              const double* __restrict__ r, double* p, double* po, double* uo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pc.n) return;
    advect_one(pc, stage, fpi + 3 * i, fpp + 3 * i, r ? r[i] : pc.r_p, p + 3 * i, po + 3 * i, uo + 3 * i);
}

fipi_status particles_advect(fipi_ctx* ctx, int stage, const double* f_pi, const double* f_pp, const double* r,
                             double* p, double* p_old, double* u_old) {
    const int n = ctx->pb.n;
    DevScratch ds{ctx};
    const size_t b3 = sizeof(double) * 3 * n;
    double* a = ds.get<double>(3 * (size_t)n);
    double* bpp = ds.get<double>(3 * (size_t)n);
    double* rd = r ? ds.get<double>(n) : nullptr;
    double* pd = ds.get<double>(3 * (size_t)n);
    double* pod = ds.get<double>(3 * (size_t)n);
    double* uod = ds.get<double>(3 * (size_t)n);
    if (!a || !bpp || !pd || !pod || !uod) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    FIPI_CUDA(ctx, h2d(ctx, a, f_pi, b3));
    FIPI_CUDA(ctx, h2d(ctx, bpp, f_pp, b3));
    if (rd) FIPI_CUDA(ctx, h2d(ctx, rd, r, sizeof(double) * n));
    FIPI_CUDA(ctx, h2d(ctx, pd, p, b3));
    FIPI_CUDA(ctx, h2d(ctx, pod, p_old, b3));
    FIPI_CUDA(ctx, h2d(ctx, uod, u_old, b3));
    const PC pc = make_pc(ctx);
    { LaunchScope ls_(ctx, "advect", 0.0); k_advect_many<<<(n + 255) / 256, 256, 0, ctx->stream>>>(pc, stage, a, bpp, rd, pd, pod, uod); }
    FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    FIPI_CUDA(ctx, d2h(ctx, p, pd, b3));
    FIPI_CUDA(ctx, d2h(ctx, p_old, pod, b3));
    FIPI_CUDA(ctx, d2h(ctx, u_old, uod, b3));
    return FIPI_OK;
}

fipi_status particles_spread_host(fipi_ctx* ctx, const double* p, const double* f_pp, double* out) {
    ParticleBufs& b = ctx->pb;
    const int n = b.n;
    const size_t V = (size_t)ctx->g.V;
    DevScratch ds{ctx};
    double* pd = ds.get<double>(3 * (size_t)n);
    double* fd = ds.get<double>(3 * (size_t)n);
    if (!pd || !fd) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
    fipi_status st = to_dev_soa(ctx, p, pd, n);
    if (st != FIPI_OK) return st;
    st = to_dev_soa(ctx, f_pp, fd, n);
    if (st != FIPI_OK) return st;
    if (ctx->prec == FIPI_MIXED) {
        float* g = ds.get<float>(3 * V);
        if (!g) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
        FIPI_CUDA(ctx, cudaMemsetAsync(g, 0, sizeof(float) * 3 * V, ctx->stream));
        float* f3[3] = {g, g + V, g + 2 * V};
        spread_t<float>(ctx, pd, fd, f3, false);
        std::vector<float> h(3 * V);
        FIPI_CUDA(ctx, cudaMemcpyAsync(h.data(), g, sizeof(float) * 3 * V, cudaMemcpyDeviceToHost, ctx->stream));
        FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (size_t i = 0; i < 3 * V; ++i) out[i] = h[i];
    } else {
        double* g = ds.get<double>(3 * V);
        if (!g) return set_error(ctx, FIPI_ERR_CUDA, "cudaMalloc failed");
        FIPI_CUDA(ctx, cudaMemsetAsync(g, 0, sizeof(double) * 3 * V, ctx->stream));
        double* f3[3] = {g, g + V, g + 2 * V};
        spread_t<double>(ctx, pd, fd, f3, false);
        FIPI_CUDA(ctx, cudaMemcpyAsync(out, g, sizeof(double) * 3 * V, cudaMemcpyDeviceToHost, ctx->stream));
        FIPI_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return FIPI_OK;
}

// ------------------------------------------------------------ step index
__global__ void k_set_tick(int* d_t, double* d_rmp, int t, double thr) {
    *d_t = t;
    const double x = (double)(t + 1);
    *d_rmp = (x < 0) ? 0.0 : (x < thr ? x / thr : 1.0);
}

void set_tick(fipi_ctx* ctx, int t) {
    LaunchScope ls_(ctx, "step tick", 0.0);
    k_set_tick<<<1, 1, 0, ctx->stream>>>(ctx->d_t, ctx->d_rmp, t, 0.2 * ctx->P.t_end);
}

// ------------------------------------------------------------ adjoint
// Reverse mode of the two Heun stages (element.cpp:156-185,
// cluster.cpp:174-275, element.cpp:75-97, field.cpp:223-248) and of the
// spreading (cluster.cpp:344-410), FP64.  Branches (interpolation cell,
// |phi| <= tanh 2, |d| < r, |d| < r_eq) are those of the forward step.

// Trilinear value and position gradient of v at (x, y, z) (field.cpp:223-248).
__device__ __forceinline__ void interp_grad(const PC& pc, double x, double y, double z, const double* __restrict__ v,
                                            double g[3]) {
    const double fx = floor(x / pc.dx), fy = floor(y / pc.dy), fz = floor(z / pc.dz);
    const int i = wrapi((int)fx, pc.N[0]), j = wrapi((int)fy, pc.N[1]), k = wrapi((int)fz, pc.N[2]);
    const double m = x / pc.dx - fx, nn = y / pc.dy - fy, o = z / pc.dz - fz;
    const int i1 = (i + 1) % pc.N[0], j1 = (j + 1) % pc.N[1], k1 = (k + 1) % pc.N[2];
    const size_t sy = (size_t)pc.N[0], sz = (size_t)pc.N[0] * pc.N[1];
    const double v000 = v[i + j * sy + k * sz], v100 = v[i1 + j * sy + k * sz];
    const double v010 = v[i + j1 * sy + k * sz], v110 = v[i1 + j1 * sy + k * sz];
    const double v001 = v[i + j * sy + k1 * sz], v101 = v[i1 + j * sy + k1 * sz];
    const double v011 = v[i + j1 * sy + k1 * sz], v111 = v[i1 + j1 * sy + k1 * sz];
    const double dm = (1 - nn) * (1 - o) * (v100 - v000) + nn * (1 - o) * (v110 - v010) +
                      (1 - nn) * o * (v101 - v001) + nn * o * (v111 - v011);
    const double dn = (1 - m) * (1 - o) * (v010 - v000) + m * (1 - o) * (v110 - v100) +
                      (1 - m) * o * (v011 - v001) + m * o * (v111 - v101);
    const double dd = (1 - m) * (1 - nn) * (v001 - v000) + m * (1 - nn) * (v101 - v100) +
                      (1 - m) * nn * (v011 - v010) + m * nn * (v111 - v110);
    g[0] = dm / pc.dx;
    g[1] = dn / pc.dy;
    g[2] = dd / pc.dz;
}

// Adjoint of f_pi_of: lf = cotangent of f_pi -> cotangents of phi and grad c,
// and of the parameters: lct (the particle's cos theta: df_pi/dct = A pi r
// sigma n) and lsig (sigma through f_pi alone: df_pi/dsigma = -A pi (d - r ct) n).
__device__ __forceinline__ void f_pi_adj(const PC& pc, double phi, double gx, double gy, double gz, double r, double ct,
                                         const double lf[3], double* lphi, double lg[3], double* lct, double* lsig) {
    const double gn = sqrt(gx * gx + gy * gy + gz * gz);
    *lphi = 0.0;
    *lct = *lsig = 0.0;
    lg[0] = lg[1] = lg[2] = 0.0;
    if (!(fabs(phi) <= pc.tanh2 && gn != 0.0)) return;
    const double s2e = 1.4142135623730951 * pc.epsilon;
    const double d = 0.5 * log((1.0 + phi) / (1.0 - phi)) * s2e;
    double f_mag = 0.0, dmag = 0.0;
    const bool on = fabs(d) < r;
    if (on) {
        f_mag = -pc.A * pc.pi * (d - r * ct) * pc.sigma;
        dmag = -pc.A * pc.pi * pc.sigma * s2e / (1.0 - phi * phi);  // d(d)/d(phi) = sqrt2 eps / (1 - phi^2)
    }
    const double nh[3] = {gx / gn, gy / gn, gz / gn};
    const double s = nh[0] * lf[0] + nh[1] * lf[1] + nh[2] * lf[2];
    *lphi = s * dmag;
    for (int a = 0; a < 3; ++a) lg[a] = f_mag / gn * (lf[a] - nh[a] * s);
    if (on) {
        *lct = s * pc.A * pc.pi * r * pc.sigma;
        *lsig = s * (-pc.A * pc.pi * (d - r * ct));
    }
}

// Forward recompute of one stage's interpolation (c, grad c) and f_pi.
__global__ void k_adj_interp(PC pc, const double* __restrict__ p, const double* __restrict__ c,
                             const double* __restrict__ g0, const double* __restrict__ g1,
                             const double* __restrict__ g2, const double* __restrict__ r,
                             const double* __restrict__ cth, double* loc, double* fpi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (i >= n) return;
    const double* fl[4] = {c, g0, g1, g2};
    double vals[4];
    interp_fields<double, double>(pc, p[i], p[n + i], p[2 * n + i], fl, 4, vals);
    for (int q = 0; q < 4; ++q) loc[q * n + i] = vals[q];
    if (fpi) {
        double f[3];
        f_pi_of(pc, vals[0], vals[1], vals[2], vals[3], r[i], cth[i], f);
        for (int a = 0; a < 3; ++a) fpi[a * n + i] = f[a];
    }
}

// Stage-1 advection recomputed: p1 = wrap(p + dt (f_pi + f_pp)/(6 pi mu r)).
__global__ void k_adj_advect1(PC pc, const double* __restrict__ p0, const double* __restrict__ fpi,
                              const double* __restrict__ fpp, const double* __restrict__ r, double* p1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (i >= n) return;
    double pp[3] = {p0[i], p0[n + i], p0[2 * n + i]}, po[3], uo[3];
    const double a[3] = {fpi[i], fpi[n + i], fpi[2 * n + i]};
    const double b[3] = {fpp[i], fpp[n + i], fpp[2 * n + i]};
    advect_one(pc, 1, a, b, r[i], pp, po, uo);
    for (int q = 0; q < 3; ++q) p1[q * n + i] = pp[q];
}

// Adjoint of one stage at positions p: given the cotangent lv of this
// stage's velocity, writes the cotangent of its contact forces (lamF =
// kappa lv + extra), of the interpolated values (lamloc, 4n) and of p
// through the interpolation (lam_p = base + ...), kappa = 1/(6 pi mu r).
//   stage 2: lv = dt/2 lp_end,              extra = lfpp_end, base = 0
//   stage 1: lv = dt/2 lp_end + dt lam_p1,  extra = 0,        base = lp_end + lam_p1
__global__ void k_adj_stage(PC pc, int stage, const double* __restrict__ p, const double* __restrict__ c,
                            const double* __restrict__ g0, const double* __restrict__ g1,
                            const double* __restrict__ g2, const double* __restrict__ loc,
                            const double* __restrict__ r, const double* __restrict__ cth,
                            const double* lp_end, const double* __restrict__ lfpp_end,
                            const double* __restrict__ lam_p1_in, double* lamF, double* lamloc, double* lam_p,
                            double* dct, double* psig) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (i >= n) return;
    const double kappa = 1.0 / 6.0 / pc.pi / pc.mu / r[i];
    double lv[3], lf[3];
    for (int a = 0; a < 3; ++a) {
        lv[a] = 0.5 * pc.dt * lp_end[a * n + i];
        if (stage == 1) lv[a] += pc.dt * lam_p1_in[a * n + i];
        lf[a] = kappa * lv[a];
        lamF[a * n + i] = lf[a] + (stage == 2 ? lfpp_end[a * n + i] : 0.0);
    }
    double lphi, lg[3], lct, lsig;
    f_pi_adj(pc, loc[i], loc[n + i], loc[2 * n + i], loc[3 * n + i], r[i], cth[i], lf, &lphi, lg, &lct, &lsig);
    dct[i] += lct;
    psig[i] += lsig;
    lamloc[i] = lphi;
    for (int a = 0; a < 3; ++a) lamloc[(1 + a) * n + i] = lg[a];
    const double x = p[i], y = p[n + i], z = p[2 * n + i];
    double acc[3], gr[3];
    interp_grad(pc, x, y, z, c, gr);
    for (int a = 0; a < 3; ++a) acc[a] = lphi * gr[a];
    const double* gf[3] = {g0, g1, g2};
    for (int d = 0; d < 3; ++d) {
        interp_grad(pc, x, y, z, gf[d], gr);
        for (int a = 0; a < 3; ++a) acc[a] += lg[d] * gr[a];
    }
    for (int a = 0; a < 3; ++a) {
        double base = 0.0;
        if (stage == 1) base = lp_end[a * n + i] + lam_p1_in[a * n + i];
        lam_p[a * n + i] = base + acc[a];
    }
}

// Adjoint of compute_f_pp with respect to positions: for every pair of the
// forward evaluation (same cells, minimum-image rule of cluster.cpp:225-232
// and |d| < r_eq test), lam_p[i] += J(d) (lamF[i] - lamF[j]) with
// J = ramp k_n ((r_eq/|d| - 1) I - r_eq d d^T / |d|^3), which is even in d.
// With respect to k_n: pkn[i] += lamF[i] . (force on i) / k_n, the force on
// i being +F(d) when i < j and -F(d) otherwise (f_pp[it] += F, f_pp[id] -= F,
// cluster.cpp:246-255), F(d) = (r_eq - |d|) ramp k_n d / |d|.
// Warp per home cell, lane per home particle as in k_f_pp; coincident pairs
// (random separation in the reference) contribute nothing.
__global__ void k_f_pp_adj(PC pc, const double* __restrict__ p, const unsigned* __restrict__ ids,
                           const int* __restrict__ off, const double* __restrict__ rmp_p,
                           const double* __restrict__ lamF, double* lam_p, double* pkn) {
    const int lane = threadIdx.x & 31;
    const int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int ncells = pc.nc[0] * pc.nc[1] * pc.nc[2];
    if (cell >= ncells) return;
    const int n = pc.n;
    const int ci = cell % pc.nc[0], cj = (cell / pc.nc[0]) % pc.nc[1], ck = cell / (pc.nc[0] * pc.nc[1]);
    const int beg = off[cell], end = off[cell + 1];
    const double T0 = pc.dc[0] * (pc.nc[0] - 2), T1 = pc.dc[1] * (pc.nc[1] - 2), T2 = pc.dc[2] * (pc.nc[2] - 2);
    const double sc = (*rmp_p) * pc.k_n;
    for (int base = beg; base < end; base += 32) {
        const int s = base + lane;
        const bool active = s < end;
        const int i = active ? (int)ids[s] : 0;
        const double xi = p[i], yi = p[n + i], zi = p[2 * n + i];
        const double li[3] = {lamF[i], lamF[n + i], lamF[2 * n + i]};
        double acc[3] = {0.0, 0.0, 0.0};
        double acc_kn = 0.0;
        for (int dk = -1; dk <= 1; ++dk)
            for (int dj = -1; dj <= 1; ++dj)
                for (int di = -1; di <= 1; ++di) {
                    const int co = (ci + di + pc.nc[0]) % pc.nc[0] + (cj + dj + pc.nc[1]) % pc.nc[1] * pc.nc[0] +
                                   (ck + dk + pc.nc[2]) % pc.nc[2] * pc.nc[0] * pc.nc[1];
                    const int qe = off[co + 1];
                    for (int q = off[co]; q < qe; ++q) {
                        const int j = (int)ids[q];
                        if (!active || j == i) continue;
                        double d[3];
                        if (i < j) {
                            d[0] = xi - p[j];
                            d[1] = yi - p[n + j];
                            d[2] = zi - p[2 * n + j];
                        } else {
                            d[0] = p[j] - xi;
                            d[1] = p[n + j] - yi;
                            d[2] = p[2 * n + j] - zi;
                        }
                        if (d[0] > T0) d[0] = d[0] - pc.L[0];
                        else if (d[0] < -T0) d[0] = d[0] + pc.L[0];
                        if (d[1] > T1) d[1] = d[1] - pc.L[1];
                        else if (d[1] < -T1) d[1] = d[1] + pc.L[1];
                        if (d[2] > T2) d[2] = d[2] - pc.L[2];
                        else if (d[2] < -T2) d[2] = d[2] + pc.L[2];
                        const double dn = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                        if (!(dn < pc.r_eq) || dn == 0.0) continue;
                        const double dl[3] = {li[0] - lamF[j], li[1] - lamF[n + j], li[2] - lamF[2 * n + j]};
                        const double a = pc.r_eq / dn - 1.0;
                        const double b = pc.r_eq / (dn * dn * dn) * (d[0] * dl[0] + d[1] * dl[1] + d[2] * dl[2]);
                        for (int e = 0; e < 3; ++e) acc[e] += sc * (a * dl[e] - b * d[e]);
                        const double fk = (pc.r_eq - dn) * (*rmp_p) / dn * (d[0] * li[0] + d[1] * li[1] + d[2] * li[2]);
                        acc_kn += (i < j) ? fk : -fk;
                    }
                }
        if (active) {
            for (int e = 0; e < 3; ++e) lam_p[e * n + i] += acc[e];
            pkn[i] += acc_kn;
        }
    }
}

// Spreading records of the interpolation adjoint: 8 corners of each of the
// 2n interpolations (entity e = stage * n + i), node keys, fractions and
// the 4 cotangents per entity.
__global__ void k_adj_records(PC pc, const double* __restrict__ p0, const double* __restrict__ p1,
                              const double* __restrict__ lamloc, unsigned* keys, unsigned* vals, double* rw) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (e >= 2 * n) return;
    const int st = e / n, i = e - st * n;
    const double* p = st == 0 ? p0 : p1;
    int ix[3];
    double fr[3];
    cell_and_frac(pc, p[i], p[n + i], p[2 * n + i], ix, fr);
    for (int c = 0; c < 8; ++c) {
        const int x = (ix[0] + c_corner[c][0]) % pc.N[0];
        const int y = (ix[1] + c_corner[c][1]) % pc.N[1];
        const int z = (ix[2] + c_corner[c][2]) % pc.N[2];
        keys[8 * e + c] = (unsigned)(x + (size_t)y * pc.N[0] + (size_t)z * pc.N[0] * pc.N[1]);
        vals[8 * e + c] = (unsigned)(8 * e + c);
    }
    const int m = 2 * n;
    for (int a = 0; a < 3; ++a) rw[a * m + e] = fr[a];
    for (int q = 0; q < 4; ++q) rw[(3 + q) * m + e] = lamloc[(st * 4 + q) * n + i];
}

// Sorted segmented reduction of the records: part[q][node] = sum of w_c lam_q
// in ascending record order (deterministic, no atomics).
__global__ void k_adj_reduce(const unsigned* __restrict__ keys, const unsigned* __restrict__ vals, int m, int ne,
                             const double* __restrict__ rw, double* part, size_t V) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    const unsigned node = keys[s];
    if (s > 0 && keys[s - 1] == node) return;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int q = s; q < m && keys[q] == node; ++q) {
        const unsigned rec = vals[q];
        const int e = (int)(rec >> 3), c = (int)(rec & 7u);
        const double o = rw[e], pp = rw[ne + e], qq = rw[2 * ne + e];
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[k] += corner_value<double>(rw[(3 + k) * ne + e], c, o, pp, qq);
    }
    for (int k = 0; k < 4; ++k) part[k * V + node] = acc[k];
}

// Adjoint of the spreading of f_pp^n at p^n given lamF (3 real fields).
__global__ void k_adj_spread(PC pc, const double* __restrict__ p, const double* __restrict__ fpp,
                             const double* __restrict__ lamF, size_t V, double* la_fpp, double* la_p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = pc.n;
    if (i >= n) return;
    const double x = p[i], y = p[n + i], z = p[2 * n + i];
    const double inv = 1.0 / pc.dx / pc.dy / pc.dz;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < 3; ++d) {
        const double* f = lamF + d * V;
        const double* fl[1] = {f};
        double val;
        interp_fields<double, double>(pc, x, y, z, fl, 1, &val);
        la_fpp[d * n + i] = val * inv;
        double gr[3];
        interp_grad(pc, x, y, z, f, gr);
        const double w = fpp[d * n + i] * inv;
        for (int a = 0; a < 3; ++a) acc[a] += w * gr[a];
    }
    for (int a = 0; a < 3; ++a) la_p[a * n + i] += acc[a];
}

fipi_status particles_adjoint_alloc(fipi_ctx* ctx) {
    AdjBufs& a = ctx->ad;
    const int n = ctx->pb.n > 0 ? ctx->pb.n : 1;
    auto A = [&](void** ptr, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(ptr, bytes);
        if (e == cudaSuccess) {
            ctx->device_bytes += bytes;
            e = cudaMemsetAsync(*ptr, 0, bytes, ctx->stream);
        }
        return e;
    };
    const size_t b3 = sizeof(double) * 3 * n;
    double** v3[] = {&a.la_p, &a.la_fpp, &a.tp0, &a.tfpp0, &a.p1, &a.fpi1, &a.fpp1, &a.lamF1, &a.lamF2, &a.lam_p1};
    for (double** q : v3) FIPI_CUDA(ctx, A((void**)q, b3));
    double** v1[] = {&a.dct, &a.pp_sig, &a.pp_kn};
    for (double** q : v1) FIPI_CUDA(ctx, A((void**)q, sizeof(double) * n));
    FIPI_CUDA(ctx, A((void**)&a.loc, sizeof(double) * 8 * n));
    FIPI_CUDA(ctx, A((void**)&a.lamloc, sizeof(double) * 8 * n));
    unsigned** r16[] = {&a.rk, &a.rv, &a.rk2, &a.rv2};
    for (unsigned** q : r16) FIPI_CUDA(ctx, A((void**)q, sizeof(unsigned) * 16 * n));
    FIPI_CUDA(ctx, A((void**)&a.rw, sizeof(double) * 14 * n));
    FIPI_CUDA(ctx, A((void**)&a.rmp, sizeof(double)));
    return FIPI_OK;
}

void particles_adjoint_free(fipi_ctx* ctx) {
    AdjBufs& a = ctx->ad;
    void* all[] = {a.la_p, a.la_fpp, a.tp0, a.tfpp0, a.p1, a.fpi1, a.fpp1, a.lamF1, a.lamF2, a.lam_p1,
                   a.loc, a.lamloc, a.rk, a.rv, a.rk2, a.rv2, a.rw, a.rmp, a.dct, a.pp_sig, a.pp_kn};
    for (void* p : all)
        if (p) cudaFree(p);
    a.la_p = a.la_fpp = a.tp0 = a.tfpp0 = a.p1 = a.fpi1 = a.fpp1 = a.lamF1 = a.lamF2 = a.lam_p1 = nullptr;
    a.dct = a.pp_sig = a.pp_kn = nullptr;
    a.loc = a.lamloc = a.rw = a.rmp = nullptr;
    a.rk = a.rv = a.rk2 = a.rv2 = nullptr;
}

// Runs after the taped forward step: ctx->fb.c, fb.g hold c^{n+1}, grad c^{n+1};
// a.tp0 holds p^n, a.rmp the ramp(t + 1, 0.2 t_end) factor of the reversed step.
fipi_status particles_adjoint(fipi_ctx* ctx) {
    ParticleBufs& b = ctx->pb;
    AdjBufs& a = ctx->ad;
    const PC pc = make_pc(ctx);
    const int n = b.n;
    const int nb = (n + 255) / 256;
    const double* c = (const double*)ctx->fb.c;
    const double* g0 = (const double*)ctx->fb.g[0];
    const double* g1 = (const double*)ctx->fb.g[1];
    const double* g2 = (const double*)ctx->fb.g[2];
    const int cells_blocks = (b.ncells * 32 + 255) / 256;
    // stage 1 recomputed at p^n: interpolation, f_pi, contact forces, p1
    { LaunchScope ls_(ctx, "adjoint: interpolate + f_pi", 0.0); k_adj_interp<<<nb, 256, 0, ctx->stream>>>(pc, a.tp0, c, g0, g1, g2, b.r, b.cth, a.loc, a.fpi1); }
    build_cells(ctx, a.tp0);
    { LaunchScope ls_(ctx, "adjoint: contact forces", 0.0); k_f_pp<double, 0><<<cells_blocks, 256, 0, ctx->stream>>>(pc, a.tp0, b.ids, b.cell_off, a.rmp, nullptr, b.it_mark, a.fpp1, nullptr, nullptr, nullptr, nullptr); }
    { LaunchScope ls_(ctx, "adjoint: advect", 0.0); k_adj_advect1<<<nb, 256, 0, ctx->stream>>>(pc, a.tp0, a.fpi1, a.fpp1, b.r, a.p1); }
    { LaunchScope ls_(ctx, "adjoint: interpolate", 0.0); k_adj_interp<<<nb, 256, 0, ctx->stream>>>(pc, a.p1, c, g0, g1, g2, b.r, b.cth, a.loc + 4 * n, nullptr); }
    // stage 2 reversed at p1
    // per-particle terms of this step's sigma (f_pi) and k_n cotangents
    FIPI_CUDA(ctx, cudaMemsetAsync(a.pp_sig, 0, sizeof(double) * n, ctx->stream));
    FIPI_CUDA(ctx, cudaMemsetAsync(a.pp_kn, 0, sizeof(double) * n, ctx->stream));
    { LaunchScope ls_(ctx, "adjoint: stage", 0.0); k_adj_stage<<<nb, 256, 0, ctx->stream>>>(pc, 2, a.p1, c, g0, g1, g2, a.loc + 4 * n, b.r, b.cth, a.la_p, a.la_fpp, nullptr, a.lamF2, a.lamloc + 4 * n, a.lam_p1, a.dct, a.pp_sig); }
    build_cells(ctx, a.p1);
    { LaunchScope ls_(ctx, "adjoint: contact forces", 0.0); k_f_pp_adj<<<cells_blocks, 256, 0, ctx->stream>>>(pc, a.p1, b.ids, b.cell_off, a.rmp, a.lamF2, a.lam_p1, a.pp_kn); }
    // stage 1 reversed at p^n (la_p becomes the start-state cotangent)
    { LaunchScope ls_(ctx, "adjoint: stage", 0.0); k_adj_stage<<<nb, 256, 0, ctx->stream>>>(pc, 1, a.tp0, c, g0, g1, g2, a.loc, b.r, b.cth, a.la_p, nullptr, a.lam_p1, a.lamF1, a.lamloc, a.la_p, a.dct, a.pp_sig); }
    build_cells(ctx, a.tp0);
    { LaunchScope ls_(ctx, "adjoint: contact forces", 0.0); k_f_pp_adj<<<cells_blocks, 256, 0, ctx->stream>>>(pc, a.tp0, b.ids, b.cell_off, a.rmp, a.lamF1, a.la_p, a.pp_kn); }
    param_acc(ctx, a.pp_sig, n, 1.0, a.pg + kPgSigmaAttach);
    param_acc(ctx, a.pp_kn, n, 1.0, a.pg + kPgKn);
    // interpolation adjoint onto the grid: part = [c, g0, g1, g2] cotangents
    const int m = 16 * n;
    { LaunchScope ls_(ctx, "adjoint: records", 0.0); k_adj_records<<<(2 * n + 255) / 256, 256, 0, ctx->stream>>>(pc, a.tp0, a.p1, a.lamloc, a.rk, a.rv, a.rw); }
    radix_sort(ctx, a.rk, a.rv, a.rk2, a.rv2, m, bits_for(ctx->g.V - 1));
    FIPI_CUDA(ctx, cudaMemsetAsync(a.part, 0, sizeof(double) * 4 * (size_t)ctx->g.V, ctx->stream));
    { LaunchScope ls_(ctx, "adjoint: records reduce", 0.0); k_adj_reduce<<<(m + 255) / 256, 256, 0, ctx->stream>>>(a.rk, a.rv, m, 2 * n, a.rw, a.part, (size_t)ctx->g.V); }
    FIPI_CUDA(ctx, cudaGetLastError());
    return FIPI_OK;
}

void particles_adjoint_spread(fipi_ctx* ctx) {
    AdjBufs& a = ctx->ad;
    const PC pc = make_pc(ctx);
    const int n = ctx->pb.n;
    LaunchScope ls_(ctx, "adjoint: spread", 0.0);
    k_adj_spread<<<(n + 255) / 256, 256, 0, ctx->stream>>>(pc, a.tp0, a.tfpp0, a.lamF, (size_t)ctx->g.V, a.la_fpp, a.la_p);
}

}  // namespace fipi

// ------------------------------------------------------------ no-allocation cell list
// A variant of the cell-list build (cluster::sorting) for callers that may
// not allocate device memory: code that runs inside a host framework owning
// a fixed device-memory pool, real-time loops that forbid driver
// allocations, or any caller that only hands over buffers it already has.
// Its scratch (positions in SoA order, radix-sort ping-pong arrays,
// histograms, the error word) lives in the file-scope array below, sized
// for at most FIPI_NOALLOC_MAX_PARTICLES particles.  Every GPU that loads
// this library holds the array until the process exits.
namespace fipi {
namespace {

constexpr int kNoallocMaxN = FIPI_NOALLOC_MAX_PARTICLES;
constexpr int kNoallocHistBlocks = kNoallocMaxN / RS_TILE + 1;
constexpr size_t kNoallocPos = 0;                                                 // double[3 n]
constexpr size_t kNoallocKA = kNoallocPos + sizeof(double) * 3 * kNoallocMaxN;    // unsigned[n]
constexpr size_t kNoallocKB = kNoallocKA + sizeof(unsigned) * kNoallocMaxN;       // unsigned[n]
constexpr size_t kNoallocIB = kNoallocKB + sizeof(unsigned) * kNoallocMaxN;       // unsigned[n]
constexpr size_t kNoallocHist = kNoallocIB + sizeof(unsigned) * kNoallocMaxN;     // unsigned[256 blocks]
constexpr size_t kNoallocStatus = kNoallocHist + sizeof(unsigned) * 256 * kNoallocHistBlocks;  // int
constexpr size_t kNoallocBytes = kNoallocStatus + 256;

static __device__ __align__(256) unsigned char g_cells_scratch[kNoallocBytes];

// Device address of g_cells_scratch per device, looked up once per device.
std::mutex g_noalloc_mu;
void* g_noalloc_addr[256] = {};

__global__ void k_aos_to_soa(const double* __restrict__ aos, double* __restrict__ soa, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int a = 0; a < 3; ++a) soa[(size_t)a * n + i] = aos[3 * (size_t)i + a];
}

}  // namespace
}  // namespace fipi

extern "C" fipi_status fipi_cells_build_noalloc(const fipi_params* P, const double* d_pos, int* d_keys,
                                                int* d_sorted, int* d_offsets, void* stream) {
    using namespace fipi;
    if (!P || !d_pos || !d_keys || !d_sorted || !d_offsets)
        return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    const int n = P->n_p;
    if (n <= 0) return set_error(nullptr, FIPI_ERR_BAD_ARG, "n_p must be positive");
    if (n > kNoallocMaxN)
        return set_error(nullptr, FIPI_ERR_UNSUPPORTED,
                         "n_p = " + std::to_string(n) + " exceeds the " + std::to_string(kNoallocMaxN) +
                             "-particle scratch of fipi_cells_build_noalloc");
    int nc[3];
    double dc[3];
    const fipi_status gs = fipi_cell_geometry(P, nc, dc);  // checks r_c and the cell counts' range
    if (gs != FIPI_OK) return gs;
    if (nc[0] < 1 || nc[1] < 1 || nc[2] < 1)
        return set_error(nullptr, FIPI_ERR_BAD_PARAMS, "empty cell grid (r_c larger than the box)");
    const long long ncells = (long long)nc[0] * nc[1] * nc[2];
    if (ncells > (1ll << 30)) return set_error(nullptr, FIPI_ERR_UNSUPPORTED, "too many cells");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 256)
        return set_error(nullptr, FIPI_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    unsigned char* base = nullptr;
    {
        // set-up, once per device, with that device current: the array's name
        // is a host-side stand-in in host code, so its device address is
        // looked up here and passed to the kernels
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_cells_scratch);
            if (e != cudaSuccess || !ptr)
                return set_error(nullptr, FIPI_ERR_CUDA,
                                 std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
            g_noalloc_addr[dev] = ptr;
        }
        base = (unsigned char*)g_noalloc_addr[dev];
    }
    double* pos = (double*)(base + kNoallocPos);
    unsigned* kA = (unsigned*)(base + kNoallocKA);
    unsigned* kB = (unsigned*)(base + kNoallocKB);
    unsigned* iB = (unsigned*)(base + kNoallocIB);
    unsigned* hist = (unsigned*)(base + kNoallocHist);
    int* status = (int*)(base + kNoallocStatus);
    unsigned* iA = (unsigned*)d_sorted;  // ids start in the caller's output

    PC pc{};
    pc.n = n;
    for (int a = 0; a < 3; ++a) {
        pc.nc[a] = nc[a];
        pc.dc[a] = dc[a];
    }
    pc.margin = P->margin;
    // the error word keeps the previous call's value: clear it first
    e = cudaMemsetAsync(status, 0, sizeof(int), st);
    if (e != cudaSuccess) return set_error(nullptr, FIPI_ERR_CUDA, std::string("status clear: ") + cudaGetErrorString(e));
    const int nb = (n + 255) / 256;
    k_aos_to_soa<<<nb, 256, 0, st>>>(d_pos, pos, n);
    k_cell_keys<<<nb, 256, 0, st>>>(pc, pos, kA, iA, status);
    // per-particle keys in particle order, before the sort permutes them
    e = cudaMemcpyAsync(d_keys, kA, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return set_error(nullptr, FIPI_ERR_CUDA, std::string("keys copy: ") + cudaGetErrorString(e));
    const int nblk = (n + RS_TILE - 1) / RS_TILE;
    const int bits = bits_for(ncells - 1);
    unsigned *k = kA, *v = iA, *k2 = kB, *v2 = iB;
    for (int shift = 0; shift < bits; shift += 8) {
        k_rs_hist<<<nblk, RS_T, 0, st>>>(k, n, shift, hist, nblk);
        k_scan_excl<<<1, 1024, 0, st>>>(hist, 256 * nblk);
        k_rs_scatter<<<nblk, RS_T, 0, st>>>(k, v, k2, v2, n, shift, hist, nblk);
        std::swap(k, k2);
        std::swap(v, v2);
    }
    if (v != iA) {
        e = cudaMemcpyAsync(iA, v, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return set_error(nullptr, FIPI_ERR_CUDA, std::string("ids copy: ") + cudaGetErrorString(e));
    }
    k_cell_offsets<<<(int)((ncells + 1 + 255) / 256), 256, 0, st>>>(k, n, d_offsets, (int)ncells);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(nullptr, FIPI_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    int hst = 0;
    e = cudaMemcpyAsync(&hst, status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_error(nullptr, FIPI_ERR_CUDA, std::string("sync: ") + cudaGetErrorString(e));
    if (hst & ERR_NONFINITE) return set_error(nullptr, FIPI_ERR_NONFINITE, "non-finite particle position");
    if (hst & ERR_OUT_OF_RANGE)
        return set_error(nullptr, FIPI_ERR_OUT_OF_RANGE, "particle out of sorting range (cluster.cpp:144-163)");
    return FIPI_OK;
}
