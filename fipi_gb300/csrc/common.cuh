// Shared device helpers of the FIPI GB300 library: complex arithmetic on
// float2/double2, error plumbing, small numeric utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fipi {

template <typename T> struct cplx_of;
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<double> { using type = double2; };
template <typename T> using cplx = typename cplx_of<T>::type;

template <typename C> __host__ __device__ __forceinline__ C mkc(decltype(C{}.x) re, decltype(C{}.x) im) {
    C c;
    c.x = re;
    c.y = im;
    return c;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mkc<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mkc<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return mkc<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __device__ __forceinline__ C cconj(C a) { return mkc<C>(a.x, -a.y); }
template <typename C, typename T> __device__ __forceinline__ C cscale(C a, T s) { return mkc<C>(a.x * s, a.y * s); }
// multiply by -i (dir < 0) or +i (dir > 0)
template <typename C> __device__ __forceinline__ C cmul_i(C a, int dir) {
    return dir < 0 ? mkc<C>(a.y, -a.x) : mkc<C>(-a.y, a.x);
}

// Device error word bits (read back by the host after each step).
enum : int {
    ERR_OUT_OF_RANGE = 1,  // particle outside the cell grid (cluster.cpp:144-163)
    ERR_NONFINITE = 2,     // NaN/Inf seen in a particle position
    ERR_TMA_TIMEOUT = 4,   // a bounded wait for a bulk copy gave up
    ERR_SPREAD_RANGE = 8,  // a fixed-point spread sum left the int64 range
};

__host__ __device__ __forceinline__ int ilog2i(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

}  // namespace fipi
