// Conversions between FP32 and the 64-bit fixed-point units (2^-32) of the
// mixed form's spreading, with integer operations only: GB300 runs
// conversions to and from 64-bit types on its narrow FP64 pipe.  Host and
// device share the code, so the host test checks it against llrint and a
// once-rounded conversion.
#pragma once

#include <cstring>

#ifdef __CUDACC__
#define FIPI_HD __host__ __device__ __forceinline__
#else
#define FIPI_HD inline
#endif

namespace fipi {

FIPI_HD unsigned fx_bits(float v) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(v);
#else
    unsigned b;
    std::memcpy(&b, &v, sizeof b);
    return b;
#endif
}

FIPI_HD float fx_float(unsigned b) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float v;
    std::memcpy(&v, &b, sizeof v);
    return v;
#endif
}

FIPI_HD int fx_msb(unsigned long long u) {  // u != 0
#ifdef __CUDA_ARCH__
    return 63 - __clzll((long long)u);
#else
    return 63 - __builtin_clzll(u);
#endif
}

// llrint(v * 2^32) for a finite |v| < 2^30 (round half to even, as llrint):
// v = m 2^(e - 150) with the 24-bit significand m and the biased exponent
// e, so v 2^32 = m 2^(e - 118).
FIPI_HD long long fx_units(float v) {
    const unsigned b = fx_bits(v);
    const int e = (int)((b >> 23) & 0xffu);
    if (e == 0) return 0;  // zero or subnormal: |v 2^32| < 2^-94
    const long long m = (long long)((b & 0x7fffffu) | 0x800000u);
    const int sh = e - 118;
    long long r;
    if (sh >= 0) {
        r = m << sh;  // sh <= 38 for |v| < 2^30
    } else if (sh < -62) {
        r = 0;
    } else {
        const int s = -sh;
        const long long q = m >> s, rem = m & ((1ll << s) - 1), half = 1ll << (s - 1);
        r = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
    }
    return (b >> 31) ? -r : r;
}

// v 2^-32 as FP32, rounded once to nearest even: the 24 leading bits of
// |v| with the rest rounded off, v 2^-32 = 1.m 2^(msb - 32).
FIPI_HD float fx_to_float(long long v) {
    if (v == 0) return 0.f;
    const unsigned sign = v < 0 ? 0x80000000u : 0u;
    const unsigned long long u = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    int msb = fx_msb(u);
    unsigned long long m;
    if (msb <= 23) {
        m = u << (23 - msb);
    } else {
        const int s = msb - 23;
        m = u >> s;
        const unsigned long long rem = u & ((1ull << s) - 1), half = 1ull << (s - 1);
        if (rem > half || (rem == half && (m & 1ull))) ++m;
        if (m == (1ull << 24)) {
            m >>= 1;
            ++msb;
        }
    }
    return fx_float(sign | ((unsigned)(msb + 95) << 23) | ((unsigned)m & 0x7fffffu));
}

}  // namespace fipi

#undef FIPI_HD
