"""The mixed form's fixed-point conversions (fipi_gb300/csrc/fixed_point.cuh)
use integer operations only; host and device share the code.  Compiled
here with g++: fx_units(v) must equal llrint(v * 2^32) and fx_to_float(u)
the once-rounded u * 2^-32, on edge values (ties, powers of two, the range
limits) and on random values of every exponent."""
import subprocess
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent

PROG = r"""
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include "fixed_point.cuh"

static long long ref_units(float v) { return llrint((double)v * 4294967296.0); }
static float ref_float(long long u) { return (float)((long double)u / 4294967296.0L); }

int main() {
    std::mt19937_64 g(12345);
    long long bad = 0, n = 0;
    auto chk_u = [&](float v) {
        if (!(std::fabs(v) < 1073741824.0f)) return;
        ++n;
        if (fipi::fx_units(v) != ref_units(v)) { if (bad++ < 5) std::printf("units %a\n", (double)v); }
    };
    auto chk_f = [&](long long u) {
        ++n;
        const float a = fipi::fx_to_float(u), b = ref_float(u);
        if (std::memcmp(&a, &b, 4) != 0) { if (bad++ < 5) std::printf("float %lld\n", u); }
    };
    // every exponent, random significands, both signs
    for (int e = 1; e < 157; ++e)
        for (int k = 0; k < 20000; ++k) {
            const unsigned b = ((unsigned)e << 23) | (unsigned)(g() & 0x7fffffu) | ((g() & 1) ? 0x80000000u : 0u);
            float v; std::memcpy(&v, &b, 4);
            chk_u(v);
        }
    // ties of llrint (x.5 in 2^-32 units) and their neighbours, zeros, subnormals, the limit
    for (int s = 1; s <= 26; ++s)
        for (int k = 0; k < 2000; ++k) {
            const double t = (double)((long long)(g() % (1ull << 20)) * 2 + 1) * 0.5;
            float v = (float)std::ldexp(t, -32);
            chk_u(v); chk_u(-v); chk_u(std::nextafter(v, 0.f)); chk_u(std::nextafter(v, 1e30f));
            chk_u((float)std::ldexp(1.0, -s - 32)); chk_u(-(float)std::ldexp(1.0, -s - 32));
        }
    chk_u(0.f); chk_u(-0.f); chk_u(FLT_TRUE_MIN); chk_u(-FLT_MIN); chk_u(std::nextafter(1073741824.0f, 0.f));
    // fixed-point sums: random magnitudes of every bit length, ties at each rounding position
    for (int L = 0; L < 64; ++L)
        for (int k = 0; k < 20000; ++k) {
            unsigned long long u = L == 0 ? 0ull : (g() >> (64 - L)) | (1ull << (L - 1));
            long long v = (long long)u;
            if (L == 64) v = (long long)u;  // negative as a signed value
            chk_f(v); chk_f(-v);
        }
    for (int s = 1; s < 40; ++s)
        for (int k = 0; k < 2000; ++k) {
            const unsigned long long m = (g() & 0xffffffull) | 0x1000000ull;  // 25 bits: one past FP32's
            const long long v = (long long)((m << s) | (1ull << (s - 1)));     // a tie below the kept bits
            if (v > 0) { chk_f(v); chk_f(-v); chk_f(v + 1); chk_f(v - 1); }
        }
    chk_f(INT64_MIN); chk_f(INT64_MAX); chk_f(1); chk_f(-1);
    std::printf("%lld %lld\n", n, bad);
    return bad != 0;
}
"""


def test_fixed_point_conversions(tmp_path):
    src = tmp_path / "fx.cpp"
    src.write_text(PROG)
    exe = tmp_path / "fx"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", str(REPO / "fipi_gb300" / "csrc"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout
    n, bad = map(int, r.stdout.split()[-2:])
    assert n > 4_000_000 and bad == 0
