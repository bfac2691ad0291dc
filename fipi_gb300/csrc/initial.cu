// Initial state of the reference's set-up, drawn as the reference draws it
// (host only): srand(seed) (main.cpp:24 seeds from the clock), the phase
// field's draws in its constructor (field.cpp:85-99, constructed at
// main.cpp:34) and cluster::distribute's random sequential addition
// (cluster.cpp:53-113, called at main.cpp:61-66).
//
// rand() is the C library's.  glibc's rand() is random() with the default
// 31-word state: an additive lagged-Fibonacci generator
// r_i = r_{i-3} + r_{i-31} (mod 2^32) whose first 31 words come from
// r_i = 16807 r_{i-1} mod (2^31 - 1), with 310 outputs discarded and
// output r_i >> 1.  It is restated below so any host gives the same draws.
//
// The reference's overlap test (cluster.cpp:98-113) scans every earlier
// particle; a uniform hash grid of cells no smaller than the contact distance
// finds the same overlaps (the test is a pure "any j < i" predicate with the
// same distance expression), in O(1) per candidate instead of O(i).
//
// Compiled with -ffp-contract=off: c = k/1e3*0.2 - 0.1 must not fuse.
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "ctx.hpp"

namespace fipi {
namespace {

class GlibcRand {
   public:
    explicit GlibcRand(unsigned int seed) {
        int32_t word = (int32_t)(seed == 0 ? 1u : seed);
        r_[0] = word;
        for (int i = 1; i < kDeg; ++i) {
            // 16807 * word mod (2^31 - 1) without overflow (Schrage)
            const int32_t hi = word / 127773, lo = word % 127773;
            word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            r_[i] = word;
        }
        f_ = kSep;
        b_ = 0;
        for (int i = 0; i < 10 * kDeg; ++i) next();
    }
    int next() {
        const uint32_t v = (uint32_t)r_[f_] + (uint32_t)r_[b_];
        r_[f_] = (int32_t)v;
        f_ = f_ + 1 == kDeg ? 0 : f_ + 1;
        b_ = b_ + 1 == kDeg ? 0 : b_ + 1;
        return (int)(v >> 1);
    }

   private:
    static constexpr int kDeg = 31, kSep = 3;
    int32_t r_[kDeg];
    int f_, b_;
};

// vector::norm (primitive.hpp:58) of a - b compared with 2 r_p as
// check_overlap does (cluster.cpp:104).
inline bool closer_than(const double* a, const double* b, double dmin) {
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    const double s = std::pow(dx, 2) + std::pow(dy, 2) + std::pow(dz, 2);
    if (s > dmin * dmin * 1.001) return false;  // pow(s, 0.5) is within an ulp of sqrt(s)
    return std::pow(s, 0.5) < dmin;
}

}  // namespace
}  // namespace fipi

using namespace fipi;

extern "C" fipi_status fipi_reference_initial_state(const fipi_params* P, unsigned int seed, double* c, double* pos) {
    if (!P) return set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    GlibcRand rnd(seed);
    const size_t V = (size_t)P->nx * P->ny * P->nz;
    for (size_t it = 0; it < V; ++it) {
        const double v = double(rnd.next() % 1000) / 1e3 * 0.2 - 0.1;  // field.cpp:96
        if (c) c[it] = v;
    }
    const int n = P->n_p;
    if (!P->switch_particle || n <= 0) return FIPI_OK;
    const double L[3] = {P->lx, P->ly, P->lz};
    const double dmin = 2.0 * P->r_p;
    int gc[3];
    double gs[3];
    for (int a = 0; a < 3; ++a) {
        gc[a] = dmin > 0.0 ? std::max(1, (int)std::floor(L[a] / dmin)) : 1;
        if (gc[a] > 1024) gc[a] = 1024;
        gs[a] = L[a] / gc[a];
    }
    std::vector<std::vector<int>> grid((size_t)gc[0] * gc[1] * gc[2]);
    std::vector<double> p(3 * (size_t)n);
    auto cell_of = [&](const double* x, int* ci) {
        for (int a = 0; a < 3; ++a) {
            int k = (int)(x[a] / gs[a]);
            ci[a] = k < 0 ? 0 : (k >= gc[a] ? gc[a] - 1 : k);
        }
    };
    const long long max_candidates = 10000000;
    for (int it = 0; it < n; ++it) {
        double* x = &p[3 * (size_t)it];
        bool placed = false;
        for (long long cand = 0; cand < max_candidates && !placed; ++cand) {
            for (int a = 0; a < 3; ++a) x[a] = L[a] * (double(rnd.next() % 1000) / 1e3);  // cluster.cpp:63-71
            int ci[3];
            cell_of(x, ci);
            bool overlap = false;
            for (int dk = -1; dk <= 1 && !overlap; ++dk)
                for (int dj = -1; dj <= 1 && !overlap; ++dj)
                    for (int di = -1; di <= 1 && !overlap; ++di) {
                        const int i = ci[0] + di, j = ci[1] + dj, k = ci[2] + dk;
                        if (i < 0 || j < 0 || k < 0 || i >= gc[0] || j >= gc[1] || k >= gc[2]) continue;
                        for (int q : grid[(size_t)i + (size_t)j * gc[0] + (size_t)k * gc[0] * gc[1]])
                            if (closer_than(&p[3 * (size_t)q], x, dmin)) {
                                overlap = true;
                                break;
                            }
                    }
            placed = !overlap;
        }
        if (!placed)
            return set_error(nullptr, FIPI_ERR_BAD_PARAMS,
                             "cluster::distribute found no place for particle " + std::to_string(it) +
                                 " within 1e7 candidates (the reference would loop forever)");
        int ci[3];
        cell_of(x, ci);
        grid[(size_t)ci[0] + (size_t)ci[1] * gc[0] + (size_t)ci[2] * gc[0] * gc[1]].push_back(it);
    }
    if (pos)
        for (size_t i = 0; i < 3 * (size_t)n; ++i) pos[i] = p[i];
    return FIPI_OK;
}
