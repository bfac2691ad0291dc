// fipi.hpp — header-only C++ view of the C ABI in fipi.h, in the
// reference's vocabulary.  `fipi::simulation` owns a context (the fields of
// main.cpp:29-58 and the `cluster` of cluster.cpp:21-40 on the GPU);
// its members are named after the reference calls they replace.  Errors
// throw fipi::error (the reference printed and called exit(0)).
#ifndef FIPI_HPP
#define FIPI_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "fipi.h"

namespace fipi {

class error : public std::runtime_error {
public:
    error(fipi_status s, const char* msg) : std::runtime_error(msg ? msg : ""), code(s) {}
    fipi_status code;
};

inline void check(fipi_status s) {
    if (s != FIPI_OK) throw error(s, fipi_last_error_string());
}

inline fipi_params reference_params() {
    fipi_params p;
    check(fipi_params_reference(&p));
    return p;
}

class simulation {
public:
    explicit simulation(const fipi_params& p, fipi_precision prec = FIPI_FP64, int device = 0) : p_(p) {
        check(fipi_create(&p_, prec, device, &ctx_));
    }
    ~simulation() { fipi_destroy(ctx_); }
    simulation(const simulation&) = delete;
    simulation& operator=(const simulation&) = delete;

    size_t grid_size() const { return (size_t)p_.nx * p_.ny * p_.nz; }
    int particles() const { return p_.n_p; }
    fipi_ctx* handle() const { return ctx_; }

    // ---- state (field c, field u, cluster::particle[])
    void set_phase(const std::vector<double>& c) { need(c, grid_size()); check(fipi_set_phase(ctx_, c.data())); }
    void set_velocity(const std::vector<double>& u) { need(u, 3 * grid_size()); check(fipi_set_velocity(ctx_, u.data())); }
    void set_particles(const std::vector<double>& p, const double* r = nullptr, const double* cos_theta = nullptr,
                       const double* f_pp = nullptr) {
        need(p, 3 * (size_t)p_.n_p);
        check(fipi_set_particles(ctx_, p.data(), r, cos_theta, f_pp));
    }
    std::vector<double> phase() {
        std::vector<double> c(grid_size());
        check(fipi_get_phase(ctx_, c.data()));
        return c;
    }
    std::vector<double> velocity() {
        std::vector<double> u(3 * grid_size());
        check(fipi_get_velocity(ctx_, u.data()));
        return u;
    }
    std::vector<double> positions() {
        std::vector<double> p(3 * (size_t)p_.n_p);
        check(fipi_get_particles(ctx_, p.data(), nullptr, nullptr));
        return p;
    }

    // ---- the loop body of main.cpp:75-219
    void step(int n = 1) { check(fipi_step(ctx_, n)); }
    int time() const {
        int t = 0;
        check(fipi_get_time(ctx_, &t));
        return t;
    }

    // ---- field calls
    std::vector<double> fft(const std::vector<double>& x) {  // field::fft (real input, half spectrum)
        need(x, grid_size());
        std::vector<double> out(2 * (size_t)p_.nz * (p_.nx / 2 + 1) * p_.ny);
        check(fipi_fft_r2c(ctx_, x.data(), out.data()));
        return out;
    }
    std::vector<double> ifft(const std::vector<double>& half) {  // field::ifft + normalize
        std::vector<double> out(grid_size());
        check(fipi_fft_c2r(ctx_, half.data(), out.data()));
        return out;
    }
    std::vector<double> grad(const std::vector<double>& c) {  // field::grad + ifft
        need(c, grid_size());
        std::vector<double> g(3 * grid_size());
        check(fipi_grad(ctx_, c.data(), g.data()));
        return g;
    }

    // ---- cluster / element calls (on given positions)
    struct cells {
        std::vector<int> keys, sorted, offsets;
    };
    cells sorting(const std::vector<double>& p) {  // cluster::sorting
        int nc[3];
        double dc[3];
        check(fipi_cell_geometry(&p_, nc, dc));
        cells c;
        c.keys.resize(p_.n_p);
        c.sorted.resize(p_.n_p);
        c.offsets.resize((size_t)nc[0] * nc[1] * nc[2] + 1);
        check(fipi_cells_build(ctx_, p.data(), c.keys.data(), c.sorted.data(), c.offsets.data()));
        return c;
    }
    std::vector<double> compute_f_pp(const std::vector<double>& p, int t, double* tau = nullptr,
                                     const double* f_pi = nullptr) {
        std::vector<double> f(3 * (size_t)p_.n_p);
        check(fipi_f_pp(ctx_, p.data(), t, f_pi, f.data(), tau));
        return f;
    }
    std::vector<double> compute_f_r(const std::vector<double>& p, const std::vector<double>& f_pp) {
        std::vector<double> out(3 * grid_size());
        check(fipi_spread(ctx_, p.data(), f_pp.data(), out.data()));
        return out;
    }
    std::vector<double> interpolate(const std::vector<double>& fields, int nfields, const std::vector<double>& p) {
        std::vector<double> out((size_t)p_.n_p * nfields);
        check(fipi_interpolate(ctx_, fields.data(), nfields, p.data(), out.data()));
        return out;
    }
    std::vector<double> get_f_pi(const std::vector<double>& c_loc, const std::vector<double>& dcdx,
                                 const double* r = nullptr, const double* cos_theta = nullptr) {
        std::vector<double> f(3 * (size_t)p_.n_p);
        check(fipi_f_pi(ctx_, c_loc.data(), dcdx.data(), r, cos_theta, f.data()));
        return f;
    }
    void advect(int stage, const std::vector<double>& f_pi, const std::vector<double>& f_pp, std::vector<double>& p,
                std::vector<double>& p_old, std::vector<double>& u_old, const double* r = nullptr) {
        check(fipi_advect(ctx_, stage, f_pi.data(), f_pp.data(), r, p.data(), p_old.data(), u_old.data()));
    }

    // ---- diagnostics
    double mass() {
        double v = 0;
        check(fipi_mass(ctx_, &v));
        return v;
    }
    double free_energy() {
        double v = 0;
        check(fipi_free_energy(ctx_, &v));
        return v;
    }
    double packing_energy() {
        double v = 0;
        check(fipi_packing_tau(ctx_, &v));
        return v;
    }

    // ---- the three parts of an iteration, the output step, checkpoints
    void step_ch() { check(fipi_step_ch(ctx_)); }
    void step_stokes() { check(fipi_step_stokes(ctx_)); }
    void step_particles() { check(fipi_step_particles(ctx_)); }
    void write_vtk(int what, const char* path) { check(fipi_write_vtk(ctx_, what, path)); }
    void checkpoint_reserve(int slots) { check(fipi_checkpoint_reserve(ctx_, slots)); }
    void checkpoint_save(int slot) { check(fipi_checkpoint_save(ctx_, slot)); }
    void checkpoint_load(int slot) { check(fipi_checkpoint_load(ctx_, slot)); }

    // ---- reverse mode (FIPI_FP64 contexts): gradient of a trajectory's
    // final-state functional with respect to its first state
    void trajectory_forward(int nsteps, int stride = 0) { check(fipi_trajectory_forward(ctx_, nsteps, stride)); }
    std::vector<double> trajectory_backward_phase(const std::vector<double>& dc_final) {
        need(dc_final, grid_size());
        check(fipi_trajectory_backward(ctx_, dc_final.data(), nullptr, nullptr, nullptr));
        std::vector<double> dc(grid_size());
        check(fipi_adjoint_get(ctx_, dc.data(), nullptr, nullptr, nullptr));
        return dc;
    }

    // ---- particle-model extensions (off by default)
    void set_fluid_coupling(bool on) { check(fipi_set_fluid_coupling(ctx_, on ? 1 : 0)); }
    void set_brownian(double kt, uint64_t seed) { check(fipi_set_brownian(ctx_, kt, seed)); }

    // ---- device-pointer state I/O (FP64 device arrays, no host copies)
    void set_phase_device(const double* d_c) { check(fipi_set_phase_device(ctx_, d_c)); }
    void get_phase_device(double* d_c) { check(fipi_get_phase_device(ctx_, d_c)); }
    void set_particles_device(const double* d_p, const double* d_r = nullptr, const double* d_cos_theta = nullptr,
                              const double* d_f_pp = nullptr) {
        check(fipi_set_particles_device(ctx_, d_p, d_r, d_cos_theta, d_f_pp));
    }
    void get_particles_device(double* d_p, double* d_f_pp = nullptr, double* d_f_pi = nullptr) {
        check(fipi_get_particles_device(ctx_, d_p, d_f_pp, d_f_pi));
    }

private:
    static void need(const std::vector<double>& v, size_t n) {
        if (v.size() != n) throw error(FIPI_ERR_BAD_ARG, "array size does not match the grid / particle count");
    }
    fipi_params p_;
    fipi_ctx* ctx_ = nullptr;
};

}  // namespace fipi

#endif  // FIPI_HPP
