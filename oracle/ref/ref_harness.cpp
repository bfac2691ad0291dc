/*
 * TEST INFRASTRUCTURE ONLY (oracle recipe).
 *
 * Harness around the reference's own objects (field, cluster, element),
 * compiled together with the reference sources where they lie.  main.cpp is
 * not compiled: its set-up (main.cpp:29-73) and loop body
 * (main.cpp:75-219) are restated call for call below, with seeded initial
 * conditions injected after construction (replacing rand() in
 * field.cpp:96 and cluster.cpp:59-89) and the VTK output skipped.
 *
 * The generated configuration header (pre-included) defines the HEAD guard,
 * every constant of head.hpp and `private` as `public`, so the harness can
 * reach field::v and cluster::particle.
 */
#include "cluster.hpp"
#include "field.hpp"
#include "primitive.hpp"

#include <cstring>

namespace {

struct Sim {
    field kf{"VECTORS", "wave_vector"};
    field kf2{"SCALARS"};
    field c{"SCALARS"};
    field c_new{"SCALARS"};
    field c_old{"SCALARS"};
    field f{"SCALARS"};
    field f_old{"SCALARS"};
    field grad_c{"VECTORS"};
    field conv_c{"SCALARS"};
    field conv_c_old{"SCALARS"};
    field u{"VECTORS"};
    field pch{"SCALARS"};
    field g{"VECTORS", "gravity"};
    field f_total{"VECTORS"};
    cluster suspension;
    fftw_plan p_forward, p_backward;
    int t = 0;

    Sim() {
        kf2 = kf.power(2.0); /* main.cpp:31 */
        fftw_init_threads();
        fftw_plan_with_nthreads(4); /* main.cpp:70 */
        fftw_complex* dummy = (fftw_complex*)fftw_malloc(sizeof(fftw_complex) * Nx * Ny * Nz);
        p_forward = fftw_plan_dft_3d(Nz, Ny, Nx, dummy, dummy, FFTW_FORWARD, FFTW_ESTIMATE);
        p_backward = fftw_plan_dft_3d(Nz, Ny, Nx, dummy, dummy, FFTW_BACKWARD, FFTW_ESTIMATE);
        fftw_free(dummy);
    }

    /* Loop body of main.cpp:75-219 for the current t. */
    void step() {
        if (switch_ch) {
            f = (lambda / sqr(epsilon)) * (c.power(3.0) - c);
            f.fft(p_forward);
            c.fft(p_forward);
            if (switch_ns) {
                grad_c = c.grad(kf);
                grad_c.ifft(p_backward);
                conv_c = u.dot(grad_c);
                conv_c.fft(p_forward);
            }
            if (t == 0) {
                c_old = c;
                f_old = f;
                if (switch_ns) conv_c_old = conv_c;
                c -= dt * mobility * kf2 * f;
                if (switch_ns) c -= dt * conv_c;
                c /= 1.0 + (dt * mobility * lambda) * (kf2.power(2.0));
            } else {
                c_new = 4.0 * c - c_old;
                c_new -= (4.0 * dt * mobility) * kf2 * f;
                c_new += (2.0 * dt * mobility) * kf2 * f_old;
                if (switch_ns) {
                    c_new -= (4.0 * dt) * conv_c;
                    c_new += (2.0 * dt) * conv_c_old;
                }
                c_new /= 3.0 + (2.0 * dt * mobility * lambda) * (kf2.power(2.0));
                c_old = c;
                f_old = f;
                if (switch_ns) conv_c_old = conv_c;
                c = c_new;
            }
            c.ifft(p_backward);
        }
        if (switch_ns) {
            f_total.reset("p");
            if (switch_ch) {
                f = (lambda / sqr(epsilon)) * (c.power(3.0) - c);
                f.fft(p_forward);
                c.fft(p_forward);
                pch = lambda * kf2 * c + f;
                pch.ifft(p_backward);
                grad_c = c.grad(kf);
                grad_c.ifft(p_backward);
                c.ifft(p_backward);
                f_total += pch * grad_c;
            }
            if (switch_particle) f_total += suspension.compute_f_r();
            f_total += ((1.0 + c) / 2.0 * rho1 + (1.0 - c) / 2.0 * rho2) * g;
            f_total.fft(p_forward);
            u = f_total - kf * (kf.dot(f_total)) / kf2;
            u /= mu * kf2;
            u.ifft(p_backward);
        }
        if (switch_particle) {
            if (switch_ch) {
                c.fft(p_forward);
                grad_c = c.grad(kf);
                grad_c.ifft(p_backward);
                c.ifft(p_backward);
            }
            suspension.interpolate_local_variables(u, c, grad_c);
            suspension.sorting();
            suspension.compute_f_pi();
            suspension.compute_f_pp(t + 1);
            suspension.compute_f_ext(t + 1);
            suspension.advect("1");
            suspension.enforce_bc();
            suspension.interpolate_local_variables(u, c, grad_c);
            suspension.sorting();
            suspension.compute_f_pi();
            suspension.compute_f_pp(t + 1);
            suspension.compute_f_ext(t + 1);
            suspension.advect("2");
            suspension.enforce_bc();
        }
        ++t;
    }
};

Sim* g_sim = nullptr;
const long V = (long)Nx * Ny * Nz;

/* cluster::sorting exits the process on an out-of-range particle
 * (cluster.cpp:144-163); check the same expression first. */
bool in_sorting_range(const cluster& s, const double* p, int n) {
    for (int it = 0; it < n; ++it) {
        int i = int(floor(p[3 * it] / s.dx_cell + margin / s.dx_cell));
        int j = int(floor(p[3 * it + 1] / s.dy_cell + margin / s.dy_cell));
        int k = int(floor(p[3 * it + 2] / s.dz_cell + margin / s.dz_cell));
        if (i < 0 || i >= s.nx_cell || j < 0 || j >= s.ny_cell || k < 0 || k >= s.nz_cell)
            return false;
    }
    return true;
}

void load_particles(cluster& s, const double* p, const double* r) {
    for (int it = 0; it < s.N; ++it) {
        s.particle[it].p.set_value(p[3 * it], p[3 * it + 1], p[3 * it + 2]);
        s.particle[it].p_old = s.particle[it].p;
        if (r) s.particle[it].r = r[it];
    }
}

}  // namespace

extern "C" {

/* The compiled-in configuration, in fipi_params field order (doubles). */
void ref_config(double* out) {
    const double v[] = {double(Nx), double(Ny), double(Nz), Lx,       Ly,      Lz,
                        dt,         double(t_end), pi,     sigma,    epsilon, lambda,
                        mobility,   mu,         rho1,      rho2,     gravity, A,
                        k_n,        margin,     r_p,       r_eq,     r_c,     double(N_p),
                        double(switch_particle), double(switch_ch), double(switch_ns)};
    std::memcpy(out, v, sizeof(v));
}

int ref_init(const double* c0, const double* p0, const double* r0, const double* f_pp0) {
    delete g_sim;
    g_sim = new Sim();
    for (long it = 0; it < V; ++it) g_sim->c.set_value(0, (int)it, c0[it]);
    if (N_p > 0) {
        if (!in_sorting_range(g_sim->suspension, p0, N_p)) return 4;
        load_particles(g_sim->suspension, p0, r0);
        if (f_pp0)
            for (int it = 0; it < N_p; ++it)
                g_sim->suspension.particle[it].f_pp.set_value(f_pp0[3 * it], f_pp0[3 * it + 1],
                                                               f_pp0[3 * it + 2]);
    }
    return 0;
}

int ref_step(void) {
    if (!g_sim) return 7;
    if (switch_particle && N_p > 0) {
        double* p = new double[3 * N_p];
        for (int it = 0; it < N_p; ++it) {
            p[3 * it] = g_sim->suspension.particle[it].p.get_x();
            p[3 * it + 1] = g_sim->suspension.particle[it].p.get_y();
            p[3 * it + 2] = g_sim->suspension.particle[it].p.get_z();
        }
        bool ok = in_sorting_range(g_sim->suspension, p, N_p);
        delete[] p;
        if (!ok) return 4;
    }
    g_sim->step();
    return 0;
}

static void get_real(const field& fl, int d, double* out) {
    for (long it = 0; it < V; ++it) out[it] = fl.v[d][it][0];
}

void ref_get_phase(double* out) { get_real(g_sim->c, 0, out); }
void ref_get_phase_imag(double* out) {
    for (long it = 0; it < V; ++it) out[it] = g_sim->c.v[0][it][1];
}
void ref_get_velocity(double* out) {
    for (int d = 0; d < 3; ++d) get_real(g_sim->u, d, out + d * V);
}
void ref_get_grad(double* out) {
    for (int d = 0; d < 3; ++d) get_real(g_sim->grad_c, d, out + d * V);
}
void ref_get_particles(double* p, double* f_pp, double* f_pi) {
    const cluster& s = g_sim->suspension;
    for (int it = 0; it < s.N; ++it) {
        const element& e = s.particle[it];
        if (p) {
            p[3 * it] = e.p.get_x();
            p[3 * it + 1] = e.p.get_y();
            p[3 * it + 2] = e.p.get_z();
        }
        if (f_pp) {
            f_pp[3 * it] = e.f_pp.get_x();
            f_pp[3 * it + 1] = e.f_pp.get_y();
            f_pp[3 * it + 2] = e.f_pp.get_z();
        }
        if (f_pi) {
            f_pi[3 * it] = e.f_pi.get_x();
            f_pi[3 * it + 1] = e.f_pi.get_y();
            f_pi[3 * it + 2] = e.f_pi.get_z();
        }
    }
}
double ref_tau(void) { return g_sim->suspension.tau; }

/* main.cpp:232 free energy, summed like field.cpp:507-516. */
double ref_free_energy(void) {
    field fe("SCALARS");
    fe = lambda * (0.5 * g_sim->grad_c.power(2.0) +
                   0.25 / sqr(epsilon) * (g_sim->c.power(2.0) - 1.0).power(2.0));
    double sum = 0.0;
    for (long it = 0; it < V; ++it) sum += fe.v[0][it][0] * cubic(dx);
    return sum;
}

/* ---------------------------------------------- fine-grained reference calls */

/* field::fft / field::ifft on a complex array (data: V interleaved pairs). */
void ref_fft(double* data, int sign, int normalise) {
    if (!g_sim) g_sim = new Sim();
    field a("SCALARS");
    std::memcpy(a.v[0], data, sizeof(fftw_complex) * V);
    if (sign < 0) a.fft(g_sim->p_forward);
    else if (normalise) a.ifft(g_sim->p_backward);
    else fftw_execute_dft(g_sim->p_backward, a.v[0], a.v[0]);
    std::memcpy(data, a.v[0], sizeof(fftw_complex) * V);
}

/* c.fft; grad_c = c.grad(kf); grad_c.ifft  (main.cpp:190-192) */
void ref_grad(const double* c, double* out) {
    if (!g_sim) g_sim = new Sim();
    field a("SCALARS");
    for (long it = 0; it < V; ++it) a.set_value(0, (int)it, c[it]);
    a.fft(g_sim->p_forward);
    field gr("VECTORS");
    gr = a.grad(g_sim->kf);
    gr.ifft(g_sim->p_backward);
    for (int d = 0; d < 3; ++d) get_real(gr, d, out + d * V);
}

/* cluster::sorting: keys, per-cell lists flattened in list order, offsets. */
int ref_sorting(const double* p, int* keys, int* sorted, int* offsets, int* it_mark) {
    cluster s;
    if (!in_sorting_range(s, p, s.N)) return 4;
    load_particles(s, p, nullptr);
    s.sorting();
    const int ncell = s.nx_cell * s.ny_cell * s.nz_cell;
    int pos = 0;
    for (int cidx = 0; cidx < ncell; ++cidx) {
        offsets[cidx] = pos;
        for (node* nd = s.cell[cidx].front; nd != NULL; nd = nd->next) {
            sorted[pos++] = nd->value;
            keys[nd->value] = cidx;
        }
    }
    offsets[ncell] = pos;
    *it_mark = s.it_mark;
    return 0;
}

/* cluster::sorting + compute_f_pi (with injected f_pi) + compute_f_pp(t). */
int ref_f_pp(const double* p, int t, const double* f_pi, double* f_pp, double* tau) {
    cluster s;
    if (!in_sorting_range(s, p, s.N)) return 4;
    load_particles(s, p, nullptr);
    for (int it = 0; it < s.N; ++it)
        s.particle[it].f_pi.set_value(f_pi ? f_pi[3 * it] : 0.0, f_pi ? f_pi[3 * it + 1] : 0.0,
                                      f_pi ? f_pi[3 * it + 2] : 0.0);
    s.sorting();
    s.compute_f_pp(t);
    for (int it = 0; it < s.N; ++it) {
        f_pp[3 * it] = s.particle[it].f_pp.get_x();
        f_pp[3 * it + 1] = s.particle[it].f_pp.get_y();
        f_pp[3 * it + 2] = s.particle[it].f_pp.get_z();
    }
    *tau = s.tau;
    return 0;
}

/* field::interpolate of one real field at n positions. */
void ref_interpolate(const double* vals, int n, const double* p, double* out) {
    field a("SCALARS");
    for (long it = 0; it < V; ++it) a.set_value(0, (int)it, vals[it]);
    for (int q = 0; q < n; ++q) out[q] = a.interpolate(vector(p[3 * q], p[3 * q + 1], p[3 * q + 2]), 0);
}

/* element::get_f_pi for injected local c and dcdx. */
void ref_f_pi(int n, const double* c_loc, const double* dcdx, const double* r, double* f_pi) {
    for (int q = 0; q < n; ++q) {
        element e;
        if (r) e.r = r[q];
        e.c = c_loc[q];
        e.dcdx.set_value(dcdx[3 * q], dcdx[3 * q + 1], dcdx[3 * q + 2]);
        e.get_f_pi();
        f_pi[3 * q] = e.f_pi.get_x();
        f_pi[3 * q + 1] = e.f_pi.get_y();
        f_pi[3 * q + 2] = e.f_pi.get_z();
    }
}

/* element::advect(stage) + element::enforce_bc, state in/out. */
void ref_advect(int n, int stage, const double* f_pi, const double* f_pp, const double* r,
                double* p, double* p_old, double* u_old) {
    for (int q = 0; q < n; ++q) {
        element e;
        if (r) e.r = r[q];
        e.uf.set_value(0.0, 0.0, 0.0);
        e.f_pi.set_value(f_pi[3 * q], f_pi[3 * q + 1], f_pi[3 * q + 2]);
        e.f_pp.set_value(f_pp[3 * q], f_pp[3 * q + 1], f_pp[3 * q + 2]);
        e.f_ext.set_value(0.0, 0.0, 0.0);
        e.p.set_value(p[3 * q], p[3 * q + 1], p[3 * q + 2]);
        e.p_old.set_value(p_old[3 * q], p_old[3 * q + 1], p_old[3 * q + 2]);
        e.u_old.set_value(u_old[3 * q], u_old[3 * q + 1], u_old[3 * q + 2]);
        e.advect(stage == 1 ? "1" : "2");
        e.enforce_bc();
        p[3 * q] = e.p.get_x();
        p[3 * q + 1] = e.p.get_y();
        p[3 * q + 2] = e.p.get_z();
        p_old[3 * q] = e.p_old.get_x();
        p_old[3 * q + 1] = e.p_old.get_y();
        p_old[3 * q + 2] = e.p_old.get_z();
        u_old[3 * q] = e.u_old.get_x();
        u_old[3 * q + 1] = e.u_old.get_y();
        u_old[3 * q + 2] = e.u_old.get_z();
    }
}

/* cluster::compute_f_r for injected positions and f_pp. */
void ref_spread(const double* p, const double* f_pp, double* out) {
    cluster s;
    load_particles(s, p, nullptr);
    for (int it = 0; it < s.N; ++it) {
        s.particle[it].f_pp.set_value(f_pp[3 * it], f_pp[3 * it + 1], f_pp[3 * it + 2]);
        s.particle[it].f_ext.set_value(0.0, 0.0, 0.0);
    }
    field fr("VECTORS");
    fr = s.compute_f_r();
    for (int d = 0; d < 3; ++d) get_real(fr, d, out + d * V);
}

/* field::div (field.cpp:332-361) of a real vector field, then field::ifft, real part. */
void ref_div(const double* v, double* out) {
    if (!g_sim) g_sim = new Sim();
    field a("VECTORS");
    for (int d = 0; d < 3; ++d)
        for (long it = 0; it < V; ++it) {
            a.v[d][it][0] = v[d * V + it];
            a.v[d][it][1] = 0.0;
        }
    a.fft(g_sim->p_forward);
    field dv = a.div(g_sim->kf);
    dv.ifft(g_sim->p_backward);
    get_real(dv, 0, out);
}

/* field::interpolate2 (field.cpp:250-281) of one real field at n positions. */
void ref_interpolate2(const double* vals, int n, const double* p, double* out) {
    field a("SCALARS");
    for (long it = 0; it < V; ++it) a.set_value(0, (int)it, vals[it]);
    for (int q = 0; q < n; ++q) out[q] = a.interpolate2(vector(p[3 * q], p[3 * q + 1], p[3 * q + 2]), 0);
}

/* ------------------------------------------------------------ VTK output */
/* field::output_to_file (field.cpp:469-503) of given values. */
int ref_write_field(const double* values, int components, const char* name, const char* path) {
    field a(components == 1 ? "SCALARS" : "VECTORS");
    for (int d = 0; d < components; ++d)
        for (long it = 0; it < V; ++it) {
            a.v[d][it][0] = values[d * V + it];
            a.v[d][it][1] = 0.0;
        }
    a.output_to_file(path, name);
    return 0;
}

/* The free-energy field of main.cpp:232 from c and grad c, written like main.cpp:233. */
int ref_write_free_energy(const double* c, const double* g, const char* path) {
    field cc("SCALARS"), gc("VECTORS"), fe("SCALARS");
    for (long it = 0; it < V; ++it) {
        cc.v[0][it][0] = c[it];
        cc.v[0][it][1] = 0.0;
        for (int d = 0; d < 3; ++d) {
            gc.v[d][it][0] = g[d * V + it];
            gc.v[d][it][1] = 0.0;
        }
    }
    fe = lambda * (0.5 * gc.power(2.0) + 0.25 / sqr(epsilon) * (cc.power(2.0) - 1.0).power(2.0));
    fe.output_to_file(path, "free_energy");
    return 0;
}

/* cluster::output (cluster.cpp:415-456) of given particles. */
int ref_write_particles(const double* p, const double* r, const double* f_pp, const char* path) {
    if (!g_sim) g_sim = new Sim();
    load_particles(g_sim->suspension, p, r);
    for (int it = 0; it < N_p; ++it)
        g_sim->suspension.particle[it].f_pp.set_value(f_pp[3 * it], f_pp[3 * it + 1], f_pp[3 * it + 2]);
    g_sim->suspension.output(path);
    return 0;
}

/* srand(seed) (main.cpp:24), field c("SCALARS","phase_field") (main.cpp:34)
 * and cluster::distribute (main.cpp:58-66) with the C library's rand(). */
int ref_initial_state(unsigned int seed, double* c, double* pos) {
    srand(seed);
    field cf("SCALARS", "phase_field");
    for (long it = 0; it < V; ++it) c[it] = cf.v[0][it][0];
    if (switch_particle && N_p > 0) {
        cluster s;
        s.distribute();
        for (int it = 0; it < N_p; ++it) {
            pos[3 * it] = s.particle[it].p.get_x();
            pos[3 * it + 1] = s.particle[it].p.get_y();
            pos[3 * it + 2] = s.particle[it].p.get_z();
        }
    }
    return 0;
}

}  // extern "C"
