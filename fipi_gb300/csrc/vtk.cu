// VTK legacy ASCII writers of the reference's output steps (main.cpp:225-238):
// field::output_to_file (field.cpp:469-503) for the phase field, the
// free-energy density and the velocity, and cluster::output
// (cluster.cpp:415-456) for the particles.  The text is produced with the
// same std::ostream insertions in the same order, so for the same values the
// files are byte-for-byte the reference's.  Host code only, compiled with
// -ffp-contract=off (no fused multiply-add on any host).
#include <cmath>
#include <fstream>
#include <string>
#include <vector>

#include "ctx.hpp"

namespace {

// field::power calls pow(v, b) with a run-time exponent; a volatile pointer
// keeps the compiler from turning pow(x, 2.0) into x * x.
double (*volatile vtk_pow)(double, double) = std::pow;

bool params_ok(const fipi_params* p) { return p && p->nx > 0 && p->ny > 0 && p->nz > 0; }

}  // namespace

extern "C" {

fipi_status fipi_vtk_write_field(const fipi_params* p, const char* path, const char* name, int components,
                                 const double* values) {
    if (!params_ok(p) || !path || !name || !values)
        return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument or empty grid");
    if (components != 1 && components != 3)
        return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, "components must be 1 (SCALARS) or 3 (VECTORS)");
    std::ofstream output(path);
    if (!output) return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, std::string("cannot open ") + path);
    const long long V = (long long)p->nx * p->ny * p->nz;
    output << "# vtk DataFile Version 2.0\n";
    output << name << " PROFILE\n";
    output << "ASCII\n";
    output << "\n";
    output << "DATASET STRUCTURED_POINTS\n";
    output << "DIMENSIONS " << p->nx << " " << p->ny << " " << p->nz << "\n";
    output << "ASPECT_RATIO 1 1 1\n";
    output << "ORIGIN 0 0 0\n";
    output << "POINT_DATA " << p->nx * p->ny * p->nz << "\n";
    output << (components == 1 ? "SCALARS" : "VECTORS") << " " << name << " double\n";
    if (components == 1) output << "LOOKUP_TABLE default\n";
    for (long long it = 0; it < V; ++it) {
        for (int d = 0; d < components; ++d) {
            if (d == components - 1) output << values[d * V + it] << "\n";
            else output << values[d * V + it] << " ";
        }
    }
    output.close();
    if (!output) return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, std::string("write failed: ") + path);
    return FIPI_OK;
}

fipi_status fipi_vtk_write_particles(const fipi_params* p, const char* path, int n, const double* pos,
                                     const double* r, const double* f_pp) {
    if (!params_ok(p) || !path || n < 0 || (n > 0 && (!pos || !f_pp)))
        return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    std::ofstream traject(path);
    if (!traject) return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, std::string("cannot open ") + path);
    const double dx = p->lx / p->nx, dy = p->ly / p->ny, dz = p->lz / p->nz;
    traject << "# vtk DataFile Version 2.0\n";
    traject << "particles\n";
    traject << "ASCII\n";
    traject << "\n";
    traject << "DATASET UNSTRUCTURED_GRID\n";
    traject << "POINTS " << n << " double\n";
    for (int it = 0; it < n; ++it) {
        traject << pos[3 * it] / dx << " ";
        traject << pos[3 * it + 1] / dy << " ";
        traject << pos[3 * it + 2] / dz << "\n";
    }
    traject << "\n";
    traject << "POINT_DATA " << n << "\n";
    traject << "SCALARS radius double\n";
    traject << "LOOKUP_TABLE default\n";
    for (int it = 0; it < n; ++it) traject << (r ? r[it] : p->r_p) / dx << "\n";
    traject << "\n";
    traject << "SCALARS f_pp double\n";
    traject << "LOOKUP_TABLE default\n";
    for (int it = 0; it < n; ++it) {
        // vector::norm (primitive.hpp:58): pow(x^2 + y^2 + z^2, 0.5) with pow(., 2) terms
        const double x = f_pp[3 * it], y = f_pp[3 * it + 1], z = f_pp[3 * it + 2];
        const double nrm = vtk_pow(vtk_pow(x, 2) + vtk_pow(y, 2) + vtk_pow(z, 2), 0.5);
        traject << nrm / p->A / p->pi / p->sigma / p->r_p << "\n";
    }
    traject.close();
    if (!traject) return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, std::string("write failed: ") + path);
    return FIPI_OK;
}

// lambda (0.5 |grad c|^2 + 0.25/eps^2 (c^2 - 1)^2) per node (main.cpp:232),
// with field::power's accumulation from 0 (field.cpp:408-431).
fipi_status fipi_free_energy_density(const fipi_params* p, const double* c, const double* grad_c, double* out) {
    if (!params_ok(p) || !c || !grad_c || !out) return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, "NULL argument");
    const long long V = (long long)p->nx * p->ny * p->nz;
    const double e2 = 0.25 / (p->epsilon * p->epsilon);
    for (long long it = 0; it < V; ++it) {
        double g2 = 0.0;
        for (int d = 0; d < 3; ++d) g2 += vtk_pow(grad_c[d * V + it], 2.0);
        double c2 = 0.0;
        c2 += vtk_pow(c[it], 2.0);
        const double w = c2 - 1.0;
        double w2 = 0.0;
        w2 += vtk_pow(w, 2.0);
        out[it] = p->lambda * (0.5 * g2 + e2 * w2);
    }
    return FIPI_OK;
}

fipi_status fipi_write_vtk(fipi_ctx* ctx, int what, const char* path) {
    if (!ctx || !path) return fipi::set_error(ctx, FIPI_ERR_BAD_ARG, "NULL argument");
    const fipi_params& P = ctx->P;
    const size_t V = (size_t)P.nx * P.ny * P.nz;
    fipi_status st = FIPI_OK;
    switch (what) {
        case FIPI_VTK_PHASE: {
            std::vector<double> c(V);
            if ((st = fipi_get_phase(ctx, c.data())) != FIPI_OK) return st;
            return fipi_vtk_write_field(&P, path, "phase", 1, c.data());
        }
        case FIPI_VTK_FREE_ENERGY: {
            std::vector<double> c(V), g(3 * V), fe(V);
            if ((st = fipi_get_phase(ctx, c.data())) != FIPI_OK) return st;
            if ((st = fipi::fields_get_grad(ctx, g.data())) != FIPI_OK) return st;
            fipi_free_energy_density(&P, c.data(), g.data(), fe.data());
            return fipi_vtk_write_field(&P, path, "free_energy", 1, fe.data());
        }
        case FIPI_VTK_VELOCITY: {
            std::vector<double> u(3 * V);
            if ((st = fipi_get_velocity(ctx, u.data())) != FIPI_OK) return st;
            return fipi_vtk_write_field(&P, path, "u", 3, u.data());
        }
        case FIPI_VTK_PARTICLES: {
            const int n = ctx->pb.n;
            std::vector<double> pos(3 * (size_t)n), fpp(3 * (size_t)n), r((size_t)n);
            if (n > 0) {
                if ((st = fipi_get_particles(ctx, pos.data(), fpp.data(), nullptr)) != FIPI_OK) return st;
                if ((st = fipi::particles_get_radii(ctx, r.data())) != FIPI_OK) return st;
            }
            return fipi_vtk_write_particles(&P, path, n, pos.data(), r.data(), fpp.data());
        }
        default:
            return fipi::set_error(ctx, FIPI_ERR_BAD_ARG, "unknown VTK output");
    }
}

}  // extern "C"
