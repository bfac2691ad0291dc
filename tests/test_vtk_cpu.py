"""VTK output of the reference's output step (main.cpp:225-238).

The library's host writers must produce, for the same values, the same
bytes as the reference's field::output_to_file (field.cpp:469-503) and
cluster::output (cluster.cpp:415-456), compiled in place from the
reference sources (skipped where those are absent).  No device is needed.
"""
import numpy as np
import pytest

from conftest import seeded_state


@pytest.fixture(scope="module")
def ref_mod(oracle_mod):
    if not oracle_mod.reference_available():
        pytest.skip("reference sources absent")
    return oracle_mod


@pytest.mark.parametrize("name", ["t16", "t32_2pi"])
def test_vtk_bytes_equal_reference(fipi, ref_mod, name, tmp_path):
    w = fipi.workload(name)
    P, c, p, r, ct = seeded_state(w, 21)
    ref = ref_mod.Ref(name)
    rng = np.random.default_rng(4)
    V, n = w.V, w.n_p
    g = 0.3 * rng.standard_normal(3 * V)
    u = 1e-3 * rng.standard_normal(3 * V)
    fpp = rng.standard_normal(3 * n)
    cases = []
    # phase field (SCALARS), velocity (VECTORS)
    fipi.vtk_write_field(P, tmp_path / "a_phase.vtk", "phase", c, 1)
    ref.write_field(c, 1, "phase", tmp_path / "b_phase.vtk")
    cases.append("phase")
    fipi.vtk_write_field(P, tmp_path / "a_u.vtk", "u", u, 3)
    ref.write_field(u, 3, "u", tmp_path / "b_u.vtk")
    cases.append("u")
    # free-energy density from c and grad c
    fe = fipi.free_energy_density(P, c, g)
    fipi.vtk_write_field(P, tmp_path / "a_fe.vtk", "free_energy", fe, 1)
    ref.write_free_energy(c, g, tmp_path / "b_fe.vtk")
    cases.append("fe")
    # particles: positions / dx, radii / dx, |f_pp| / (A pi sigma r_p)
    fipi.vtk_write_particles(P, tmp_path / "a_particle.vtk", p, r, fpp)
    ref.write_particles(p, r, fpp, tmp_path / "b_particle.vtk")
    cases.append("particle")
    for k in cases:
        a = (tmp_path / f"a_{k}.vtk").read_bytes()
        b = (tmp_path / f"b_{k}.vtk").read_bytes()
        assert len(a) > 100
        assert a == b, k


def test_free_energy_density_sums_to_oracle_total(fipi, oracle_mod):
    """The density summed times dx^3 is the oracle's (and the reference's)
    total free energy of the same state."""
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 5)
    port = oracle_mod.Port(P)
    port.set_state(c, p, r, ct)
    port.step(2)
    fe = fipi.free_energy_density(P, port.phase(), port.grad())
    dx = P.lx / P.nx
    total = 0.0
    for v in fe:
        total += v * dx ** 3
    assert total == port.free_energy()
