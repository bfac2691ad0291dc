"""Particle-model extensions on the GPU against the oracle.

Fluid coupling (uf = u^{n+1} interpolated at the particle, the commented-out
body of get_local_u, element.cpp:38-52) and the Brownian force of
get_f_rand (element.cpp:109-144) drawn from Philox-4x32-10: the plain-FP64
step with either or both on matches the oracle to the FP64 bars of the
reference step (relative L2 <= 1e-10); the transcendental functions of the
Box-Muller draw may differ by an ulp between the GPU and the host.
"""
import numpy as np
import pytest

from conftest import rel_l2, seeded_state

pytestmark = pytest.mark.gpu

CASES = {"couple": (True, 0.0), "brownian": (False, 1.0), "both": (True, 1.0)}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("name", ["t32", "t32_2pi"])
def test_extensions_fp64_match_oracle(fipi, oracle_mod, name, case):
    couple, kt = CASES[case]
    w = fipi.workload(name)
    P, c, p, r, ct = seeded_state(w, 31)
    if name == "t32_2pi":
        kt *= 1e-6  # mu = 1e-3, r = 0.06: keep the Brownian step well inside a cell
    port = oracle_mod.Port(P)
    port.set_state(c, p, r, ct)
    port.set_extensions(couple, kt, 5)
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c)
        s.set_particles(p, r, ct)
        s.set_fluid_coupling(couple)
        s.set_brownian(kt, 5)
        for step in range(w.steps):
            s.step(1)
            assert port.step(1) == 0
            pp, pf, _ = port.particles()
            gp, gf, _ = s.get_particles()
            assert rel_l2(s.get_phase(), port.phase()) < 1e-10, step
            assert rel_l2(s.get_velocity(), port.velocity()) < 1e-10, step
            assert rel_l2(gp, pp) < 1e-10, step
            assert rel_l2(gf, pf) < 1e-9, step
        # the extension moved the particles
        with fipi.Simulation(P, "fp64") as s0:
            s0.set_phase(c)
            s0.set_particles(p, r, ct)
            s0.step(w.steps)
            assert not np.array_equal(s0.get_particles()[0], gp)


def test_extensions_mixed_and_switching(fipi):
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 32)
    out = {}
    for prec in ("fp64", "mixed"):
        with fipi.Simulation(P, prec) as s:
            s.set_phase(c)
            s.set_particles(p, r, ct)
            s.step(1)                       # captured graph without extensions
            s.set_fluid_coupling(True)
            s.set_brownian(1.0, 9)
            s.step(2)
            s.set_brownian(0.0)
            s.set_fluid_coupling(False)
            s.step(1)
            out[prec] = s.get_particles()[0]
            assert np.all(np.isfinite(out[prec]))
    assert np.abs(out["mixed"] - out["fp64"]).max() < 1e-4


def test_adjoint_rejects_extensions(fipi):
    w = fipi.workload("t16")
    P, c, p, r, ct = seeded_state(w, 33)
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c)
        s.set_particles(p, r, ct)
        s.set_brownian(1.0, 1)
        with pytest.raises(fipi.FipiError):
            s.adjoint_seed(dc=np.ones(w.V))
