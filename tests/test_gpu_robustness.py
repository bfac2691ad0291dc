"""Error paths and the mass-conserving mode, through the C ABI.

* The mass-conserving mode (fipi_set_mass_conserving) against the oracle's
  restatement of it, and the integral of phi it keeps to 1e-12.
* The range guard of the mixed form's fixed-point spreading: a host-made
  force that no 64-bit accumulator of 2^-32 units holds must come back as
  FIPI_ERR_RANGE, and the context must step normally afterwards.
* The bounded waits of the Y pass: a test hook makes every block's first
  bulk-copy wait give up at once; the call must return FIPI_ERR_TIMEOUT
  (the block drains its copies in flight before it returns) and the next
  call, with the hook off, must be exact again.  No fault is provoked: the
  wait gives up on a copy that does land, and the drain waits for it.
"""
import numpy as np
import pytest

from conftest import rel_l2, seeded_state

pytestmark = pytest.mark.gpu

FIPI_ERR_RANGE = 9
FIPI_ERR_TIMEOUT = 10


def _drift(m, m0, c, P):
    dv = P.lx * P.ly * P.lz / (P.nx * P.ny * P.nz)
    return abs(m - m0) / (np.abs(c).sum() * dv)


@pytest.mark.parametrize("name", ["t32", "t32_bo"])
def test_mass_conserving_fp64_matches_oracle(fipi, oracle_mod, name):
    w = fipi.workload(name)
    P, c, p, r, ct = seeded_state(w, 31)
    port = oracle_mod.Port(P)
    port.set_state(c, p, r, ct)
    port.set_mass_conserving(True)
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c)
        s.set_particles(p, r, ct)
        s.set_mass_conserving(True)
        m0 = s.mass()
        for step in range(4):
            s.step(1)
            assert port.step(1) == 0
            assert rel_l2(s.get_phase(), port.phase()) < 1e-10, step
            assert rel_l2(s.get_velocity(), port.velocity()) < 1e-10, step
            assert rel_l2(s.get_particles()[0], port.particles()[0]) < 1e-12, step
        assert _drift(s.mass(), m0, c, P) <= 1e-12


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_mass_conserving_keeps_the_integral(fipi, prec):
    """cfg1_64 over 30 steps: the reference's drift without the mode, none
    (<= 1e-12 of sum |phi| dV) with it."""
    w = fipi.workload("cfg1_64")
    P, c, p, r, ct = seeded_state(w, 32)
    drift = {}
    for on in (False, True):
        with fipi.Simulation(P, prec) as s:
            s.set_phase(c)
            s.set_particles(p, r, ct)
            s.set_mass_conserving(on)
            m0 = s.mass()
            s.step(30)
            drift[on] = _drift(s.mass(), m0, c, P)
    assert drift[True] <= 1e-12, drift
    assert drift[False] > 10 * max(drift[True], 1e-16), drift  # the reference's Nyquist drift is there without it


def test_spread_range_guard(fipi):
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 33)
    n = w.n_p
    with fipi.Simulation(P, "mixed") as s:
        s.set_phase(c)
        big = np.zeros(3 * n)
        big[3 * 5] = 1e12  # spread at the next step: far beyond 2^31 units per node
        s.set_particles(p, r, ct, big)
        with pytest.raises(fipi.FipiError) as e:
            s.step(1)
        assert e.value.code == FIPI_ERR_RANGE
        # the context is usable again once its state is set anew
        s.set_phase(c)
        s.set_velocity(np.zeros(3 * w.V))
        s.set_particles(p, r, ct)
        s.step(2)
        assert np.isfinite(s.get_phase()).all()
    # contributions each inside the bound whose sum at one node is not:
    # every particle on the same grid node (weight 1 there) with 1e8 units
    pile = np.tile(np.array([8.0, 8.0, 8.0]), n)
    fx = np.zeros(3 * n)
    fx[0::3] = 1e8
    with fipi.Simulation(P, "mixed") as s:
        s.set_phase(c)
        s.set_particles(pile, r, ct, fx)
        with pytest.raises(fipi.FipiError) as e:
            s.step(1)
        assert e.value.code == FIPI_ERR_RANGE
    # a force the accumulators do hold gives the FP64 form's spread
    ok = np.zeros(3 * n)
    ok[3 * 5 + 2] = 1e6
    with fipi.Simulation(P, "mixed") as s:
        s.set_phase(c)
        s.set_particles(p, r, ct, ok)
        s.step(1)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_ypass_wait_timeout_reports_and_recovers(fipi, prec):
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 34)
    x = np.random.default_rng(8).standard_normal(w.V)
    hook = fipi.lib.FIPI_DEBUG_FFT_FIRST_WAIT_POLLS
    with fipi.Simulation(P, prec) as s2:  # the undisturbed run
        s2.set_phase(c)
        s2.set_particles(p, r, ct)
        s2.step(2)
        ref_c = s2.get_phase()
    with fipi.Simulation(P, prec) as s:
        ref = s.fft_r2c(x)
        s.set_debug(hook, 0)
        with pytest.raises(fipi.FipiError) as e:
            s.fft_r2c(x)
        assert e.value.code == FIPI_ERR_TIMEOUT
        s.set_debug(hook, -1)
        assert np.array_equal(s.fft_r2c(x), ref)
        # a step whose Y passes give up, then the same run from the start
        s.set_phase(c)
        s.set_particles(p, r, ct)
        s.set_debug(hook, 0)
        with pytest.raises(fipi.FipiError) as e:
            s.step(1)
        assert e.value.code == FIPI_ERR_TIMEOUT
        s.set_debug(hook, -1)
        s.set_phase(c)
        s.set_velocity(np.zeros(3 * w.V))
        s.set_particles(p, r, ct)
        s.step(2)
        assert np.array_equal(s.get_phase(), ref_c)
