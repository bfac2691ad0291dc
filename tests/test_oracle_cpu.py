"""The CPU oracle against the reference: golden vectors generated by the
reference itself (tests/golden/), the live compiled reference where its
sources exist, and the transform against numpy.fft."""
import numpy as np
import pytest

from conftest import rel_l2

GOLDEN = ["t16", "t32", "t32_aniso", "t32_2pi"]


def load_golden(name):
    from pathlib import Path

    d = np.load(Path(__file__).parent / "golden" / f"{name}.npz")
    c0 = d["c0_lattice"].astype(np.float64) / 1e3 * 0.2 - 0.1
    return d, c0


# ------------------------------------------------------------------ transform
@pytest.mark.parametrize("shape", [(16, 16, 16), (8, 16, 32), (32, 32, 32)])
def test_fft_against_numpy(oracle_mod, shape):
    from fipi_gb300.params import FipiParams

    P = FipiParams()
    P.nz, P.ny, P.nx = shape
    rng = np.random.default_rng(0)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    X = oracle_mod.fft3(P, x.ravel(), -1).reshape(shape)
    assert rel_l2(X.view(float), np.fft.fftn(x).view(float)) < 1e-14
    y = oracle_mod.fft3(P, X.ravel(), +1).reshape(shape) / x.size
    assert rel_l2(y.view(float), x.view(float)) < 1e-14
    # delta -> ones; single mode -> one spike of size V
    d = np.zeros(shape, complex)
    d[0, 0, 0] = 1
    assert np.allclose(oracle_mod.fft3(P, d.ravel(), -1), 1.0, atol=1e-15)
    k, j, i = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    m = np.exp(2j * np.pi * (1 * k / shape[0] + 2 * j / shape[1] + 3 * i / shape[2]))
    M = oracle_mod.fft3(P, m.ravel(), -1).reshape(shape)
    assert abs(M[1, 2, 3] - x.size) < 1e-9
    M[1, 2, 3] = 0
    assert np.abs(M).max() < 1e-9


# ------------------------------------------------------------------ golden vectors
@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_step_matches_golden(oracle_mod, name):
    from fipi_gb300.params import workload

    d, c0 = load_golden(name)
    w = workload(name)
    port = oracle_mod.Port(w.params())
    port.set_state(c0, d["p0"])
    assert port.step(int(d["steps"])) == 0
    p, fpp, fpi = port.particles()
    # bit-exact on the host the vectors were generated on; libm may differ
    # in the last ulp elsewhere, so the bar is 1e-12
    assert rel_l2(port.phase(), d["phase"]) < 1e-12
    if d["velocity"].size:
        assert rel_l2(port.velocity(), d["velocity"]) < 1e-12
    assert abs(np.linalg.norm(port.velocity()) - d["velocity_l2"]) <= 1e-12 * d["velocity_l2"]
    assert rel_l2(p, d["p"]) < 1e-14
    assert rel_l2(fpp, d["f_pp"]) < 1e-11
    assert rel_l2(fpi, d["f_pi"]) < 1e-11
    assert abs(port.tau() - d["tau"]) <= 1e-11 * max(1.0, abs(d["tau"]))
    assert abs(port.free_energy() - d["free_energy"]) <= 1e-12 * abs(d["free_energy"])


@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_particle_calls_match_golden(oracle_mod, name):
    from fipi_gb300.params import workload

    d, _ = load_golden(name)
    P = workload(name).params()
    st, keys, srt, off, mark = oracle_mod.sorting(P, d["p0"])
    assert st == 0
    assert np.array_equal(keys, d["keys"])
    assert np.array_equal(srt, d["sorted"])
    assert np.array_equal(off, d["offsets"])
    assert mark == int(d["it_mark"])
    st, fpp, tau, _ = oracle_mod.f_pp(P, d["p0"], 3, d["f_pi_in"])
    assert st == 0
    assert np.array_equal(fpp, d["f_pp0"])
    assert tau == float(d["tau0"])
    sp = oracle_mod.spread(P, d["p0"], d["f_pp0"])
    idx = np.nonzero(sp)[0]
    assert np.array_equal(idx, d["spread_idx"])
    assert np.array_equal(sp[idx], d["spread_val"])


# ------------------------------------------------------------------ live reference
def _ref_or_skip(oracle_mod):
    if not oracle_mod.reference_available():
        pytest.skip("reference sources not present on this host")


@pytest.mark.parametrize("name", GOLDEN + ["t256x", "t512x", "t32_bo", "t256yz"])
def test_oracle_bit_exact_with_live_reference(oracle_mod, name):
    _ref_or_skip(oracle_mod)
    from fipi_gb300.params import workload

    w = workload(name)
    rng = np.random.default_rng(5)
    c0 = rng.uniform(-0.05, 0.05, w.V)
    p0 = (rng.uniform(0, 1, (w.n_p, 3)) * [w.lx, w.ly, w.lz]).ravel()
    ref = oracle_mod.Ref(name)
    port = oracle_mod.Port(w.params())
    assert ref.init(c0, p0) == 0
    port.set_state(c0, p0)
    for _ in range(w.steps):
        assert ref.step() == 0 and port.step() == 0
        assert np.array_equal(ref.phase(), port.phase())
        assert np.array_equal(ref.phase_imag(), port.phase_imag())
        assert np.array_equal(ref.velocity(), port.velocity())
        for a, b in zip(ref.particles(), port.particles()):
            assert np.array_equal(a, b)
        assert ref.tau() == port.tau()
    assert ref.free_energy() == port.free_energy()


def test_fine_grained_calls_bit_exact_with_live_reference(oracle_mod):
    _ref_or_skip(oracle_mod)
    from fipi_gb300.params import workload

    name = "t32_2pi"
    w = workload(name)
    P = w.params()
    ref = oracle_mod.Ref(name)
    rng = np.random.default_rng(9)
    p = (rng.uniform(0, 1, (w.n_p, 3)) * [w.lx, w.ly, w.lz]).ravel()
    field = rng.uniform(-1, 1, w.V)
    assert np.array_equal(ref.interpolate(field, p), oracle_mod.interpolate(P, field, p))
    c_loc = rng.uniform(-1, 1, w.n_p)
    dcdx = rng.standard_normal(3 * w.n_p)
    assert np.array_equal(ref.f_pi(c_loc, dcdx), oracle_mod.f_pi(P, c_loc, dcdx))
    fpi, fpp = rng.standard_normal(3 * w.n_p), rng.standard_normal(3 * w.n_p)
    a = ref.advect(1, fpi, fpp, None, p, p, np.zeros_like(p))
    b = oracle_mod.advect(P, 1, fpi, fpp, None, p, p, np.zeros_like(p))
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert np.array_equal(ref.gradient(field), oracle_mod.grad(P, field))
    data = rng.standard_normal(w.V) + 1j * rng.standard_normal(w.V)
    assert np.array_equal(ref.fft(data, -1), oracle_mod.fft3(P, data, -1))


# ------------------------------------------------------------------ edge cases
def test_oracle_out_of_range_particle(oracle_mod):
    from fipi_gb300.params import workload

    w = workload("t32")
    P = w.params()
    p = np.full(3 * w.n_p, 1.0)
    p[5] = w.lx + 1.0  # outside the cell grid: the reference exits (cluster.cpp:144-163)
    st, *_ = oracle_mod.sorting(P, p)
    assert st == 4
    port = oracle_mod.Port(P)
    port.set_state(np.zeros(w.V), p)
    assert port.step() == 4


def test_oracle_rejects_too_few_cells(oracle_mod):
    from fipi_gb300.params import workload

    P = workload("t16").with_(r_p=2.0).params()  # r_c = 10 -> 1 cell per axis
    with pytest.raises(ValueError):
        oracle_mod.Port(P)


def test_oracle_without_particles(oracle_mod):
    from fipi_gb300.params import workload

    w = workload("t16").with_(n_p=0)
    port = oracle_mod.Port(w.params())
    c0 = np.random.default_rng(1).uniform(-0.05, 0.05, w.V)
    port.set_state(c0)
    assert port.step(2) == 0
    assert np.isfinite(port.phase()).all()


@pytest.mark.parametrize("name", ["t16", "t32_aniso", "t32_2pi"])
def test_div_and_interpolate2_bit_exact_with_reference(oracle_mod, name):
    """field::div and field::interpolate2 (dead code in the reference's loop,
    part of the field API): the C restatement equals the reference."""
    if not oracle_mod.reference_available():
        pytest.skip("reference sources absent")
    import fipi_gb300 as F

    w = F.workload(name)
    P = w.params()
    ref = oracle_mod.Ref(name)
    rng = np.random.default_rng(6)
    v = rng.standard_normal(3 * w.V)
    assert np.array_equal(oracle_mod.div(P, v), ref.div(v))
    fld = rng.standard_normal(w.V)
    p = (rng.random((50, 3)) * np.array([P.lx, P.ly, P.lz])).ravel()
    assert np.array_equal(oracle_mod.interpolate2(P, fld, p), ref.interpolate2(fld, p))


def test_oracle_mass_conserving_mode(oracle_mod):
    """The library's mass-conserving mode restated in the oracle: without it
    the reference's Nyquist drift of the integral of phi is there, with it
    the integral stays constant to rounding."""
    from fipi_gb300.params import workload

    w = workload("t32")
    P = w.params()
    rng = np.random.default_rng(12)
    c0 = rng.uniform(-0.05, 0.05, w.V)
    p0 = (rng.uniform(0, 1, (w.n_p, 3)) * [w.lx, w.ly, w.lz]).ravel()
    dv = w.lx * w.ly * w.lz / w.V
    drift = {}
    for on in (False, True):
        port = oracle_mod.Port(P)
        port.set_state(c0, p0)
        port.set_mass_conserving(on)
        m0 = port.mass()
        assert port.step(8) == 0
        drift[on] = abs(port.mass() - m0) / (np.abs(c0).sum() * dv)
    assert drift[True] <= 1e-14, drift
    assert drift[False] > 1e-13, drift
