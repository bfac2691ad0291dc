"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Bars: bit-exact for cell keys, sort order, pair sets, advection and
spreading; relative L2 <= 1e-10 (plain FP64) for phase field, velocity and
positions after several steps; FFT against numpy to ~1e-14 (FP64) and
~1e-6 (FP32).
"""
import os

import numpy as np
import pytest

from conftest import rel_l2, seeded_state

pytestmark = pytest.mark.gpu

SMALL = ["t16", "t32", "t32_aniso", "t32_2pi", "t32_bo", "t256x", "t512x"]
# y and z lengths of the 256^3 and 512^3 workloads (the 256- and 512-point
# Y / Z codelets and tile shapes), plus the CPU-runnable 64^3 case
HEADLINE = ["cfg1_64", "t256yz", "t512yz"]
THREADS = os.cpu_count() or 1  # the oracle's transforms are threaded over independent lines


def half_spectrum_from_numpy(x, P):
    """numpy rfftn in the library's layout [kz][kx][ky] (ky fastest)."""
    a = x.reshape(P.nz, P.ny, P.nx)
    F = np.fft.rfftn(a, axes=(0, 1, 2))  # [kz][ky][kx], kx in [0, nx/2]
    return np.ascontiguousarray(F.transpose(0, 2, 1)).ravel()


@pytest.mark.parametrize("name", SMALL)
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_fft_r2c_c2r(fipi, name, prec):
    w = fipi.workload(name)
    P = w.params()
    if prec == "mixed" and P.ny < 16:
        pytest.skip("mixed form needs ny >= 16")
    rng = np.random.default_rng(3)
    x = rng.standard_normal(w.V)
    with fipi.Simulation(P, prec) as s:
        X = s.fft_r2c(x)
        ref = half_spectrum_from_numpy(x, P)
        tol = 1e-14 if prec == "fp64" else 2e-6
        assert rel_l2(X.view(np.float64), ref.view(np.float64)) < tol
        y = s.fft_c2r(ref)
        assert rel_l2(y, x) < tol


@pytest.mark.parametrize("shape", [(16, 256, 16), (16, 16, 256), (16, 512, 16), (16, 16, 512),
                                   (16, 256, 256), (256, 256, 256)])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_fft_headline_shapes(fipi, shape, prec):
    """R2C / C2R against numpy.rfftn on the axis lengths the 256^3 and
    512^3 workloads transform (the field::fft / ifft of main.cpp:72-73 is
    one 3-D plan over all axes), with the small grids' tolerances."""
    nx, ny, nz = shape
    w = fipi.workload("t32").with_(name="fft", nx=nx, ny=ny, nz=nz, lx=float(nx), ly=float(ny), lz=float(nz),
                                   n_p=0)
    P = w.params()
    rng = np.random.default_rng(nx + 3 * ny + 7 * nz)
    x = rng.standard_normal(w.V)
    with fipi.Simulation(P, prec) as s:
        X = s.fft_r2c(x)
        ref = half_spectrum_from_numpy(x, P)
        tol = 1e-14 if prec == "fp64" else 2e-6
        assert rel_l2(X.view(np.float64), ref.view(np.float64)) < tol
        y = s.fft_c2r(ref)
        assert rel_l2(y, x) < tol
        # a single mode at the largest wave numbers below Nyquist: V/2 at
        # (kx, ky, kz) of the half spectrum and nothing else
        kx, ky, kz = nx // 2 - 1, ny // 2 - 1, nz // 2 - 1
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        m = np.cos(2 * np.pi * (kx * i / nx + ky * j / ny + kz * k / nz)).ravel()
        M = s.fft_r2c(m).reshape(nz, nx // 2 + 1, ny)
        bar = (1e-13 if prec == "fp64" else 2e-6) * w.V
        assert abs(M[kz, kx, ky] - w.V / 2) < bar
        M[kz, kx, ky] = 0
        assert np.abs(M).max() < bar


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_fft_known_answers(fipi, prec):
    w = fipi.workload("t32")
    P = w.params()
    with fipi.Simulation(P, prec) as s:
        # delta at the origin -> flat spectrum of ones
        x = np.zeros(w.V)
        x[0] = 1.0
        X = s.fft_r2c(x)
        assert np.allclose(X, 1.0, atol=1e-6 if prec == "mixed" else 1e-15)
        # single mode cos(2 pi (3x + 5y + 7z)/32) -> V/2 at (3,5,7) of the half spectrum
        i, j, k = np.meshgrid(np.arange(32), np.arange(32), np.arange(32), indexing="ij")
        x = np.cos(2 * np.pi * (3 * k + 5 * j + 7 * i) / 32).ravel()  # x fastest: k is x index
        X = s.fft_r2c(x).reshape(P.nz, P.nx // 2 + 1, P.ny)
        peak = X[7, 3, 5]
        assert abs(peak - w.V / 2) < (1e-9 if prec == "fp64" else 1e-1)
        X[7, 3, 5] = 0
        X[-7, 3, -5] = 0
        assert np.abs(X).max() < (1e-9 if prec == "fp64" else 2e-2)


@pytest.mark.parametrize("name", SMALL)
def test_grad_matches_oracle(fipi, oracle_mod, name):
    w = fipi.workload(name)
    P = w.params()
    c = np.random.default_rng(5).uniform(-1, 1, w.V)
    with fipi.Simulation(P, "fp64") as s:
        g = s.grad(c)
    assert rel_l2(g, oracle_mod.grad(P, c)) < 1e-13


@pytest.mark.parametrize("name", ["t16", "t32", "t32_aniso", "t32_2pi", "cfg1_64"])
def test_cells_bit_exact(fipi, oracle_mod, name):
    w = fipi.workload(name)
    P, c, p, r, ct = seeded_state(w, 11)
    with fipi.Simulation(P, "fp64") as s:
        keys, srt, off = s.cells_build(p)
    st, k2, s2, o2, _ = oracle_mod.sorting(P, p)
    assert st == 0
    assert np.array_equal(keys, k2)
    assert np.array_equal(srt, s2)
    assert np.array_equal(off, o2)


@pytest.mark.parametrize("n_p", [1000, 70000])
def test_cells_bit_exact_one_block_and_multi_block(fipi, oracle_mod, n_p):
    """Up to 65,536 particles the cell list is built by one block, above by
    the multi-block radix sort; both must equal the reference's sorting."""
    w = fipi.workload("cfg1_64")
    P = w.params()
    P.n_p = n_p
    rng = np.random.default_rng(n_p)
    p = (rng.random((n_p, 3)) * np.array([P.lx, P.ly, P.lz])).ravel()
    with fipi.Simulation(P, "fp64") as s:
        keys, srt, off = s.cells_build(p)
    st, k2, s2, o2, _ = oracle_mod.sorting(P, p)
    assert st == 0
    assert np.array_equal(keys, k2)
    assert np.array_equal(srt, s2)
    assert np.array_equal(off, o2)


@pytest.mark.parametrize("name", ["t16", "t32", "t32_aniso", "t32_2pi", "cfg1_64"])
def test_pairs_and_f_pp(fipi, oracle_mod, name):
    w = fipi.workload(name)
    P, c, p, r, ct = seeded_state(w, 12)
    rng = np.random.default_rng(1)
    f_pi = rng.standard_normal(3 * w.n_p) * (rng.random(3 * w.n_p) > 0.3)
    with fipi.Simulation(P, "fp64") as s:
        pairs = s.pairs(p)
        fpp, tau = s.f_pp(p, 3, f_pi)
    st, fpp2, tau2, pairs2 = oracle_mod.f_pp(P, p, 3, f_pi, want_pairs=True)
    assert st == 0
    assert pairs.shape == pairs2.shape and np.array_equal(pairs, pairs2)
    assert rel_l2(fpp, fpp2) < 1e-13
    assert abs(tau - tau2) <= 1e-12 * max(1.0, abs(tau2))


@pytest.mark.parametrize("name", ["t32", "t32_2pi"])
def test_interpolate_f_pi_advect_spread(fipi, oracle_mod, name):
    w = fipi.workload(name)
    P, c, p, r, ct = seeded_state(w, 13)
    rng = np.random.default_rng(2)
    fields = rng.uniform(-1, 1, 4 * w.V)
    with fipi.Simulation(P, "fp64") as s:
        vals = s.interpolate(fields, p)
        for f in range(4):
            ref = oracle_mod.interpolate(P, fields[f * w.V:(f + 1) * w.V], p)
            assert np.array_equal(vals[:, f], ref)
        c_loc = rng.uniform(-1, 1, w.n_p)
        dcdx = rng.standard_normal(3 * w.n_p)
        cth = rng.uniform(-0.5, 0.5, w.n_p)
        for cos_t in (None, cth):
            fpi = s.f_pi(c_loc, dcdx, None, cos_t)
            ref = oracle_mod.f_pi(P, c_loc, dcdx, None, cos_t)
            assert np.allclose(fpi, ref, rtol=1e-14, atol=1e-300)
        fpp = rng.standard_normal(3 * w.n_p)
        fpi = rng.standard_normal(3 * w.n_p)
        p_old = p.copy()
        u_old = np.zeros(3 * w.n_p)
        a = s.advect(1, fpi, fpp, None, p, p_old, u_old)
        b = oracle_mod.advect(P, 1, fpi, fpp, None, p, p_old, u_old)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
        a2 = s.advect(2, fpi * 0.5, fpp, None, *a)
        b2 = oracle_mod.advect(P, 2, fpi * 0.5, fpp, None, *b)
        for x, y in zip(a2, b2):
            assert np.array_equal(x, y)
        sp = s.spread(p, fpp)
        assert np.array_equal(sp, oracle_mod.spread(P, p, fpp))


@pytest.mark.parametrize("name", SMALL + HEADLINE)
def test_step_fp64_matches_oracle(fipi, oracle_mod, name):
    w = fipi.workload(name)
    w = w.with_(steps=min(w.steps, 3))
    P, c, p, r, ct = seeded_state(w, 21)
    port = oracle_mod.Port(P, threads=THREADS)
    port.set_state(c, p, r, ct)
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c)
        s.set_particles(p, r, ct)
        for step in range(w.steps):
            s.step(1)
            assert port.step(1) == 0
            pc, pu = port.phase(), port.velocity()
            pp, pf, _ = port.particles()
            gc, gu = s.get_phase(), s.get_velocity()
            gp, gf, _ = s.get_particles()
            assert rel_l2(gc, pc) < 1e-10, step
            assert rel_l2(gu, pu) < 1e-10, step
            assert rel_l2(gp, pp) < 1e-12, step
            assert rel_l2(gf, pf) < 1e-10, step
        assert s.time == w.steps
        assert abs(s.free_energy() - port.free_energy()) <= 1e-10 * abs(port.free_energy())
        assert abs(s.mass() - port.mass()) <= 1e-12 * np.abs(c).sum()
        assert abs(s.packing_tau() - port.tau()) <= 1e-9 * max(1.0, abs(port.tau()))


def test_cfg2_256_matches_oracle(fipi, oracle_mod):
    """The 256^3, 20,000-sphere workload itself, two steps (the IMEX start
    and the first SBDF2 step) from the seeded state: the FP64 form within
    the parity bars of the oracle, the mixed form within its stated error."""
    w = fipi.workload("cfg2_256")
    P, c, p, r, ct = seeded_state(w, 1)
    port = oracle_mod.Port(P, threads=THREADS)
    port.set_state(c, p, r, ct)
    sims = {prec: fipi.Simulation(P, prec) for prec in ("fp64", "mixed")}
    try:
        for s in sims.values():
            s.set_phase(c)
            s.set_particles(p, r, ct)
        for step in range(2):
            assert port.step(1) == 0
            pc, pu = port.phase(), port.velocity()
            pp, pf, _ = port.particles()
            for s in sims.values():
                s.step(1)
            g = sims["fp64"]
            gp, gf, _ = g.get_particles()
            assert rel_l2(g.get_phase(), pc) < 1e-10, step
            assert rel_l2(g.get_velocity(), pu) < 1e-10, step
            assert rel_l2(gp, pp) < 1e-12, step
            assert rel_l2(gf, pf) < 1e-10, step
            m = sims["mixed"]
            assert rel_l2(m.get_phase(), pc) < 1e-5, step
            assert rel_l2(m.get_velocity(), pu) < 1e-3, step
            assert rel_l2(m.get_particles()[0], pp) < 1e-8, step
        assert abs(g.mass() - port.mass()) <= 1e-12 * np.abs(c).sum()
        assert abs(g.free_energy() - port.free_energy()) <= 1e-10 * abs(port.free_energy())
    finally:
        for s in sims.values():
            s.close()


@pytest.mark.parametrize("name", ["t32", "t32_2pi", "cfg1_64", "t256x"])
def test_step_mixed_close_to_fp64(fipi, name):
    w = fipi.workload(name)
    P, c, p, r, ct = seeded_state(w, 22)
    steps = 5
    out = {}
    for prec in ("fp64", "mixed"):
        with fipi.Simulation(P, prec) as s:
            s.set_phase(c)
            s.set_particles(p, r, ct)
            m0 = s.mass()
            s.step(steps)
            out[prec] = (s.get_phase(), s.get_velocity(), s.get_particles()[0], s.mass(), m0)
    a, b = out["mixed"], out["fp64"]
    assert rel_l2(a[0], b[0]) < 1e-5
    assert rel_l2(a[1], b[1]) < 1e-3
    assert np.abs(a[2] - b[2]).max() < 1e-6
    # The mixed form carries the k = 0 mode in FP64 and follows the FP64
    # mass history (the reference's own drift comes from its Nyquist-plane
    # projection, so it is matched, not removed).
    assert abs(a[3] - b[3]) <= 1e-11 * np.abs(c).sum()


def test_deterministic(fipi):
    w = fipi.workload("cfg1_64")
    P, c, p, r, ct = seeded_state(w, 23)
    res = []
    for _ in range(2):
        with fipi.Simulation(P, "mixed") as s:
            s.set_phase(c)
            s.set_particles(p)
            s.step(3)
            res.append((s.get_phase(), s.get_particles()[0]))
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_graph_replay_matches_direct_launches(fipi, prec):
    """Steps t >= 1 replay CUDA graphs; with kernel timing on they launch
    directly.  Both must give the same bits."""
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 25)
    res = []
    for timing in (False, True):
        with fipi.Simulation(P, prec) as s:
            s.set_phase(c)
            s.set_particles(p)
            s.set_kernel_timing(timing)
            for _ in range(3):  # odd count: both buffer states and the step-by-step path
                s.step(1)
            s.step(2)
            res.append((s.get_phase(), s.get_velocity(), s.get_particles()[0], s.packing_tau()))
            if timing:
                assert any(k["launches"] > 0 for k in s.kernel_stats())
    for x, y in zip(res[0][:3], res[1][:3]):
        assert np.array_equal(x, y)
    assert res[0][3] == res[1][3]


def test_out_of_range_particle_reports_error(fipi):
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 24)
    p = p.copy()
    p[0] = -5.0  # outside [0, L): cluster::sorting would exit(0)
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c)
        s.set_particles(p)
        with pytest.raises(fipi.FipiError) as e:
            s.step(1)
        assert e.value.code == 4
        with pytest.raises(fipi.FipiError):
            s.cells_build(p)


def test_full_size_512_forms_agree(fipi):
    """The 512³, 200,000-sphere workload (polydisperse radii, contact angles)
    at full size, where the oracle cannot follow: both forms run, stay
    finite, agree with each other to mixed-precision accuracy, keep the same
    mass history, and the FP64 form is deterministic."""
    w = fipi.workload("cfg3_512")
    P, c, p, r, ct = seeded_state(w, 3)
    res = {}
    for prec in ("fp64", "mixed"):
        with fipi.Simulation(P, prec) as s:
            s.set_phase(c)
            s.set_particles(p, r, ct)
            m0 = s.mass()
            s.step(2)
            res[prec] = (s.get_phase(), s.get_particles()[0], s.mass(), m0)
    a, b = res["mixed"], res["fp64"]
    assert np.isfinite(a[0]).all() and np.isfinite(b[0]).all()
    assert rel_l2(a[0], b[0]) < 1e-5
    L = np.array([P.lx, P.ly, P.lz])
    d = np.abs(a[1] - b[1]).reshape(-1, 3)
    assert np.minimum(d, L - d).max() < 1e-5
    scale = np.abs(c).sum() * P.lx * P.ly * P.lz / w.V
    assert abs((a[2] - a[3]) - (b[2] - b[3])) < 1e-12 * scale
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c)
        s.set_particles(p, r, ct)
        s.step(2)
        assert np.array_equal(s.get_phase(), b[0])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_substeps_equal_step(fipi, prec):
    """fipi_step_ch + fipi_step_stokes + fipi_step_particles == fipi_step(1),
    bit for bit; out-of-order calls are refused."""
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 31)
    res = []
    for split in (False, True):
        with fipi.Simulation(P, prec) as s:
            s.set_phase(c)
            s.set_particles(p, r, ct)
            for _ in range(3):
                if split:
                    s.step_ch()
                    s.step_stokes()
                    s.step_particles()
                else:
                    s.step(1)
            res.append((s.get_phase(), s.get_velocity(), s.get_particles()[0], s.time))
            if split:
                with pytest.raises(fipi.FipiError):
                    s.step_stokes()
                s.step_ch()
                with pytest.raises(fipi.FipiError):
                    s.step(1)
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b)


def test_wrap_matches_oracle(fipi, oracle_mod):
    w = fipi.workload("t32")
    P = w.params()
    rng = np.random.default_rng(8)
    p = (rng.random(3 * w.n_p) * 3 - 1) * 32.0  # inside and outside [0, L)
    L = P.lx
    edges = np.array([-L, -0.0, 0.0, L - 2 ** -48, L, 2 * L, -L - 2 ** -40, 3 * L + 0.5, 1e300, -1e300,
                      np.nextafter(-L, 0.0), np.nextafter(L, 0.0), np.inf, -np.inf, np.nan])
    p[:len(edges)] = edges
    with fipi.Simulation(P, "fp64") as s:
        got = s.wrap(p)
    ref = oracle_mod.enforce_bc(P, p)
    # bit for bit, signed zeros included; NaN where the oracle has NaN (the
    # payload of a NaN made by fmod is the platform's)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.int64), ref[~nan].view(np.int64))


def test_write_vtk_from_context(fipi, tmp_path):
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 33)
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c)
        s.set_particles(p, r, ct)
        s.write_vtk("phase", tmp_path / "a.vtk")
        fipi.vtk_write_field(P, tmp_path / "b.vtk", "phase", c, 1)
        assert (tmp_path / "a.vtk").read_bytes() == (tmp_path / "b.vtk").read_bytes()
        s.step(2)
        s.write_vtk("u", tmp_path / "u.vtk")
        fipi.vtk_write_field(P, tmp_path / "u2.vtk", "u", s.get_velocity(), 3)
        assert (tmp_path / "u.vtk").read_bytes() == (tmp_path / "u2.vtk").read_bytes()
        s.write_vtk("particles", tmp_path / "p.vtk")
        pos, fpp, _ = s.get_particles()
        fipi.vtk_write_particles(P, tmp_path / "p2.vtk", pos, r, fpp)
        assert (tmp_path / "p.vtk").read_bytes() == (tmp_path / "p2.vtk").read_bytes()
        s.write_vtk("free_energy", tmp_path / "fe.vtk")
        lines = (tmp_path / "fe.vtk").read_text().splitlines()
        assert lines[9] == "SCALARS free_energy double" and len(lines) == 11 + w.V
        vals = np.array([float(x) for x in lines[11:]])
        dx = P.lx / P.nx
        assert abs(vals.sum() * dx ** 3 - s.free_energy()) < 1e-4 * abs(s.free_energy())


@pytest.mark.parametrize("name", ["t16", "t32_aniso", "t32_2pi"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_div_and_interpolate2(fipi, oracle_mod, name, prec):
    """field::div and field::interpolate2 (field API, not in the loop)."""
    w = fipi.workload(name)
    P = w.params()
    if prec == "mixed" and P.ny < 16:
        pytest.skip("mixed form needs ny >= 16")
    rng = np.random.default_rng(12)
    v = rng.standard_normal(3 * w.V)
    fld = rng.standard_normal(w.V)
    p = (rng.random((w.n_p, 3)) * np.array([P.lx, P.ly, P.lz])).ravel()
    with fipi.Simulation(P, prec) as s:
        d = s.div(v)
        i2 = s.interpolate2(fld, p).ravel()
    d_ref = oracle_mod.div(P, v)
    i_ref = oracle_mod.interpolate2(P, fld, p)
    if prec == "fp64":
        assert rel_l2(d, d_ref) < 1e-12
        assert np.array_equal(i2, i_ref)
    else:
        assert rel_l2(d, d_ref) < 1e-5
        assert rel_l2(i2, i_ref) < 1e-6

