"""Checkpoints and the FP64 adjoint through the C ABI.

- checkpoint resume is bit-exact (both forms), also through export/import;
- the adjoint gradient of a linear functional of the final state matches
  central finite differences of the FP64 forward path along random
  directions in c0, u0, the positions and f_pp (the coupled path: CH,
  Stokes, both Heun stages, contact forces, spreading);
- the sqrt(N)-checkpointed trajectory gives the same gradient as reversing
  every step from a stored state;
- the torch.autograd.Function harness on a structure-factor loss agrees
  with finite differences to 1e-3.
"""
import numpy as np
import pytest

from conftest import seeded_state

pytestmark = pytest.mark.gpu


def _state(sim):
    p, fpp, _ = sim.get_particles() if sim.n else (None, None, None)
    return sim.get_phase(), sim.get_velocity(), p, fpp


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_checkpoint_resume_bit_exact(fipi, prec):
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 5)
    with fipi.Simulation(P, prec) as s:
        s.set_phase(c)
        s.set_particles(p, r, ct)
        s.step(3)
        s.checkpoint_reserve(2)
        s.checkpoint_save(0)
        s.step(4)
        a = _state(s)
        t_a = s.time
        s.checkpoint_load(0)
        assert s.time == 3
        s.step(4)
        b = _state(s)
        assert s.time == t_a
        for x, y in zip(a, b):
            if x is not None:
                assert np.array_equal(x, y)
        blob = s.checkpoint_export(0)
        assert blob[:8] == b"FIPICKP1"
        s.checkpoint_import(1, blob)
        s.checkpoint_load(1)
        s.step(4)
        for x, y in zip(a, _state(s)):
            if x is not None:
                assert np.array_equal(x, y)


def _linear_loss(sim, w):
    c, u, p, fpp = _state(sim)
    L = np.dot(w["c"], c) + np.dot(w["u"], u)
    if sim.n:
        L += np.dot(w["p"], p) + np.dot(w["f"], fpp)
    return L


def _run(fipi, P, c0, u0, p0, r, ct, f0, nsteps, w):
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c0)
        s.set_velocity(u0)
        s.set_particles(p0, r, ct, f0)
        s.step(nsteps)
        return _linear_loss(s, w)


@pytest.mark.parametrize("what", ["c", "u", "p", "f"])
def test_adjoint_matches_finite_differences(fipi, what):
    w_ = fipi.workload("t32")
    P, c0, p0, r, ct = seeded_state(w_, 7)
    V, n = w_.V, w_.n_p
    rng = np.random.default_rng(11)
    u0 = 0.05 * rng.standard_normal(3 * V)
    f0 = 0.2 * rng.standard_normal(3 * n)
    nsteps = 4
    wts = {"c": rng.standard_normal(V), "u": rng.standard_normal(3 * V), "p": rng.standard_normal(3 * n),
           "f": rng.standard_normal(3 * n)}
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c0)
        s.set_velocity(u0)
        s.set_particles(p0, r, ct, f0)
        s.trajectory_forward(nsteps, 2)
        s.trajectory_backward(wts["c"], wts["u"], wts["p"], wts["f"])
        dc, du, dp, df = s.adjoint_get()
    grads = {"c": dc, "u": du, "p": dp, "f": df}
    d = rng.standard_normal(grads[what].size)
    # steps sized so the central difference is neither truncation- nor
    # roundoff-limited (the loss is O(100), f_pp0 enters only through one
    # spreading)
    h = {"c": 1e-6, "u": 1e-4, "p": 1e-7, "f": 1e-3}[what]
    args = {"c": c0, "u": u0, "p": p0, "f": f0}

    def L(x):
        a = dict(args)
        a[what] = x
        return _run(fipi, P, a["c"], a["u"], a["p"], r, ct, a["f"], nsteps, wts)

    fd = (L(args[what] + h * d) - L(args[what] - h * d)) / (2 * h)
    ad = float(np.dot(grads[what], d))
    assert abs(fd) > 0
    assert abs(ad - fd) <= 1e-5 * abs(fd), (what, ad, fd)


def test_checkpointed_trajectory_equals_stepwise(fipi):
    w_ = fipi.workload("t32")
    P, c0, p0, r, ct = seeded_state(w_, 9)
    rng = np.random.default_rng(2)
    wc = rng.standard_normal(w_.V)
    nsteps = 5
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c0)
        s.set_particles(p0, r, ct)
        s.trajectory_forward(nsteps, 2)  # 3 segments of <= 2 steps
        s.trajectory_backward(wc)
        g1 = s.adjoint_get()
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c0)
        s.set_particles(p0, r, ct)
        s.checkpoint_reserve(nsteps)
        for k in range(nsteps):
            s.checkpoint_save(k)
            s.step(1)
        s.adjoint_seed(wc)
        for k in reversed(range(nsteps)):
            s.adjoint_step(k)
        g2 = s.adjoint_get()
    for a, b in zip(g1, g2):
        assert np.array_equal(a, b)


def test_adjoint_rejects_mixed_and_bad_slots(fipi):
    w_ = fipi.workload("t32")
    P, c0, p0, r, ct = seeded_state(w_, 3)
    with fipi.Simulation(P, "mixed") as s:
        s.set_phase(c0)
        with pytest.raises(fipi.FipiError) as e:
            s.adjoint_seed(np.zeros(w_.V))
        assert e.value.code == 8  # FIPI_ERR_UNSUPPORTED
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c0)
        s.set_particles(p0, r, ct)
        s.checkpoint_reserve(1)
        s.checkpoint_save(0)
        s.step(2)
        s.adjoint_seed(np.ones(w_.V))
        with pytest.raises(fipi.FipiError) as e:
            s.adjoint_step(0)  # slot holds t = 0, cotangent refers to t = 2
        assert e.value.code == 7  # FIPI_ERR_STATE
        with pytest.raises(fipi.FipiError):
            s.checkpoint_load(3)


def test_structure_factor_gradient_harness(fipi):
    torch = pytest.importorskip("torch")
    from fipi_gb300 import gradcheck as G

    w_ = fipi.workload("t32")
    P, c0, p0, r, ct = seeded_state(w_, 4)
    init = G.InitialState(p0=p0, r=r, cos_theta=ct)
    Pt, ct0, _, _, _ = seeded_state(w_, 40)
    target = G.structure_factor(torch.from_numpy(ct0), (P.nz, P.ny, P.nx))
    rng = np.random.default_rng(5)
    d = rng.standard_normal(w_.V)
    with fipi.Simulation(P, "fp64") as s:
        res = G.fd_check(s, c0, init, 6, target, d, 1e-6, stride=3)
    assert res["rel"] < 1e-3, res
