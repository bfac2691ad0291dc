"""Gradients with respect to the step's parameters through the FP64 adjoint.

The loss is a random linear functional of the final state (c, u, positions,
f_pp) after four steps (the IMEX start and three SBDF2 steps) of the t32
case, with contact forces active and per-particle wettabilities cos(theta)
away from 90 degrees.  The adjoint's cotangents of the mobility M, of
lambda, k_n and sigma (through f_pi alone, and in total with lambda =
3 sigma eps / (2 sqrt 2) and k_n = sigma / 2 following it) and of every
particle's cos(theta) (along a random direction) are checked against

* central finite differences of the FP64 GPU forward step (h = 1e-6
  relative), and
* an FP64 reference gradient independent of the GPU: central finite
  differences of the CPU oracle (the C restatement of the reference step,
  itself pinned bit for bit to the compiled reference).

Bar: 1e-3 relative (the gradient-check target); in practice the two agree
far closer (the branches of the step -- interpolation cells, |phi| <= tanh 2,
|d| < r, |d| < r_eq -- do not flip at these steps).
"""
import numpy as np
import pytest

from conftest import seeded_state

pytestmark = pytest.mark.gpu

NSTEPS = 4
SQ2 = np.sqrt(2.0)


def _case(fipi):
    w = fipi.workload("t32")
    P, c0, p0, r, _ = seeded_state(w, 61)
    rng = np.random.default_rng(62)
    ct = rng.uniform(-0.6, 0.6, w.n_p)
    u0 = 0.05 * rng.standard_normal(3 * w.V)
    wts = {"c": rng.standard_normal(w.V), "u": rng.standard_normal(3 * w.V), "p": rng.standard_normal(3 * w.n_p),
           "f": rng.standard_normal(3 * w.n_p)}
    dct = rng.standard_normal(w.n_p)
    return w, P, c0, u0, p0, r, ct, wts, dct


def _loss(c, u, p, f, wts):
    return float(np.dot(wts["c"], c) + np.dot(wts["u"], u) + np.dot(wts["p"], p) + np.dot(wts["f"], f))


def _perturbed(P, what, h):
    """Parameters with `what` moved by h (sigma: lambda and k_n follow)."""
    Q = type(P).from_buffer_copy(P)
    if what == "mobility":
        Q.mobility += h
    elif what == "lambda":
        Q.lambda_ += h
    elif what == "k_n":
        Q.k_n += h
    elif what == "sigma_attach":
        Q.sigma += h
    elif what == "sigma":
        Q.sigma += h
        Q.lambda_ = Q.sigma * Q.epsilon * 3.0 / 2.0 / SQ2
        Q.k_n = 0.5 * Q.sigma
    return Q


def _gpu_loss(fipi, P, c0, u0, p0, r, ct, wts):
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c0)
        s.set_velocity(u0)
        s.set_particles(p0, r, ct)
        s.step(NSTEPS)
        p, f, _ = s.get_particles()
        return _loss(s.get_phase(), s.get_velocity(), p, f, wts)


def _oracle_loss(oracle_mod, P, c0, u0, p0, r, ct, wts):
    port = oracle_mod.Port(P)
    port.set_state(c0, p0, r, ct, u=u0)
    assert port.step(NSTEPS) == 0
    p, f, _ = port.particles()
    return _loss(port.phase(), port.velocity(), p, f, wts)


@pytest.fixture(scope="module")
def adjoint_grads(fipi):
    w, P, c0, u0, p0, r, ct, wts, dct = _case(fipi)
    with fipi.Simulation(P, "fp64") as s:
        s.set_phase(c0)
        s.set_velocity(u0)
        s.set_particles(p0, r, ct)
        s.trajectory_forward(NSTEPS, 2)
        s.trajectory_backward(wts["c"], wts["u"], wts["p"], wts["f"])
        g, g_ct = s.adjoint_get_params()
    return g, g_ct


@pytest.mark.parametrize("what", ["mobility", "sigma", "lambda", "k_n", "sigma_attach", "cos_theta"])
@pytest.mark.parametrize("by", ["gpu", "oracle"])
def test_parameter_gradient(fipi, oracle_mod, adjoint_grads, what, by):
    w, P, c0, u0, p0, r, ct, wts, dct = _case(fipi)
    g, g_ct = adjoint_grads
    if what == "cos_theta":
        ad = float(np.dot(g_ct, dct))
        h = 1e-6
        args_p = (P, c0, u0, p0, r, ct + h * dct, wts)
        args_m = (P, c0, u0, p0, r, ct - h * dct, wts)
    else:
        ad = g["lambda_" if what == "lambda" else what]
        base = {"mobility": P.mobility, "lambda": P.lambda_, "k_n": P.k_n}.get(what, P.sigma)
        h = 1e-6 * base
        args_p = (_perturbed(P, what, h), c0, u0, p0, r, ct, wts)
        args_m = (_perturbed(P, what, -h), c0, u0, p0, r, ct, wts)
    if by == "gpu":
        fd = (_gpu_loss(fipi, *args_p) - _gpu_loss(fipi, *args_m)) / (2 * h)
    else:
        fd = (_oracle_loss(oracle_mod, *args_p) - _oracle_loss(oracle_mod, *args_m)) / (2 * h)
    assert abs(fd) > 0, (what, fd)
    assert abs(ad - fd) <= 1e-3 * abs(fd), (what, by, ad, fd)


def test_sigma_is_the_chained_sum(adjoint_grads, fipi):
    """sigma's total derivative = through f_pi + lambda' dlambda/dsigma + k_n' / 2."""
    g, _ = adjoint_grads
    P = fipi.workload("t32").params()
    chained = g["sigma_attach"] + g["lambda_"] * P.epsilon * 3.0 / 2.0 / SQ2 + 0.5 * g["k_n"]
    assert abs(g["sigma"] - chained) <= 1e-12 * max(abs(chained), 1.0)


def test_mass_conserving_adjoint_matches_fd(fipi):
    """The adjoint of the mass-conserving mode (C(0) = 0 in the CH update)
    along a direction in c0."""
    w, P, c0, u0, p0, r, ct, wts, _ = _case(fipi)
    d = np.random.default_rng(63).standard_normal(w.V)

    def run(c):
        with fipi.Simulation(P, "fp64") as s:
            s.set_mass_conserving(True)
            s.set_phase(c)
            s.set_velocity(u0)
            s.set_particles(p0, r, ct)
            s.step(NSTEPS)
            p, f, _ = s.get_particles()
            return _loss(s.get_phase(), s.get_velocity(), p, f, wts)

    with fipi.Simulation(P, "fp64") as s:
        s.set_mass_conserving(True)
        s.set_phase(c0)
        s.set_velocity(u0)
        s.set_particles(p0, r, ct)
        s.trajectory_forward(NSTEPS, 2)
        s.trajectory_backward(wts["c"], wts["u"], wts["p"], wts["f"])
        dc = s.adjoint_get()[0]
    h = 1e-6
    fd = (run(c0 + h * d) - run(c0 - h * d)) / (2 * h)
    ad = float(np.dot(dc, d))
    assert abs(ad - fd) <= 1e-5 * abs(fd), (ad, fd)


@pytest.mark.parametrize("init", ["noise", "droplet"])
def test_harness_gradients_match_fd(fipi, init):
    """The torch.autograd.Function of the harness on the two gradient-check
    losses of the benchmark (structure factor against a second seed's, and
    interfacial area + centroid height of a coated droplet): d/dphi0, dM,
    dsigma against central differences (h = 1e-6).  These losses read c
    only, which cos(theta) reaches over five steps only through the spread
    contact forces of displaced particles (a change near the loss's
    rounding), so d/dcos(theta) is checked with h = 1e-2 on the noise case
    (the per-particle cotangents themselves are checked against a loss of
    the positions above)."""
    torch = pytest.importorskip("torch")
    from fipi_gb300 import gradcheck as G
    from fipi_gb300 import inputs

    w = fipi.workload("t32")
    rng = np.random.default_rng(65)
    if init == "droplet":
        P = w.params()
        P.rho1, P.rho2, P.gravity = 2.0, 1.0, -1e-2
        c0 = inputs.droplet_phase(P, 8.0)
        p0 = inputs.interface_particles(P, w.n_p, 8.0, 3)
        r = None

        def loss_fn(c):
            return G.area_plus_height(c, P)
    else:
        P, c0, p0, r, _ = seeded_state(w, 64)
        Pt, ct0, _, _, _ = seeded_state(w, 66)
        target = G.structure_factor(torch.from_numpy(ct0), (P.nz, P.ny, P.nx))

        def loss_fn(c):
            return G.structure_loss(c, target, (P.nz, P.ny, P.nx))
    ct = rng.uniform(-0.5, 0.5, w.n_p)
    start = G.InitialState(p0=p0, r=r, cos_theta=ct)
    which = ("phi0", "mobility", "sigma") + (("cos_theta",) if init == "noise" else ())
    h = {"phi0": 1e-6, "mobility": 1e-6, "sigma": 1e-6, "cos_theta": 1e-2}
    with fipi.Simulation(P, "fp64") as s:
        res = G.fd_all(s, c0, start, 5, loss_fn, h, stride=2, seed=3, which=which)
    for k in which:
        assert res[k]["rel"] < 1e-3, (k, res[k])
