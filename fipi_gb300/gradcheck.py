"""Gradient-check harness for the FP64 adjoint.

The trajectory (c0, M, sigma, cos theta) -> c_T of the library (N steps
with sqrt(N) checkpointing on the device, reversed by the hand-written
adjoint through the C ABI) is wrapped as a ``torch.autograd.Function`` so
that a loss written in torch can be differentiated end to end with respect
to the initial phase field, the mobility, the surface tension (lambda =
3 sigma eps / (2 sqrt 2) and k_n = sigma / 2 following it, as head.hpp:47
and parameter.hpp:18 define them) and every particle's wettability.  Torch
only computes the loss and its gradient with respect to c_T; the step and
its adjoint run in the library.  The harness checks the result against
central finite differences of the FP64 forward path.

Losses: the structure-factor mismatch ||S(k) - S_target(k)||^2; the
interfacial area of the phase field, A = 3 eps / (2 sqrt 2) sum (|grad c|^2 / 2
+ (c^2 - 1)^2 / (4 eps^2)) dV, which equals the area of a flat equilibrium
tanh interface (the free energy divided by sigma); the centroid height of
the phase c > 0, z_c = sum z (1 + c)/2 / sum (1 + c)/2.

The reference has no adjoint; the differentiated step is the loop body of
main.cpp:75-219 as the library computes it.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np
import torch

from .lib import Simulation
from .params import FipiParams


@dataclasses.dataclass
class InitialState:
    """Everything a trajectory starts from besides c0 and cos theta."""

    u0: np.ndarray | None = None   # 3 x V, None = 0
    p0: np.ndarray | None = None   # n_p x 3
    r: np.ndarray | None = None
    cos_theta: np.ndarray | None = None
    f_pp0: np.ndarray | None = None


def with_physics(P: FipiParams, mobility: float | None = None, sigma: float | None = None) -> FipiParams:
    """A copy of P with a new mobility and/or surface tension; lambda and k_n
    follow sigma (head.hpp:47, parameter.hpp:18)."""
    Q = FipiParams.from_buffer_copy(P)
    if mobility is not None:
        Q.mobility = mobility
    if sigma is not None:
        Q.sigma = sigma
        Q.lambda_ = sigma * Q.epsilon * 3.0 / 2.0 / math.pow(2, 0.5)
        Q.k_n = 0.5 * sigma
    return Q


def _start(sim: Simulation, c0: np.ndarray, init: InitialState, cos_theta=None):
    sim.set_phase(c0)
    sim.set_velocity(init.u0 if init.u0 is not None else np.zeros(3 * sim.V))
    if sim.n > 0:
        ct = cos_theta if cos_theta is not None else init.cos_theta
        sim.set_particles(init.p0, init.r, ct, init.f_pp0)


class Trajectory(torch.autograd.Function):
    """(c0 (V), theta = [M, sigma], cos_theta (n_p)) -> c_T after `nsteps`
    FP64 steps of `sim`, every input differentiable."""

    @staticmethod
    def forward(ctx, c0: torch.Tensor, theta: torch.Tensor, cos_theta: torch.Tensor, sim: Simulation,
                init: InitialState, nsteps: int, stride: int = 0):
        base = sim.params
        sim.set_params(with_physics(base, float(theta[0]), float(theta[1])))
        ct = cos_theta.detach().cpu().numpy().astype(np.float64) if sim.n > 0 else None
        _start(sim, c0.detach().cpu().numpy().astype(np.float64), init, ct)
        sim.trajectory_forward(nsteps, stride)
        ctx.sim = sim
        return torch.from_numpy(sim.get_phase()).to(c0)

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        sim = ctx.sim
        sim.trajectory_backward(dc=g.detach().cpu().numpy().astype(np.float64))
        dc, _, _, _ = sim.adjoint_get()
        pg, dct = sim.adjoint_get_params()
        dtheta = torch.tensor([pg["mobility"], pg["sigma"]], dtype=torch.float64)
        return (torch.from_numpy(dc).to(g), dtheta, torch.from_numpy(dct).to(torch.float64), None, None, None,
                None)


class PhaseTrajectory(torch.autograd.Function):
    """c0 (V, float64) -> c_T after `nsteps` FP64 steps of `sim` (the
    parameters and wettabilities of `sim` / `init` held fixed)."""

    @staticmethod
    def forward(ctx, c0: torch.Tensor, sim: Simulation, init: InitialState, nsteps: int, stride: int = 0):
        _start(sim, c0.detach().cpu().numpy().astype(np.float64), init)
        sim.trajectory_forward(nsteps, stride)
        ctx.sim = sim
        return torch.from_numpy(sim.get_phase()).to(c0)

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        sim = ctx.sim
        sim.trajectory_backward(dc=g.detach().cpu().numpy().astype(np.float64))
        dc, _, _, _ = sim.adjoint_get()
        return torch.from_numpy(dc).to(g), None, None, None, None


# ---------------------------------------------------------------- losses
def structure_factor(c: torch.Tensor, shape: tuple[int, int, int], nbins: int | None = None) -> torch.Tensor:
    """Shell-averaged S(k) = <|c_hat(k)|^2> / V over integer shells of |k| in
    index units (x fastest, like the library's real fields)."""
    nz, ny, nx = shape
    a = c.reshape(nz, ny, nx)
    F = torch.fft.fftn(a)
    P = (F.real ** 2 + F.imag ** 2) / a.numel()
    kz = torch.fft.fftfreq(nz, d=1.0 / nz, dtype=torch.float64, device=c.device)
    ky = torch.fft.fftfreq(ny, d=1.0 / ny, dtype=torch.float64, device=c.device)
    kx = torch.fft.fftfreq(nx, d=1.0 / nx, dtype=torch.float64, device=c.device)
    K = torch.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    shell = torch.round(K).long().ravel()
    nb = int(shell.max()) + 1 if nbins is None else nbins
    sums = torch.zeros(nb, dtype=P.dtype, device=c.device).index_add_(0, shell, P.ravel())
    cnt = torch.zeros(nb, dtype=P.dtype, device=c.device).index_add_(0, shell, torch.ones_like(P.ravel()))
    return sums / cnt.clamp(min=1)


def structure_loss(c: torch.Tensor, target: torch.Tensor, shape) -> torch.Tensor:
    return ((structure_factor(c, shape) - target) ** 2).sum()


def spectral_grad(c: torch.Tensor, P: FipiParams) -> list[torch.Tensor]:
    """grad c with the library's wave numbers (k = 2 pi q / L with the
    reference's pi, Nyquist index zeroed as field::grad does)."""
    nz, ny, nx = P.nz, P.ny, P.nx
    a = c.reshape(nz, ny, nx)
    F = torch.fft.rfftn(a)
    out = []
    for n, L, axis in ((nx, P.lx, 2), (ny, P.ly, 1), (nz, P.lz, 0)):
        q = torch.fft.rfftfreq(n, d=1.0 / n) if axis == 2 else torch.fft.fftfreq(n, d=1.0 / n)
        q = q.to(dtype=torch.float64, device=c.device)
        k = q * (2.0 * P.pi / L)
        k = torch.where(q.abs() == n // 2, torch.zeros_like(k), k)
        shp = [1, 1, 1]
        shp[axis] = -1
        out.append(torch.fft.irfftn(F * (1j * k.reshape(shp)), s=(nz, ny, nx)).ravel())
    return out


def interfacial_area(c: torch.Tensor, P: FipiParams) -> torch.Tensor:
    dv = P.lx * P.ly * P.lz / (P.nx * P.ny * P.nz)
    g = spectral_grad(c, P)
    e = P.epsilon
    dens = 0.5 * (g[0] ** 2 + g[1] ** 2 + g[2] ** 2) + (c * c - 1.0) ** 2 / (4.0 * e * e)
    return 3.0 * e / (2.0 * math.sqrt(2.0)) * dens.sum() * dv


def centroid_height(c: torch.Tensor, P: FipiParams) -> torch.Tensor:
    nz, ny, nx = P.nz, P.ny, P.nx
    z = torch.arange(nz, dtype=torch.float64, device=c.device) * (P.lz / nz)
    w = (1.0 + c.reshape(nz, ny, nx)) * 0.5
    return (w.sum(dim=(1, 2)) * z).sum() / w.sum()


def area_plus_height(c: torch.Tensor, P: FipiParams) -> torch.Tensor:
    return interfacial_area(c, P) + centroid_height(c, P)


# ---------------------------------------------------------------- checks
def loss_and_grads(sim: Simulation, c0: np.ndarray, init: InitialState, nsteps: int, loss_fn, stride: int = 0,
                   device: str = "cpu"):
    """Loss and its gradients with respect to c0, (M, sigma) and cos theta
    through torch autograd and the library adjoint.  `loss_fn(c_T)`."""
    P = sim.params
    n = sim.n
    x = torch.tensor(c0, dtype=torch.float64, requires_grad=True)
    th = torch.tensor([P.mobility, P.sigma], dtype=torch.float64, requires_grad=True)
    ct0 = init.cos_theta if init.cos_theta is not None else np.zeros(n)
    ct = torch.tensor(ct0, dtype=torch.float64, requires_grad=True)
    cT = Trajectory.apply(x, th, ct, sim, init, nsteps, stride)
    L = loss_fn(cT.to(device))
    L.backward()
    sim.set_params(P)
    return float(L.detach()), x.grad.numpy().copy(), th.grad.numpy().copy(), ct.grad.numpy().copy()


def loss_only(sim: Simulation, c0: np.ndarray, init: InitialState, nsteps: int, loss_fn, P: FipiParams | None = None,
              cos_theta=None, device: str = "cpu") -> float:
    base = sim.params
    if P is not None:
        sim.set_params(P)
    _start(sim, c0, init, cos_theta)
    sim.step(nsteps)
    cT = torch.from_numpy(sim.get_phase()).to(device)
    val = float(loss_fn(cT))
    sim.set_params(base)
    return val


def fd_check(sim: Simulation, c0: np.ndarray, init: InitialState, nsteps: int, target: torch.Tensor,
             direction: np.ndarray, h: float, stride: int = 0) -> dict:
    """Directional derivative of the structure-factor loss along `direction`
    in c0: adjoint vs central difference (L(c0 + h d) - L(c0 - h d)) / 2h."""
    P = sim.params
    shape = (P.nz, P.ny, P.nx)

    def loss_fn(c):
        return structure_loss(c, target, shape)

    L0, g, _, _ = loss_and_grads(sim, c0, init, nsteps, loss_fn, stride)
    ad = float(np.dot(g, direction))
    lp = loss_only(sim, c0 + h * direction, init, nsteps, loss_fn)
    lm = loss_only(sim, c0 - h * direction, init, nsteps, loss_fn)
    fd = (lp - lm) / (2 * h)
    return {"loss": L0, "adjoint": ad, "fd": fd, "rel": abs(ad - fd) / max(abs(fd), 1e-300), "grad": g}


def fd_all(sim: Simulation, c0: np.ndarray, init: InitialState, nsteps: int, loss_fn, h, stride: int = 0,
           seed: int = 0, device: str = "cpu", which=("phi0", "mobility", "sigma", "cos_theta"),
           grads=None) -> dict:
    """Adjoint gradients of `loss_fn` against central differences with
    relative step h (a number, or a dict per gradient): along a random
    direction in c0 and in cos theta, and in M and sigma.  `grads`: the
    result of loss_and_grads for the same trajectory, if already known."""
    P = sim.params
    L0, g_c, g_th, g_ct = grads if grads is not None else loss_and_grads(sim, c0, init, nsteps, loss_fn, stride,
                                                                          device)
    rng = np.random.default_rng(seed)
    ct0 = init.cos_theta if init.cos_theta is not None else np.zeros(sim.n)
    out = {"loss": L0}
    for what in which:
        h_w = h[what] if isinstance(h, dict) else h
        if what == "phi0":
            d = rng.standard_normal(c0.size)
            ad, hh = float(np.dot(g_c, d)), h_w
            lp = loss_only(sim, c0 + hh * d, init, nsteps, loss_fn, device=device)
            lm = loss_only(sim, c0 - hh * d, init, nsteps, loss_fn, device=device)
        elif what == "cos_theta":
            d = rng.standard_normal(sim.n)
            ad, hh = float(np.dot(g_ct, d)), h_w
            lp = loss_only(sim, c0, init, nsteps, loss_fn, cos_theta=ct0 + hh * d, device=device)
            lm = loss_only(sim, c0, init, nsteps, loss_fn, cos_theta=ct0 - hh * d, device=device)
        else:
            i = 0 if what == "mobility" else 1
            base = P.mobility if i == 0 else P.sigma
            ad, hh = float(g_th[i]), h_w * base
            kw = "mobility" if i == 0 else "sigma"
            lp = loss_only(sim, c0, init, nsteps, loss_fn, P=with_physics(P, **{kw: base + hh}), device=device)
            lm = loss_only(sim, c0, init, nsteps, loss_fn, P=with_physics(P, **{kw: base - hh}), device=device)
        fd = (lp - lm) / (2 * hh)
        out[what] = {"adjoint": ad, "fd": fd, "rel": abs(ad - fd) / max(abs(fd), 1e-300), "h": hh}
    return out
