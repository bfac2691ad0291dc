"""Gradient-check harness for the FP64 adjoint.

The trajectory c0 -> c_T of the library (N steps with sqrt(N)
checkpointing on the device, reversed by the hand-written adjoint through
the C ABI) is wrapped as a ``torch.autograd.Function`` so that a loss written
in torch -- here the structure-factor mismatch ||S(k) - S_target(k)||^2 --
can be differentiated end to end.  Torch only computes the loss and its
gradient with respect to c_T; the step and its adjoint run in the library.
The harness checks the result against central finite differences of the
FP64 forward path.

The reference has no adjoint; the differentiated step is the loop body of
main.cpp:75-219 as the library computes it.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import torch

from .lib import Simulation


@dataclasses.dataclass
class InitialState:
    """Everything a trajectory starts from besides c0 (kept fixed)."""

    u0: np.ndarray | None = None   # 3 x V, None = 0
    p0: np.ndarray | None = None   # n_p x 3
    r: np.ndarray | None = None
    cos_theta: np.ndarray | None = None
    f_pp0: np.ndarray | None = None


def _start(sim: Simulation, c0: np.ndarray, init: InitialState):
    sim.set_phase(c0)
    sim.set_velocity(init.u0 if init.u0 is not None else np.zeros(3 * sim.V))
    if sim.n > 0:
        sim.set_particles(init.p0, init.r, init.cos_theta, init.f_pp0)


class PhaseTrajectory(torch.autograd.Function):
    """c0 (V, float64) -> c_T after `nsteps` FP64 steps of `sim`."""

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


def structure_factor(c: torch.Tensor, shape: tuple[int, int, int], nbins: int | None = None) -> torch.Tensor:
    """Shell-averaged S(k) = <|c_hat(k)|^2> / V over integer shells of |k| in
    index units (x fastest, like the library's real fields)."""
    nz, ny, nx = shape
    a = c.reshape(nz, ny, nx)
    F = torch.fft.fftn(a)
    P = (F.real ** 2 + F.imag ** 2) / a.numel()
    kz = torch.fft.fftfreq(nz, d=1.0 / nz, dtype=torch.float64)
    ky = torch.fft.fftfreq(ny, d=1.0 / ny, dtype=torch.float64)
    kx = torch.fft.fftfreq(nx, d=1.0 / nx, dtype=torch.float64)
    K = torch.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    shell = torch.round(K).long().ravel()
    nb = int(shell.max()) + 1 if nbins is None else nbins
    sums = torch.zeros(nb, dtype=P.dtype).index_add_(0, shell, P.ravel())
    cnt = torch.zeros(nb, dtype=P.dtype).index_add_(0, shell, torch.ones_like(P.ravel()))
    return sums / cnt.clamp(min=1)


def structure_loss(c: torch.Tensor, target: torch.Tensor, shape) -> torch.Tensor:
    return ((structure_factor(c, shape) - target) ** 2).sum()


def loss_and_grad(sim: Simulation, c0: np.ndarray, init: InitialState, nsteps: int, target: torch.Tensor,
                  stride: int = 0):
    """Loss and dLoss/dc0 through torch autograd and the library adjoint."""
    P = sim.params
    shape = (P.nz, P.ny, P.nx)
    x = torch.tensor(c0, dtype=torch.float64, requires_grad=True)
    cT = PhaseTrajectory.apply(x, sim, init, nsteps, stride)
    L = structure_loss(cT, target, shape)
    L.backward()
    return float(L.detach()), x.grad.numpy().copy()


def loss_only(sim: Simulation, c0: np.ndarray, init: InitialState, nsteps: int, target: torch.Tensor) -> float:
    P = sim.params
    _start(sim, c0, init)
    sim.step(nsteps)
    cT = torch.from_numpy(sim.get_phase())
    return float(structure_loss(cT, target, (P.nz, P.ny, P.nx)))


def fd_check(sim: Simulation, c0: np.ndarray, init: InitialState, nsteps: int, target: torch.Tensor,
             direction: np.ndarray, h: float, stride: int = 0) -> dict:
    """Directional derivative of the loss along `direction`: adjoint vs
    central difference (L(c0 + h d) - L(c0 - h d)) / 2h."""
    L0, g = loss_and_grad(sim, c0, init, nsteps, target, stride)
    ad = float(np.dot(g, direction))
    lp = loss_only(sim, c0 + h * direction, init, nsteps, target)
    lm = loss_only(sim, c0 - h * direction, init, nsteps, target)
    fd = (lp - lm) / (2 * h)
    return {"loss": L0, "adjoint": ad, "fd": fd, "rel": abs(ad - fd) / max(abs(fd), 1e-300), "grad": g}
