"""Run-time parameters of the FIPI step and the named workloads.

`FipiParams` mirrors `fipi_params` of include/fipi.h, which replaces the
reference's compile-time constants (head.hpp:27-74, parameter.hpp:18-20).
The named workloads are the seeded synthetic cases the library is measured
and tested on: the 64^3 / 256^3 / 512^3 / 128^3 cases of the benchmark plan
and a few small grids that the CPU oracle finishes in seconds.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field, replace

REF_PI = 3.1415926  # head.hpp:27


class FipiParams(ctypes.Structure):
    """ctypes image of `struct fipi_params` (include/fipi.h)."""

    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("lz", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("t_end", ctypes.c_int),
        ("pi", ctypes.c_double),
        ("sigma", ctypes.c_double), ("epsilon", ctypes.c_double),
        ("lambda_", ctypes.c_double), ("mobility", ctypes.c_double),
        ("mu", ctypes.c_double),
        ("rho1", ctypes.c_double), ("rho2", ctypes.c_double),
        ("gravity", ctypes.c_double),
        ("A", ctypes.c_double), ("k_n", ctypes.c_double),
        ("margin", ctypes.c_double),
        ("r_p", ctypes.c_double), ("r_eq", ctypes.c_double), ("r_c", ctypes.c_double),
        ("n_p", ctypes.c_int),
        ("switch_particle", ctypes.c_int), ("switch_ch", ctypes.c_int),
        ("switch_ns", ctypes.c_int),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


@dataclass(frozen=True)
class Workload:
    """A named configuration plus how its initial state is drawn."""

    name: str
    nx: int
    ny: int
    nz: int
    lx: float
    ly: float
    lz: float
    n_p: int
    r_p: float
    dt: float = 1e-3
    t_end: int = 500
    steps: int = 500
    sigma: float = 1.0
    epsilon: float = 1.0
    mobility: float = 1.0
    mu: float = 1.0
    A: float = 2.0
    rho1: float = 1e-3
    rho2: float | None = None  # None: Bo = 0, rho2 = rho1 (head.hpp:53)
    gravity: float = -1e1
    phi_mean: float = 0.0
    phi_amp: float = 0.05
    radius_range: tuple | None = None    # polydisperse radii U[a, b]
    theta_range_deg: tuple | None = None  # contact angles U[a, b] degrees
    switches: tuple = (1, 1, 1)           # particle, ch, ns
    note: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def V(self) -> int:
        return self.nx * self.ny * self.nz

    def params(self) -> FipiParams:
        p = FipiParams()
        p.nx, p.ny, p.nz = self.nx, self.ny, self.nz
        p.lx, p.ly, p.lz = self.lx, self.ly, self.lz
        p.dt = self.dt
        p.t_end = self.t_end
        p.pi = REF_PI
        p.sigma = self.sigma
        p.epsilon = self.epsilon
        # lambda = sigma*epsilon*3.0/2.0/pow(2,0.5)   (head.hpp:47)
        p.lambda_ = self.sigma * self.epsilon * 3.0 / 2.0 / math.pow(2, 0.5)
        p.mobility = self.mobility
        p.mu = self.mu
        p.rho1 = self.rho1
        p.rho2 = self.rho1 if self.rho2 is None else self.rho2
        p.gravity = self.gravity
        p.A = self.A
        p.k_n = 0.5 * self.sigma  # parameter.hpp:18
        p.margin = 0.0            # parameter.hpp:20
        p.r_p = self.r_p
        p.r_eq = 5 * self.r_p     # head.hpp:64
        p.r_c = 5 * self.r_p      # head.hpp:65
        p.n_p = self.n_p
        p.switch_particle, p.switch_ch, p.switch_ns = self.switches
        return p

    def with_(self, **kw) -> "Workload":
        return replace(self, **kw)


def reference_head() -> Workload:
    """The values compiled into the reference's head.hpp (64^3, L = 2 pi)."""
    L = 2 * REF_PI
    eps = 3.0 * (L / 64) / math.pow(2, 0.5) / 2.0
    r_drop = 0.4 * L
    mu = 1e-3
    return Workload(
        name="reference_head", nx=64, ny=64, nz=64, lx=L, ly=L, lz=L,
        n_p=20000, r_p=0.03 * r_drop, dt=1e-3, t_end=20000, steps=20000,
        sigma=0.07, epsilon=eps, mobility=math.pow(0.2 * eps, 2) / mu, mu=mu,
        A=2.0, rho1=1e-3, gravity=-1e1, phi_mean=0.0, phi_amp=0.1,
        note="head.hpp:27-74 defaults")


WORKLOADS = {
    # Benchmark-plan workloads (seeded synthetic inputs).
    "cfg1_64": Workload("cfg1_64", 64, 64, 64, 64.0, 64.0, 64.0, n_p=256, r_p=4.0,
                        t_end=500, steps=500,
                        note="64^3 dx=1, 256 spheres r=4, 90 deg, 500 steps (CPU-runnable case)"),
    "cfg2_256": Workload("cfg2_256", 256, 256, 256, 256.0, 256.0, 256.0, n_p=20000, r_p=4.0,
                         t_end=1000, steps=1000,
                         note="256^3 dx=1, 20k spheres r=4 (~32% volume fraction), 90 deg, 1000 steps"),
    "cfg3_512": Workload("cfg3_512", 512, 512, 512, 512.0, 512.0, 512.0, n_p=200000, r_p=4.5,
                         dt=5e-4, t_end=2000, steps=2000, phi_mean=-0.4,
                         radius_range=(3.0, 6.0), theta_range_deg=(60.0, 120.0),
                         note="512^3, 200k spheres r~U[3,6] (contact range from mean r=4.5), "
                              "theta~U[60,120] deg, overlap allowed (63% is above RSA jamming)"),
    "cfg4_128": Workload("cfg4_128", 128, 128, 128, 128.0, 128.0, 128.0, n_p=2000, r_p=4.0,
                         t_end=200, steps=200,
                         note="128^3, 2000 spheres r=4, 200 steps (gradient-check case)"),
    "cfg5_256": Workload("cfg5_256", 256, 256, 256, 256.0, 256.0, 256.0, n_p=20000, r_p=3.0,
                         t_end=1000, steps=1000, rho1=2.0, rho2=1.0, gravity=-1e-4,
                         extra={"init": "droplet", "radius": 64.0},
                         note="256^3, one droplet of radius 64 (phi = +1 inside, tanh profile of width eps), "
                              "20,000 spheres r=3 on its interface (overlap allowed: a monolayer holds ~1650), "
                              "g = 1e-4 along -z with rho1 = 2 inside and rho2 = 1 outside, 1000 steps"),
    # Small grids the CPU oracle finishes in seconds (parity cases).
    "t16": Workload("t16", 16, 16, 16, 16.0, 16.0, 16.0, n_p=6, r_p=1.0, t_end=20, steps=4,
                    note="16^3 parity case"),
    "t32": Workload("t32", 32, 32, 32, 32.0, 32.0, 32.0, n_p=40, r_p=1.2, t_end=10, steps=3,
                    note="32^3 parity case with contact forces active from the first step"),
    "t32_aniso": Workload("t32_aniso", 32, 16, 8, 32.0, 16.0, 8.0, n_p=20, r_p=0.5,
                          t_end=10, steps=3, note="anisotropic 32x16x8 grid"),
    "t32_bo": Workload("t32_bo", 32, 32, 32, 32.0, 32.0, 32.0, n_p=40, r_p=1.2, t_end=10, steps=3,
                       rho2=5e-2, note="32^3 with a density contrast (rho2 != rho1: the buoyancy "
                                       "is not a constant the projection removes)"),
    "t256x": Workload("t256x", 256, 16, 16, 256.0, 16.0, 16.0, n_p=24, r_p=1.0, t_end=10, steps=3,
                      note="256x16x16: rows of 128 complex pairs along x"),
    "t512x": Workload("t512x", 512, 16, 16, 512.0, 16.0, 16.0, n_p=40, r_p=1.0, t_end=10, steps=2,
                      note="512x16x16: rows of 256 complex pairs along x"),
    "t256yz": Workload("t256yz", 16, 256, 256, 16.0, 256.0, 256.0, n_p=400, r_p=1.0, t_end=10, steps=3,
                       note="16x256x256: the 256-point y and z transforms of the 256^3 workload"),
    "t512yz": Workload("t512yz", 16, 512, 512, 16.0, 512.0, 512.0, n_p=800, r_p=1.0, t_end=10, steps=2,
                       note="16x512x512: the 512-point y and z transforms of the 512^3 workload"),
    "t32_2pi": Workload("t32_2pi", 32, 32, 32, 2 * REF_PI, 2 * REF_PI, 2 * REF_PI, n_p=30,
                        r_p=0.06, sigma=0.07, epsilon=0.15, mobility=0.02, mu=1e-3,
                        t_end=10, steps=3, phi_amp=0.1,
                        note="32^3 in a 2*pi box (dx != 1), reference-like constants"),
}


def workload(name: str) -> Workload:
    if name == "reference_head":
        return reference_head()
    return WORKLOADS[name]
