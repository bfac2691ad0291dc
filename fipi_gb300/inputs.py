"""Initial states of the benchmark workloads that are not i.i.d. draws.

The droplet workload (256^3, one droplet of radius 64 whose interface is
coated by spheres) starts from the phase field the reference's commented
droplet initialiser sketches (field.cpp:95 of the reference, which puts
phi = -1 inside; here phi = +1 inside) with the interface profile
tanh(d / (sqrt(2) eps)) that the attachment force's distance map assumes
(element.cpp:88: d = artanh(phi) sqrt(2) eps), and spheres placed uniformly
at random on the interface.  20,000 spheres of radius 3 do not fit on a
sphere of radius 64 as a monolayer (about 1650 do), so they are placed with
overlap allowed; the contact forces, ramped in over the first fifth of the
run (ramp(t, 0.2 t_end)), push them apart.
"""
from __future__ import annotations

import numpy as np

from .params import FipiParams, Workload


def droplet_phase(P: FipiParams, radius: float, center=None) -> np.ndarray:
    """phi = tanh((R - |x - x0|) / (sqrt(2) eps)) at the grid nodes (x fastest)."""
    x0 = np.array(center if center is not None else (P.lx / 2, P.ly / 2, P.lz / 2))
    z = np.arange(P.nz) * (P.lz / P.nz)
    y = np.arange(P.ny) * (P.ly / P.ny)
    x = np.arange(P.nx) * (P.lx / P.nx)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    d = np.sqrt((X - x0[0]) ** 2 + (Y - x0[1]) ** 2 + (Z - x0[2]) ** 2)
    return np.tanh((radius - d) / (np.sqrt(2.0) * P.epsilon)).ravel()


def interface_particles(P: FipiParams, n: int, radius: float, seed: int, center=None) -> np.ndarray:
    """n points uniform on the sphere |x - x0| = radius (n x 3, flattened),
    wrapped into [0, L)."""
    x0 = np.array(center if center is not None else (P.lx / 2, P.ly / 2, P.lz / 2))
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    p = x0 + radius * v
    L = np.array([P.lx, P.ly, P.lz])
    p = np.mod(p, L)
    p[p >= L] = 0.0
    return p.ravel()


def initial_state(w: Workload, seed: int):
    """(P, c0, positions, radii or None, cos theta or None) of a workload
    with a special initial state (extra["init"]); None for the others."""
    init = w.extra.get("init")
    if init != "droplet":
        return None
    P = w.params()
    R = float(w.extra["radius"])
    return P, droplet_phase(P, R), interface_particles(P, w.n_p, R, seed), None, None
