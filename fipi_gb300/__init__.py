"""FIPI on GB300: the per-step Eulerian/Lagrangian hot path of FIPI
(pseudo-spectral Cahn-Hilliard + Stokes + overdamped particles) as
hand-written sm_103a CUDA behind a C ABI (include/fipi.h).

Python is a thin ctypes front end used by the tests and the benchmark.
"""
from .params import FipiParams, Workload, WORKLOADS, workload, reference_head  # noqa: F401
from .lib import (  # noqa: F401
    FipiError,
    Simulation,
    cell_geometry,
    declared_symbols,
    fma_peak,
    load,
    reference_initial_state,
    reference_params,
    free_energy_density,
    seed_particles,
    seed_phase,
    vtk_write_field,
    vtk_write_particles,
)

__all__ = [
    "FipiParams", "Workload", "WORKLOADS", "workload", "reference_head", "FipiError",
    "Simulation", "cell_geometry", "declared_symbols", "fma_peak", "load", "reference_params",
    "reference_initial_state", "seed_particles", "seed_phase", "vtk_write_field", "vtk_write_particles", "free_energy_density",
]
