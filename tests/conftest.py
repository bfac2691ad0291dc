import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU case")


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def seeded_state(w, seed=1):
    """Seeded initial state of a workload (phase field + particles)."""
    import fipi_gb300 as F

    P = w.params()
    c = F.seed_phase(P, seed, w.phi_mean, w.phi_amp)
    p = r = ct = None
    if w.n_p > 0:
        p, r, ct = F.seed_particles(P, seed + 1000, w.radius_range, w.theta_range_deg,
                                    allow_overlap=w.radius_range is not None)
        if w.radius_range is None:
            r = None
        if w.theta_range_deg is None:
            ct = None
    return P, c, p, r, ct


@pytest.fixture(scope="session")
def fipi():
    import fipi_gb300 as F

    F.load()
    return F


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O

    O.build_port()
    return O
