"""Device-pointer state I/O (zero host copies) against the host calls.

The same values set through device memory (torch CUDA tensors) and through
host memory give the same state: bit for bit in the plain FP64 form; in the
mixed form the FP64 k = 0 record of a new phase field is summed on the device
in another order, so the phase agrees to rounding of that sum.
"""
import numpy as np
import pytest

from conftest import rel_l2, seeded_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_device_io_matches_host(fipi, prec):
    torch = pytest.importorskip("torch")
    w = fipi.workload("t32")
    P, c, p, r, ct = seeded_state(w, 51)
    rng = np.random.default_rng(5)
    u = 1e-3 * rng.standard_normal(3 * w.V)
    fpp = 0.1 * rng.standard_normal(3 * w.n_p)
    rr = r if r is not None else np.full(w.n_p, P.r_p)
    cc = ct if ct is not None else np.zeros(w.n_p)
    dev = torch.device("cuda:0")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(dev)
    res = {}
    for mode in ("host", "device"):
        with fipi.Simulation(P, prec) as s:
            if mode == "host":
                s.set_phase(c)
                s.set_velocity(u)
                s.set_particles(p, rr, cc, fpp)
            else:
                s.set_phase_device(T(c))
                s.set_velocity_device(T(u))
                s.set_particles_device(T(p), T(rr), T(cc), T(fpp))
            s.step(2)
            if mode == "host":
                pp, pf, pi = s.get_particles()
                res[mode] = (s.get_phase(), s.get_velocity(), pp, pf, pi)
            else:
                oc, ou = torch.empty(w.V, dtype=torch.float64, device=dev), torch.empty(3 * w.V, dtype=torch.float64, device=dev)
                op, of, oi = (torch.empty(3 * w.n_p, dtype=torch.float64, device=dev) for _ in range(3))
                s.get_phase_device(oc)
                s.get_velocity_device(ou)
                s.get_particles_device(op, of, oi)
                res[mode] = tuple(x.cpu().numpy() for x in (oc, ou, op, of, oi))
                # partial outputs: NULL pointers are skipped
                op2 = torch.empty(3 * w.n_p, dtype=torch.float64, device=dev)
                s.get_particles_device(p=op2)
                assert np.array_equal(op2.cpu().numpy(), res[mode][2])
    h, d = res["host"], res["device"]
    if prec == "fp64":
        for a, b in zip(h, d):
            assert np.array_equal(a, b)
    else:
        assert rel_l2(d[0], h[0]) < 1e-12
        assert rel_l2(d[1], h[1]) < 1e-9
        assert np.abs(d[2] - h[2]).max() < 1e-9


def test_device_io_rejects_wrong_arrays(fipi):
    torch = pytest.importorskip("torch")
    w = fipi.workload("t16")
    P, c, p, r, ct = seeded_state(w, 52)
    with fipi.Simulation(P, "fp64") as s:
        with pytest.raises(TypeError):
            s.set_phase_device(torch.zeros(w.V, dtype=torch.float32, device="cuda:0"))
        with pytest.raises(ValueError):
            s.set_phase_device(torch.zeros(w.V + 1, dtype=torch.float64, device="cuda:0"))
