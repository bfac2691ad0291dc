"""Host-side checks of the C ABI that need no GPU: the library loads and
exports every symbol the header declares, parameters are validated before
any device work, the seeded generators, the C++ header compiles, and the
replica aggregation of bench.py under a world-size-2 gloo group."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent


def header_functions():
    text = (REPO / "include" / "fipi.h").read_text()
    return sorted(set(re.findall(r"^(?:fipi_status|int|const char\*)\s+(fipi_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol(fipi):
    lib = fipi.load()
    names = header_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(fipi.declared_symbols())


def test_abi_version_and_reference_params(fipi):
    lib = fipi.load()
    assert lib.fipi_abi_version() == 1
    p = fipi.reference_params()
    assert (p.nx, p.ny, p.nz, p.n_p) == (64, 64, 64, 20000)
    assert p.pi == 3.1415926
    assert p.k_n == 0.5 * p.sigma and p.r_eq == 5 * p.r_p


def test_cell_geometry_matches_oracle(fipi, oracle_mod):
    for name in ["t16", "t32", "t32_aniso", "t32_2pi", "cfg1_64", "cfg2_256", "cfg3_512"]:
        P = fipi.workload(name).params()
        a = fipi.cell_geometry(P)
        b = oracle_mod.cell_geometry(P)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    nc, dc = fipi.cell_geometry(fipi.workload("cfg2_256").params())
    assert list(nc) == [12, 12, 12] and abs(dc[0] - (16 / 12 + 20)) < 1e-12


@pytest.mark.parametrize("field,value,code", [
    ("nx", 48, 8), ("nx", 1024, 8), ("ny", 4, 8), ("dt", 0.0, 1), ("switch_ns", 0, 8),
    ("r_p", 20.0, 8),
])
def test_create_validates_before_device(fipi, field, value, code):
    lib = fipi.load()
    P = fipi.workload("t32").params()
    setattr(P, field, value)
    if field == "r_p":
        P.r_c = 5 * value
    h = ctypes.c_void_p()
    st = lib.fipi_create(ctypes.byref(P), 0, 0, ctypes.byref(h))
    assert st == code, lib.fipi_last_error_string()
    assert not h.value


def test_create_without_device_reports_no_device(fipi):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    with pytest.raises(fipi.FipiError) as e:
        fipi.Simulation(fipi.workload("t32").params())
    assert e.value.code == 6


def test_seeded_generators(fipi):
    w = fipi.workload("cfg1_64")
    P = w.params()
    a = fipi.seed_phase(P, 3, 0.0, 0.05)
    b = fipi.seed_phase(P, 3, 0.0, 0.05)
    assert np.array_equal(a, b) and a.min() >= -0.05 and a.max() <= 0.05
    assert not np.array_equal(a, fipi.seed_phase(P, 4, 0.0, 0.05))
    p, r, ct = fipi.seed_particles(P, 5)
    p = p.reshape(-1, 3)
    L = np.array([w.lx, w.ly, w.lz])
    assert (p >= 0).all() and (p < L).all()
    d = p[:, None, :] - p[None, :, :]
    d -= L * np.round(d / L)
    dist = np.sqrt((d ** 2).sum(-1)) + np.eye(len(p)) * 1e9
    assert dist.min() >= 2 * w.r_p  # periodic non-overlap
    assert np.all(ct == 0.0)
    p2, r2, ct2 = fipi.seed_particles(P, 5, (3.0, 6.0), (60.0, 120.0), allow_overlap=True)
    assert r2.min() >= 3.0 and r2.max() <= 6.0
    assert ct2.min() >= np.cos(np.radians(120)) - 1e-12 and ct2.max() <= 0.5 + 1e-12


@pytest.mark.parametrize("name", ["t32", "cfg1_64", "cfg2_256", "cfg3_512", "t32_aniso"])
def test_oracle_seeding_equals_library(fipi, oracle_mod, name):
    """The CPU baselines draw their inputs with the oracle's restatement of
    the seeded generators (no library load); it must give the library's
    draws bit for bit, including the rejection sampling of the
    non-overlapping placement and the radius / contact-angle draws."""
    w = fipi.workload(name)
    P = w.params()
    if name == "cfg3_512":
        P.nx = P.ny = P.nz = 8  # the particle draws use only the box; keep the phase field small
    a = fipi.seed_phase(P, 17, w.phi_mean, w.phi_amp)
    b = oracle_mod.seed_phase(P, 17, w.phi_mean, w.phi_amp)
    assert np.array_equal(a, b)
    ov = w.radius_range is not None
    pa, ra, ca = fipi.seed_particles(P, 1017, w.radius_range, w.theta_range_deg, allow_overlap=ov)
    pb, rb, cb = oracle_mod.seed_particles(P, 1017, w.radius_range, w.theta_range_deg, allow_overlap=ov)
    assert np.array_equal(pa, pb) and np.array_equal(ra, rb) and np.array_equal(ca, cb)


def test_cpp_header_compiles(tmp_path):
    src = tmp_path / "use_fipi.cpp"
    src.write_text("""
#include "fipi.hpp"
int main() {
    fipi_params p = fipi::reference_params();
    p.nx = p.ny = p.nz = 32;
    try { fipi::simulation s(p, FIPI_MIXED); s.step(1); (void)s.mass(); }
    catch (const fipi::error& e) { return e.code == FIPI_ERR_NO_DEVICE ? 0 : 1; }
    return 0;
}
""")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-I", str(REPO / "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _replica_worker(rank, ws, port, q):
    import os

    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench

    elapsed = 1.0 + rank  # rank 1 is the slow one
    value, t = bench.aggregate_replicas(elapsed, steps=10, ws=ws, dist=dist, device="cpu")
    q.put((rank, value, t))
    dist.destroy_process_group()


def test_replica_aggregation_gloo_world_size_2():
    import socket
    import sys

    import torch.multiprocessing as mp

    sys.path.insert(0, str(REPO))
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    for rank, value, t in res:
        assert t == 2.0            # max over ranks
        assert value == 2 * 10 / 2.0  # all ranks' steps / slowest time
