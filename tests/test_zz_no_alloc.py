"""fipi_cells_build_noalloc: the cell-list build for callers that cannot
allocate device memory (a host framework that owns a fixed device pool, a
real-time loop that forbids driver allocations).  It takes the caller's
device buffers, keeps its scratch in a fixed array inside the library and
must give exactly what the context-based fipi_cells_build gives.

Two calls in a row (a large then a small particle set) check that the
shared scratch, which keeps the previous call's contents, does not leak
into the next result.  This file sorts last so that a stop-at-first-failure
run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import seeded_state

pytestmark = pytest.mark.gpu


def _call(lib, P, d_pos, d_keys, d_sorted, d_off, stream):
    return lib.fipi_cells_build_noalloc(ctypes.byref(P), d_pos.data_ptr(), d_keys.data_ptr(),
                                        d_sorted.data_ptr(), d_off.data_ptr(), stream)


def test_noalloc_cells_match_context_entry_point(fipi):
    torch = pytest.importorskip("torch")
    lib = fipi.load()
    stream = torch.cuda.current_stream().cuda_stream
    for name, seed in (("cfg2_256", 41), ("cfg1_64", 42)):
        w = fipi.workload(name)
        P, c, p, r, ct = seeded_state(w, seed)
        with fipi.Simulation(P, "fp64") as s:
            keys, srt, off = s.cells_build(p)
        n = w.n_p
        d_pos = torch.tensor(p, dtype=torch.float64, device="cuda")
        d_keys = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_sorted = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_off = torch.full((off.size,), -7, dtype=torch.int32, device="cuda")
        st = _call(lib, P, d_pos, d_keys, d_sorted, d_off, stream)
        assert st == 0, lib.fipi_last_error_string()
        assert np.array_equal(d_keys.cpu().numpy(), keys), name
        assert np.array_equal(d_sorted.cpu().numpy(), srt), name
        assert np.array_equal(d_off.cpu().numpy(), off), name


def test_noalloc_cells_at_the_scratch_bound(fipi):
    """Exactly FIPI_NOALLOC_MAX_PARTICLES particles: every histogram block
    and the whole position region of the scratch in use."""
    torch = pytest.importorskip("torch")
    lib = fipi.load()
    stream = torch.cuda.current_stream().cuda_stream
    w = fipi.workload("cfg1_64")
    P = w.params()
    n = P.n_p = 65536
    rng = np.random.default_rng(n)
    p = (rng.random((n, 3)) * np.array([P.lx, P.ly, P.lz])).ravel()
    with fipi.Simulation(P, "fp64") as s:
        keys, srt, off = s.cells_build(p)
    d_pos = torch.tensor(p, dtype=torch.float64, device="cuda")
    d_keys = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    d_sorted = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    d_off = torch.full((off.size,), -7, dtype=torch.int32, device="cuda")
    for _ in range(2):
        st = _call(lib, P, d_pos, d_keys, d_sorted, d_off, stream)
        assert st == 0, lib.fipi_last_error_string()
        assert np.array_equal(d_keys.cpu().numpy(), keys)
        assert np.array_equal(d_sorted.cpu().numpy(), srt)
        assert np.array_equal(d_off.cpu().numpy(), off)


def test_noalloc_rejects_sizes_beyond_its_scratch(fipi):
    torch = pytest.importorskip("torch")
    lib = fipi.load()
    w = fipi.workload("cfg1_64")
    P = w.params()
    P.n_p = 65536 + 1
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    ib = torch.zeros(8, dtype=torch.int32, device="cuda")
    st = _call(lib, P, buf, ib, ib, ib, torch.cuda.current_stream().cuda_stream)
    assert st == 8  # FIPI_ERR_UNSUPPORTED
    assert b"exceeds" in lib.fipi_last_error_string()
