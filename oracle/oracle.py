"""TEST INFRASTRUCTURE ONLY (oracle).

ctypes front end of the two CPU oracles:
  * `Port`: the plain-C restatement (oracle/fipi_oracle.c), built into
    oracle/_build/liboracle.so by `build_port()` on any host;
  * `Ref`: the reference's own sources compiled in place by
    oracle/ref/build_ref.py into oracle/_ref/ (only where they exist).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module.
"""
from __future__ import annotations

import ctypes
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
BUILD = HERE / "_build"
PORT_LIB = BUILD / "liboracle.so"
sys.path.insert(0, str(REPO))

from fipi_gb300.params import FipiParams, workload  # noqa: E402

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


def build_port(force: bool = False) -> Path:
    srcs = [HERE / "fipi_oracle.c", HERE / "fft_c2c.c"]
    hdrs = [HERE / "fipi_oracle.h", HERE / "fft_c2c.h", REPO / "include" / "fipi.h"]
    if PORT_LIB.exists() and not force:
        newest = max(p.stat().st_mtime for p in srcs + hdrs)
        if PORT_LIB.stat().st_mtime >= newest:
            return PORT_LIB
    BUILD.mkdir(exist_ok=True)
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall",
           "-o", str(PORT_LIB), *map(str, srcs), "-lm"]
    subprocess.run(cmd, check=True)
    return PORT_LIB


_port_lib = None


def port_lib():
    global _port_lib
    if _port_lib is None:
        lib = ctypes.CDLL(str(build_port()))
        P = ctypes.POINTER(FipiParams)
        lib.oracle_create.restype = ctypes.c_void_p
        lib.oracle_create.argtypes = [P]
        lib.oracle_destroy.argtypes = [ctypes.c_void_p]
        lib.oracle_set_threads.argtypes = [ctypes.c_int]
        for fn in ("oracle_set_phase", "oracle_set_velocity"):
            getattr(lib, fn).argtypes = [ctypes.c_void_p, _dp]
        lib.oracle_set_particles.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp]
        for fn in ("oracle_get_phase", "oracle_get_phase_imag", "oracle_get_velocity",
                   "oracle_get_grad"):
            getattr(lib, fn).argtypes = [ctypes.c_void_p, _dp]
        lib.oracle_get_particles.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        lib.oracle_tau.restype = ctypes.c_double
        lib.oracle_tau.argtypes = [ctypes.c_void_p]
        lib.oracle_step.argtypes = [ctypes.c_void_p]
        lib.oracle_free_energy.restype = ctypes.c_double
        lib.oracle_free_energy.argtypes = [ctypes.c_void_p]
        lib.oracle_mass.restype = ctypes.c_double
        lib.oracle_mass.argtypes = [ctypes.c_void_p]
        lib.oracle_set_extensions.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_ulonglong]
        lib.oracle_set_mass_conserving.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.oracle_philox4x32.argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.c_uint, ctypes.c_uint,
                                          ctypes.POINTER(ctypes.c_uint)]
        lib.oracle_brownian_normals.argtypes = [ctypes.c_ulonglong, ctypes.c_uint, ctypes.c_uint, ctypes.c_double,
                                                _dp]
        lib.oracle_fft3.argtypes = [P, _dp, ctypes.c_int]
        lib.oracle_grad.argtypes = [P, _dp, _dp]
        lib.oracle_div.argtypes = [P, _dp, _dp]
        lib.oracle_interpolate2.argtypes = [P, _dp, ctypes.c_int, _dp, _dp]
        lib.oracle_sorting.argtypes = [P, ctypes.c_int, _dp, _ip, _ip, _ip, _ip]
        lib.oracle_f_pp.argtypes = [P, ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, _dp, _ip,
                                    ctypes.c_int, _ip]
        lib.oracle_interpolate.argtypes = [P, _dp, ctypes.c_int, _dp, _dp]
        lib.oracle_f_pi.argtypes = [P, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
        lib.oracle_advect.argtypes = [P, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        lib.oracle_enforce_bc.argtypes = [P, ctypes.c_int, _dp]
        lib.oracle_spread.argtypes = [P, ctypes.c_int, _dp, _dp, _dp]
        lib.oracle_cell_geometry.argtypes = [P, _ip, _dp]
        lib.oracle_reference_initial_state.argtypes = [P, ctypes.c_uint, _dp, _dp, ctypes.c_long]
        lib.oracle_params_ok.argtypes = [P]
        lib.oracle_seed_phase.argtypes = [P, ctypes.c_ulonglong, ctypes.c_double, ctypes.c_double, _dp]
        lib.oracle_seed_particles.argtypes = [P, ctypes.c_ulonglong, ctypes.c_double, ctypes.c_double,
                                              ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp]
        _port_lib = lib
    return _port_lib


def cell_geometry(params: FipiParams):
    nc = np.zeros(3, np.int32)
    dc = np.zeros(3)
    port_lib().oracle_cell_geometry(ctypes.byref(params), _i(nc), _d(dc))
    return nc, dc


class Port:
    """The C restatement of the reference step (one simulation)."""

    def __init__(self, params: FipiParams, threads: int = 1):
        self.lib = port_lib()
        self.P = params
        self.V = params.nx * params.ny * params.nz
        self.n = params.n_p
        self.lib.oracle_set_threads(threads)
        self.h = self.lib.oracle_create(ctypes.byref(params))
        if not self.h:
            raise ValueError("oracle rejected the parameters")

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    def set_state(self, c, p=None, r=None, cos_theta=None, u=None, f_pp=None):
        c = np.ascontiguousarray(c, np.float64).ravel()
        self.lib.oracle_set_phase(self.h, _d(c))
        if u is not None:
            u = np.ascontiguousarray(u, np.float64).ravel()
            self.lib.oracle_set_velocity(self.h, _d(u))
        if self.n > 0 and p is not None:
            arrs = [None if a is None else np.ascontiguousarray(a, np.float64).ravel()
                    for a in (p, r, cos_theta, f_pp)]
            self.lib.oracle_set_particles(self.h, *[_d(a) for a in arrs])

    def set_extensions(self, couple: bool = False, kt: float = 0.0, seed: int = 0):
        self.lib.oracle_set_extensions(self.h, 1 if couple else 0, kt, seed)

    def set_mass_conserving(self, on: bool = True):
        self.lib.oracle_set_mass_conserving(self.h, 1 if on else 0)

    def step(self, n: int = 1):
        for _ in range(n):
            st = self.lib.oracle_step(self.h)
            if st != 0:
                return st
        return 0

    def phase(self):
        out = np.empty(self.V)
        self.lib.oracle_get_phase(self.h, _d(out))
        return out

    def phase_imag(self):
        out = np.empty(self.V)
        self.lib.oracle_get_phase_imag(self.h, _d(out))
        return out

    def velocity(self):
        out = np.empty(3 * self.V)
        self.lib.oracle_get_velocity(self.h, _d(out))
        return out

    def grad(self):
        out = np.empty(3 * self.V)
        self.lib.oracle_get_grad(self.h, _d(out))
        return out

    def particles(self):
        n = max(self.n, 0)
        p, fpp, fpi = np.empty(3 * n), np.empty(3 * n), np.empty(3 * n)
        if n:
            self.lib.oracle_get_particles(self.h, _d(p), _d(fpp), _d(fpi))
        return p, fpp, fpi

    def tau(self):
        return self.lib.oracle_tau(self.h)

    def free_energy(self):
        return self.lib.oracle_free_energy(self.h)

    def mass(self):
        return self.lib.oracle_mass(self.h)


# ---------------------------------------------------------------- stateless
def fft3(params, data_complex, sign):
    a = np.ascontiguousarray(data_complex, np.complex128).copy()
    port_lib().oracle_fft3(ctypes.byref(params), a.ctypes.data_as(_dp), sign)
    return a


def grad(params, c):
    V = params.nx * params.ny * params.nz
    out = np.zeros(3 * V)
    port_lib().oracle_grad(ctypes.byref(params), _d(np.ascontiguousarray(c, np.float64)), _d(out))
    return out


def div(params, v):
    V = params.nx * params.ny * params.nz
    out = np.zeros(V)
    port_lib().oracle_div(ctypes.byref(params), _d(np.ascontiguousarray(v, np.float64).ravel()), _d(out))
    return out


def interpolate2(params, field, p):
    n = len(p) // 3
    out = np.zeros(n)
    port_lib().oracle_interpolate2(ctypes.byref(params), _d(np.ascontiguousarray(field, np.float64)), n,
                                   _d(np.ascontiguousarray(p, np.float64)), _d(out))
    return out


def philox4x32(ctr, key):
    """Philox-4x32-10 of a 4-word counter and a 2-word key (4 words out)."""
    c = (ctypes.c_uint * 4)(*ctr)
    out = (ctypes.c_uint * 4)()
    port_lib().oracle_philox4x32(c, key[0], key[1], out)
    return list(out)


def brownian_normals(seed: int, pid: int, t: int, pi: float):
    g = np.zeros(3)
    port_lib().oracle_brownian_normals(seed, pid, t, pi, _d(g))
    return g


def reference_initial_state(params, seed: int, max_candidates: int = 10**7):
    """The reference's seeded set-up draws (oracle restatement): c, positions."""
    V = params.nx * params.ny * params.nz
    c = np.zeros(V)
    pos = np.zeros(3 * max(params.n_p, 0))
    st = port_lib().oracle_reference_initial_state(ctypes.byref(params), seed, _d(c), _d(pos), max_candidates)
    return st, c, pos


def seed_phase(params, seed: int, mean: float = 0.0, amp: float = 0.05):
    """The library's fipi_seed_phase draws, restated (no library load)."""
    V = params.nx * params.ny * params.nz
    c = np.empty(V)
    port_lib().oracle_seed_phase(ctypes.byref(params), seed, mean, amp, _d(c))
    return c


def seed_particles(params, seed: int, r_range=None, theta_range_deg=None, allow_overlap: bool = False):
    """The library's fipi_seed_particles draws, restated (no library load)."""
    n = max(params.n_p, 0)
    pos, r, ct = np.empty(3 * n), np.empty(n), np.empty(n)
    rmin, rmax = r_range if r_range else (params.r_p, params.r_p)
    tmin, tmax = theta_range_deg if theta_range_deg else (90.0, 90.0)
    st = port_lib().oracle_seed_particles(ctypes.byref(params), seed, rmin, rmax, tmin, tmax,
                                          1 if allow_overlap else 0, _d(pos), _d(r), _d(ct))
    if st != 0:
        raise ValueError("random non-overlapping placement did not converge")
    return pos, r, ct


def seeded_state(w, seed: int):
    """Seeded initial state of a workload as the benchmark draws it
    (phase field from `seed`, particles from `seed + 1000`); r and cos_theta
    are None where the workload keeps the reference's single radius / 90
    degrees."""
    P = w.params()
    c = seed_phase(P, seed, w.phi_mean, w.phi_amp)
    p = r = ct = None
    if w.n_p > 0:
        p, r, ct = seed_particles(P, seed + 1000, w.radius_range, w.theta_range_deg,
                                  allow_overlap=w.radius_range is not None)
        if w.radius_range is None:
            r = None
        if w.theta_range_deg is None:
            ct = None
    return P, c, p, r, ct


def sorting(params, p):
    n = len(p) // 3
    nc, _ = cell_geometry(params)
    keys = np.zeros(n, np.int32)
    srt = np.zeros(n, np.int32)
    off = np.zeros(int(np.prod(nc)) + 1, np.int32)
    mark = np.array([-1], np.int32)
    st = port_lib().oracle_sorting(ctypes.byref(params), n, _d(np.ascontiguousarray(p)),
                                   _i(keys), _i(srt), _i(off), _i(mark))
    return st, keys, srt, off, int(mark[0])


def f_pp(params, p, t, f_pi=None, want_pairs=False):
    n = len(p) // 3
    out = np.zeros(3 * n)
    tau = np.zeros(1)
    npairs = np.zeros(1, np.int32)
    p = np.ascontiguousarray(p, np.float64)
    fpi = None if f_pi is None else np.ascontiguousarray(f_pi, np.float64)
    lib = port_lib()
    st = lib.oracle_f_pp(ctypes.byref(params), n, _d(p), t, _d(fpi), _d(out), _d(tau), None, 0,
                         _i(npairs))
    pairs = None
    if want_pairs:
        pairs = np.zeros(2 * max(int(npairs[0]), 1), np.int32)
        lib.oracle_f_pp(ctypes.byref(params), n, _d(p), t, _d(fpi), _d(out), _d(tau), _i(pairs),
                        int(npairs[0]), _i(npairs))
        pairs = pairs[: 2 * int(npairs[0])].reshape(-1, 2)
    return st, out, float(tau[0]), pairs


def interpolate(params, field, p):
    n = len(p) // 3
    out = np.zeros(n)
    port_lib().oracle_interpolate(ctypes.byref(params), _d(np.ascontiguousarray(field)), n,
                                  _d(np.ascontiguousarray(p)), _d(out))
    return out


def f_pi(params, c_loc, dcdx, r=None, cos_theta=None):
    n = len(c_loc)
    out = np.zeros(3 * n)
    port_lib().oracle_f_pi(ctypes.byref(params), n, _d(np.ascontiguousarray(c_loc)),
                           _d(np.ascontiguousarray(dcdx)),
                           None if r is None else _d(np.ascontiguousarray(r)),
                           None if cos_theta is None else _d(np.ascontiguousarray(cos_theta)),
                           _d(out))
    return out


def advect(params, stage, f_pi_, f_pp_, r, p, p_old, u_old):
    n = len(p) // 3
    p, p_old, u_old = (np.ascontiguousarray(a, np.float64).copy() for a in (p, p_old, u_old))
    lib = port_lib()
    lib.oracle_advect(ctypes.byref(params), n, stage, _d(np.ascontiguousarray(f_pi_)),
                      _d(np.ascontiguousarray(f_pp_)),
                      None if r is None else _d(np.ascontiguousarray(r)), _d(p), _d(p_old),
                      _d(u_old))
    lib.oracle_enforce_bc(ctypes.byref(params), n, _d(p))
    return p, p_old, u_old


def enforce_bc(params, p):
    """element::enforce_bc on n x 3 positions (a copy)."""
    q = np.ascontiguousarray(p, np.float64).ravel().copy()
    port_lib().oracle_enforce_bc(ctypes.byref(params), q.size // 3, _d(q))
    return q


def spread(params, p, f_pp_):
    n = len(p) // 3
    V = params.nx * params.ny * params.nz
    out = np.zeros(3 * V)
    port_lib().oracle_spread(ctypes.byref(params), n, _d(np.ascontiguousarray(p)),
                             _d(np.ascontiguousarray(f_pp_)), _d(out))
    return out


# ---------------------------------------------------------------- reference
class Ref:
    """The reference's own code (compiled in place for one workload)."""

    def __init__(self, name: str):
        sys.path.insert(0, str(HERE / "ref"))
        import build_ref  # noqa: E402

        self.lib = ctypes.CDLL(str(build_ref.build(name)))
        w = workload(name)
        self.P = w.params()
        self.V = w.V
        self.n = w.n_p
        L = self.lib
        L.ref_config.argtypes = [_dp]
        L.ref_init.argtypes = [_dp, _dp, _dp, _dp]
        for fn in ("ref_get_phase", "ref_get_phase_imag", "ref_get_velocity", "ref_get_grad"):
            getattr(L, fn).argtypes = [_dp]
        L.ref_get_particles.argtypes = [_dp, _dp, _dp]
        L.ref_tau.restype = ctypes.c_double
        L.ref_free_energy.restype = ctypes.c_double
        L.ref_fft.argtypes = [_dp, ctypes.c_int, ctypes.c_int]
        L.ref_grad.argtypes = [_dp, _dp]
        L.ref_sorting.argtypes = [_dp, _ip, _ip, _ip, _ip]
        L.ref_f_pp.argtypes = [_dp, ctypes.c_int, _dp, _dp, _dp]
        L.ref_interpolate.argtypes = [_dp, ctypes.c_int, _dp, _dp]
        L.ref_f_pi.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp]
        L.ref_advect.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_spread.argtypes = [_dp, _dp, _dp]
        L.ref_write_field.argtypes = [_dp, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p]
        L.ref_div.argtypes = [_dp, _dp]
        L.ref_interpolate2.argtypes = [_dp, ctypes.c_int, _dp, _dp]
        L.ref_write_free_energy.argtypes = [_dp, _dp, ctypes.c_char_p]
        L.ref_write_particles.argtypes = [_dp, _dp, _dp, ctypes.c_char_p]
        L.ref_initial_state.argtypes = [ctypes.c_uint, _dp, _dp]

    def initial_state(self, seed: int):
        """srand(seed); the phase field's draws; cluster::distribute."""
        c = np.zeros(self.V)
        pos = np.zeros(3 * max(self.n, 0))
        self.lib.ref_initial_state(seed, _d(c), _d(pos))
        return c, pos

    def div(self, v):
        out = np.zeros(self.V)
        self.lib.ref_div(_d(np.ascontiguousarray(v, np.float64).ravel()), _d(out))
        return out

    def interpolate2(self, field, p):
        n = len(p) // 3
        out = np.zeros(n)
        self.lib.ref_interpolate2(_d(np.ascontiguousarray(field, np.float64)), n,
                                  _d(np.ascontiguousarray(p, np.float64)), _d(out))
        return out

    def write_field(self, values, components, name, path):
        v = np.ascontiguousarray(values, np.float64).ravel()
        self.lib.ref_write_field(_d(v), components, name.encode(), str(path).encode())

    def write_free_energy(self, c, g, path):
        c = np.ascontiguousarray(c, np.float64).ravel()
        g = np.ascontiguousarray(g, np.float64).ravel()
        self.lib.ref_write_free_energy(_d(c), _d(g), str(path).encode())

    def write_particles(self, p, r, f_pp, path):
        p = np.ascontiguousarray(p, np.float64).ravel()
        r = None if r is None else np.ascontiguousarray(r, np.float64).ravel()
        f = np.ascontiguousarray(f_pp, np.float64).ravel()
        self.lib.ref_write_particles(_d(p), _d(r), _d(f), str(path).encode())

    def config(self):
        out = np.zeros(27)
        self.lib.ref_config(_d(out))
        return out

    def init(self, c, p=None, r=None, f_pp=None):
        c = np.ascontiguousarray(c, np.float64).ravel()
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64).ravel()
                for a in (p, r, f_pp)]
        return self.lib.ref_init(_d(c), *[_d(a) for a in arrs])

    def step(self, n=1):
        for _ in range(n):
            st = self.lib.ref_step()
            if st:
                return st
        return 0

    def phase(self):
        out = np.empty(self.V)
        self.lib.ref_get_phase(_d(out))
        return out

    def phase_imag(self):
        out = np.empty(self.V)
        self.lib.ref_get_phase_imag(_d(out))
        return out

    def velocity(self):
        out = np.empty(3 * self.V)
        self.lib.ref_get_velocity(_d(out))
        return out

    def grad(self):
        out = np.empty(3 * self.V)
        self.lib.ref_get_grad(_d(out))
        return out

    def particles(self):
        n = self.n
        p, fpp, fpi = np.empty(3 * n), np.empty(3 * n), np.empty(3 * n)
        if n:
            self.lib.ref_get_particles(_d(p), _d(fpp), _d(fpi))
        return p, fpp, fpi

    def tau(self):
        return self.lib.ref_tau()

    def free_energy(self):
        return self.lib.ref_free_energy()

    def fft(self, data_complex, sign, normalise=True):
        a = np.ascontiguousarray(data_complex, np.complex128).copy()
        self.lib.ref_fft(a.ctypes.data_as(_dp), sign, 1 if normalise else 0)
        return a

    def gradient(self, c):
        out = np.empty(3 * self.V)
        self.lib.ref_grad(_d(np.ascontiguousarray(c, np.float64)), _d(out))
        return out

    def sorting(self, p):
        nc, _ = cell_geometry(self.P)
        keys = np.zeros(self.n, np.int32)
        srt = np.zeros(self.n, np.int32)
        off = np.zeros(int(np.prod(nc)) + 1, np.int32)
        mark = np.array([-1], np.int32)
        st = self.lib.ref_sorting(_d(np.ascontiguousarray(p)), _i(keys), _i(srt), _i(off),
                                  _i(mark))
        return st, keys, srt, off, int(mark[0])

    def f_pp(self, p, t, f_pi=None):
        out = np.zeros(3 * self.n)
        tau = np.zeros(1)
        fpi = None if f_pi is None else np.ascontiguousarray(f_pi, np.float64)
        st = self.lib.ref_f_pp(_d(np.ascontiguousarray(p)), t, _d(fpi), _d(out), _d(tau))
        return st, out, float(tau[0])

    def interpolate(self, field, p):
        n = len(p) // 3
        out = np.zeros(n)
        self.lib.ref_interpolate(_d(np.ascontiguousarray(field)), n, _d(np.ascontiguousarray(p)),
                                 _d(out))
        return out

    def f_pi(self, c_loc, dcdx, r=None):
        n = len(c_loc)
        out = np.zeros(3 * n)
        self.lib.ref_f_pi(n, _d(np.ascontiguousarray(c_loc)), _d(np.ascontiguousarray(dcdx)),
                          None if r is None else _d(np.ascontiguousarray(r)), _d(out))
        return out

    def advect(self, stage, f_pi_, f_pp_, r, p, p_old, u_old):
        n = len(p) // 3
        p, p_old, u_old = (np.ascontiguousarray(a, np.float64).copy() for a in (p, p_old, u_old))
        self.lib.ref_advect(n, stage, _d(np.ascontiguousarray(f_pi_)),
                            _d(np.ascontiguousarray(f_pp_)),
                            None if r is None else _d(np.ascontiguousarray(r)), _d(p), _d(p_old),
                            _d(u_old))
        return p, p_old, u_old

    def spread(self, p, f_pp_):
        out = np.zeros(3 * self.V)
        self.lib.ref_spread(_d(np.ascontiguousarray(p)), _d(np.ascontiguousarray(f_pp_)), _d(out))
        return out


def reference_available() -> bool:
    sys.path.insert(0, str(HERE / "ref"))
    import build_ref  # noqa: E402

    return build_ref.reference_available()
