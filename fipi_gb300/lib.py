"""ctypes binding of libfipi_gb300.so (the C ABI declared in include/fipi.h).

`Simulation` mirrors the reference's step interface: the loop body of
main.cpp (`step`), the `cluster` calls (`cells_build` = sorting,
`f_pp` = compute_f_pp, `spread` = compute_f_r, `advect` + wrap), the
`element` calls (`f_pi` = get_f_pi, `interpolate` = get_local_c/dcdx) and
the `field` transforms (`fft_r2c`, `fft_c2r`, `grad`).  Every call goes
through the C ABI; there is no other implementation behind it, and a
missing or unloadable library raises instead of falling back.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from .params import FipiParams

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p

FIPI_FP64 = 0
FIPI_MIXED = 1
FIPI_DEBUG_FFT_FIRST_WAIT_POLLS = 1
STATUS = {
    0: "FIPI_OK", 1: "FIPI_ERR_BAD_PARAMS", 2: "FIPI_ERR_BAD_ARG", 3: "FIPI_ERR_CUDA",
    4: "FIPI_ERR_OUT_OF_RANGE", 5: "FIPI_ERR_NONFINITE", 6: "FIPI_ERR_NO_DEVICE",
    7: "FIPI_ERR_STATE", 8: "FIPI_ERR_UNSUPPORTED", 9: "FIPI_ERR_RANGE", 10: "FIPI_ERR_TIMEOUT",
}


class ParamGrads(ctypes.Structure):
    """ctypes image of `struct fipi_param_grads` (include/fipi.h)."""

    _fields_ = [("mobility", ctypes.c_double), ("sigma", ctypes.c_double), ("lambda_", ctypes.c_double),
                ("k_n", ctypes.c_double), ("sigma_attach", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class FipiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None

# name: (restype, argtypes)
_SIGS = {
    "fipi_abi_version": (ctypes.c_int, []),
    "fipi_last_error_string": (ctypes.c_char_p, []),
    "fipi_params_reference": (ctypes.c_int, [ctypes.POINTER(FipiParams)]),
    "fipi_cell_geometry": (ctypes.c_int, [ctypes.POINTER(FipiParams), _ip, _dp]),
    "fipi_create": (ctypes.c_int, [ctypes.POINTER(FipiParams), ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(_vp)]),
    "fipi_destroy": (ctypes.c_int, [_vp]),
    "fipi_device_bytes": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_size_t)]),
    "fipi_set_phase": (ctypes.c_int, [_vp, _dp]),
    "fipi_set_velocity": (ctypes.c_int, [_vp, _dp]),
    "fipi_set_particles": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "fipi_get_phase": (ctypes.c_int, [_vp, _dp]),
    "fipi_get_velocity": (ctypes.c_int, [_vp, _dp]),
    "fipi_get_particles": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    "fipi_get_time": (ctypes.c_int, [_vp, _ip]),
    "fipi_step": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fipi_step_async": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fipi_step_ch": (ctypes.c_int, [_vp]),
    "fipi_step_stokes": (ctypes.c_int, [_vp]),
    "fipi_step_particles": (ctypes.c_int, [_vp]),
    "fipi_wrap": (ctypes.c_int, [_vp, _dp]),
    "fipi_set_fluid_coupling": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fipi_set_phase_device": (ctypes.c_int, [_vp, _vp]),
    "fipi_set_velocity_device": (ctypes.c_int, [_vp, _vp]),
    "fipi_set_particles_device": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "fipi_get_phase_device": (ctypes.c_int, [_vp, _vp]),
    "fipi_get_velocity_device": (ctypes.c_int, [_vp, _vp]),
    "fipi_get_particles_device": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "fipi_set_brownian": (ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_uint64]),
    "fipi_set_mass_conserving": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fipi_set_params": (ctypes.c_int, [_vp, ctypes.POINTER(FipiParams)]),
    "fipi_set_debug": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_longlong]),
    "fipi_interpolate2": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp, _dp]),
    "fipi_div": (ctypes.c_int, [_vp, _dp, _dp]),
    "fipi_sync": (ctypes.c_int, [_vp]),
    "fipi_stream": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "fipi_mass": (ctypes.c_int, [_vp, _dp]),
    "fipi_free_energy": (ctypes.c_int, [_vp, _dp]),
    "fipi_packing_tau": (ctypes.c_int, [_vp, _dp]),
    "fipi_fft_r2c": (ctypes.c_int, [_vp, _dp, _dp]),
    "fipi_fft_c2r": (ctypes.c_int, [_vp, _dp, _dp]),
    "fipi_grad": (ctypes.c_int, [_vp, _dp, _dp]),
    "fipi_cells_build": (ctypes.c_int, [_vp, _dp, _ip, _ip, _ip]),
    "fipi_f_pp": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp, _dp, _dp]),
    "fipi_pairs": (ctypes.c_int, [_vp, _dp, _ip, ctypes.c_int, _ip]),
    "fipi_interpolate": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp, _dp]),
    "fipi_f_pi": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp, _dp]),
    "fipi_advect": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp]),
    "fipi_spread": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    "fipi_cells_build_noalloc": (ctypes.c_int, [ctypes.POINTER(FipiParams), _vp, _vp, _vp, _vp, _vp]),
    "fipi_set_kernel_timing": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fipi_kernel_stat_count": (ctypes.c_int, [_vp, _ip]),
    "fipi_kernel_stats": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_longlong), _dp, _dp]),
    "fipi_launch_count": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
    "fipi_fma_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp]),
    "fipi_vtk_write_field": (ctypes.c_int, [ctypes.POINTER(FipiParams), ctypes.c_char_p, ctypes.c_char_p,
                                            ctypes.c_int, _dp]),
    "fipi_vtk_write_particles": (ctypes.c_int, [ctypes.POINTER(FipiParams), ctypes.c_char_p, ctypes.c_int, _dp,
                                                _dp, _dp]),
    "fipi_free_energy_density": (ctypes.c_int, [ctypes.POINTER(FipiParams), _dp, _dp, _dp]),
    "fipi_write_vtk": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_char_p]),
    "fipi_checkpoint_reserve": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fipi_checkpoint_bytes": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_size_t)]),
    "fipi_checkpoint_save": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fipi_checkpoint_load": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fipi_checkpoint_export": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_size_t]),
    "fipi_checkpoint_import": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_size_t]),
    "fipi_adjoint_seed": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "fipi_adjoint_step": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fipi_adjoint_get": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "fipi_adjoint_get_history": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    "fipi_adjoint_get_params": (ctypes.c_int, [_vp, ctypes.c_void_p, _dp]),
    "fipi_trajectory_forward": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "fipi_trajectory_backward": (ctypes.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "fipi_seed_phase": (ctypes.c_int, [ctypes.POINTER(FipiParams), ctypes.c_uint64, ctypes.c_double,
                                       ctypes.c_double, _dp]),
    "fipi_reference_initial_state": (ctypes.c_int, [ctypes.POINTER(FipiParams), ctypes.c_uint, _dp, _dp]),
    "fipi_seed_particles": (ctypes.c_int, [ctypes.POINTER(FipiParams), ctypes.c_uint64,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int, _dp, _dp, _dp]),
}


def library_path() -> Path:
    from .build import LIB

    return LIB


def load(build_if_missing: bool = True):
    """Load libfipi_gb300.so (building it first when absent or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build

    if build_if_missing:
        _build.build()
    path = library_path()
    if not path.exists():
        raise FileNotFoundError(f"{path} is missing: run fipi_gb300.build.build()")
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def declared_symbols() -> list[str]:
    return list(_SIGS)


def _check(code: int):
    if code != 0:
        msg = load().fipi_last_error_string().decode(errors="replace")
        raise FipiError(code, msg)


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _dev(x, n=None):
    """Device address of an FP64 device array: an int, or an object with
    data_ptr() (a contiguous float64 torch CUDA tensor); None stays None."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        if str(getattr(x, "dtype", "torch.float64")) != "torch.float64":
            raise TypeError("device arrays must be float64")
        if hasattr(x, "is_contiguous") and not x.is_contiguous():
            raise ValueError("device arrays must be contiguous")
        if n is not None and hasattr(x, "numel") and x.numel() != n:
            raise ValueError(f"expected {n} values, got {x.numel()}")
        return ctypes.c_void_p(x.data_ptr())
    return ctypes.c_void_p(int(x))


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


def _f64(a, n=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def reference_params() -> FipiParams:
    p = FipiParams()
    _check(load().fipi_params_reference(ctypes.byref(p)))
    return p


def cell_geometry(params: FipiParams):
    nc = np.zeros(3, np.int32)
    dc = np.zeros(3)
    _check(load().fipi_cell_geometry(ctypes.byref(params), _i(nc), _d(dc)))
    return nc, dc


def seed_phase(params: FipiParams, seed: int, mean: float = 0.0, amp: float = 0.05) -> np.ndarray:
    V = params.nx * params.ny * params.nz
    c = np.empty(V)
    _check(load().fipi_seed_phase(ctypes.byref(params), seed, mean, amp, _d(c)))
    return c


def fma_peak(device: int = 0, fp64: bool = True) -> float:
    """Measured FMA throughput of the device in TFLOP/s (FMA = 2 FLOPs)."""
    v = ctypes.c_double()
    _check(load().fipi_fma_peak(device, 1 if fp64 else 0, ctypes.byref(v)))
    return v.value


def vtk_write_field(params: FipiParams, path, name: str, values, components: int = 1):
    """field::output_to_file of the reference (no device needed)."""
    v = _f64(values, components * params.nx * params.ny * params.nz)
    _check(load().fipi_vtk_write_field(ctypes.byref(params), str(path).encode(), name.encode(), components, _d(v)))


def vtk_write_particles(params: FipiParams, path, p, r=None, f_pp=None):
    """cluster::output of the reference (no device needed)."""
    n = params.n_p
    pp = _f64(p, 3 * n)
    fp = _f64(f_pp if f_pp is not None else np.zeros(3 * n), 3 * n)
    _check(load().fipi_vtk_write_particles(ctypes.byref(params), str(path).encode(), n, _d(pp),
                                           _d(_f64(r, n)), _d(fp)))


def free_energy_density(params: FipiParams, c, grad_c) -> np.ndarray:
    V = params.nx * params.ny * params.nz
    out = np.empty(V)
    _check(load().fipi_free_energy_density(ctypes.byref(params), _d(_f64(c, V)), _d(_f64(grad_c, 3 * V)), _d(out)))
    return out


def reference_initial_state(params: FipiParams, seed: int, phase: bool = True):
    """The reference's own set-up draws for srand(seed): the phase field
    (field.cpp:85-99) and cluster::distribute (cluster.cpp:53-113).  Returns
    (c or None, positions n_p x 3 flattened)."""
    V = params.nx * params.ny * params.nz
    c = np.empty(V) if phase else None
    pos = np.empty(3 * max(params.n_p, 0))
    _check(load().fipi_reference_initial_state(ctypes.byref(params), seed, _d(c) if phase else None, _d(pos)))
    return c, pos


def seed_particles(params: FipiParams, seed: int, r_range=None, theta_range_deg=None,
                   allow_overlap: bool = False):
    n = params.n_p
    pos = np.empty(3 * max(n, 0))
    r = np.empty(max(n, 0))
    ct = np.empty(max(n, 0))
    rmin, rmax = r_range if r_range else (params.r_p, params.r_p)
    tmin, tmax = theta_range_deg if theta_range_deg else (90.0, 90.0)
    _check(load().fipi_seed_particles(ctypes.byref(params), seed, rmin, rmax, tmin, tmax,
                                      1 if allow_overlap else 0, _d(pos), _d(r), _d(ct)))
    return pos, r, ct


class Simulation:
    """One FIPI simulation on one GPU (a `fipi_ctx`)."""

    def __init__(self, params: FipiParams, precision: str = "fp64", device: int = 0):
        self.lib = load()
        self.params = params
        self.precision = precision
        prec = {"fp64": FIPI_FP64, "mixed": FIPI_MIXED}[precision]
        h = _vp()
        _check(self.lib.fipi_create(ctypes.byref(params), prec, device, ctypes.byref(h)))
        self.h = h
        self.V = params.nx * params.ny * params.nz
        self.n = params.n_p
        self.SH = params.nz * (params.nx // 2 + 1) * params.ny

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fipi_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---------------------------------------------------------------- state
    def set_phase(self, c):
        _check(self.lib.fipi_set_phase(self.h, _d(_f64(c, self.V))))

    def set_velocity(self, u):
        _check(self.lib.fipi_set_velocity(self.h, _d(_f64(u, 3 * self.V))))

    def set_particles(self, p, r=None, cos_theta=None, f_pp=None):
        _check(self.lib.fipi_set_particles(self.h, _d(_f64(p, 3 * self.n)), _d(_f64(r, self.n)),
                                           _d(_f64(cos_theta, self.n)), _d(_f64(f_pp, 3 * self.n))))

    def get_phase(self):
        out = np.empty(self.V)
        _check(self.lib.fipi_get_phase(self.h, _d(out)))
        return out

    def get_velocity(self):
        out = np.empty(3 * self.V)
        _check(self.lib.fipi_get_velocity(self.h, _d(out)))
        return out

    def get_particles(self, out=None):
        """(positions, f_pp, f_pi), n_p x 3 each; `out`: three float64 arrays
        of 3 n_p values to fill instead of new ones."""
        n = self.n
        if out is None:
            p, fpp, fpi = np.empty(3 * n), np.empty(3 * n), np.empty(3 * n)
        else:
            p, fpp, fpi = out
            for a in out:
                if a.dtype != np.float64 or a.size != 3 * n or not a.flags.c_contiguous:
                    raise ValueError(f"out arrays must be contiguous float64 of {3 * n} values")
        _check(self.lib.fipi_get_particles(self.h, _d(p), _d(fpp), _d(fpi)))
        return p, fpp, fpi

    @property
    def time(self) -> int:
        t = ctypes.c_int()
        _check(self.lib.fipi_get_time(self.h, ctypes.byref(t)))
        return t.value

    def step(self, n: int = 1):
        _check(self.lib.fipi_step(self.h, n))

    def step_ch(self):
        _check(self.lib.fipi_step_ch(self.h))

    def step_stokes(self):
        _check(self.lib.fipi_step_stokes(self.h))

    def step_particles(self):
        _check(self.lib.fipi_step_particles(self.h))

    def interpolate2(self, fields, p):
        fields = _f64(fields)
        nf = fields.size // self.V
        out = np.empty(self.n * nf)
        _check(self.lib.fipi_interpolate2(self.h, _d(fields), nf, _d(_f64(p, 3 * self.n)), _d(out)))
        return out.reshape(self.n, nf)

    def div(self, v) -> np.ndarray:
        out = np.empty(self.V)
        _check(self.lib.fipi_div(self.h, _d(_f64(v, 3 * self.V)), _d(out)))
        return out

    # device-pointer variants: no host copies (torch CUDA tensors or raw addresses)
    def set_phase_device(self, c):
        _check(self.lib.fipi_set_phase_device(self.h, _dev(c, self.V)))

    def set_velocity_device(self, u):
        _check(self.lib.fipi_set_velocity_device(self.h, _dev(u, 3 * self.V)))

    def set_particles_device(self, p, r=None, cos_theta=None, f_pp=None):
        n = self.n
        _check(self.lib.fipi_set_particles_device(self.h, _dev(p, 3 * n), _dev(r, n), _dev(cos_theta, n),
                                                  _dev(f_pp, 3 * n)))

    def get_phase_device(self, out):
        _check(self.lib.fipi_get_phase_device(self.h, _dev(out, self.V)))

    def get_velocity_device(self, out):
        _check(self.lib.fipi_get_velocity_device(self.h, _dev(out, 3 * self.V)))

    def get_particles_device(self, p=None, f_pp=None, f_pi=None):
        n = self.n
        _check(self.lib.fipi_get_particles_device(self.h, _dev(p, 3 * n), _dev(f_pp, 3 * n), _dev(f_pi, 3 * n)))

    def set_fluid_coupling(self, on: bool = True):
        """Particles advected with the interpolated fluid velocity (off: the
        reference's uf = 0)."""
        _check(self.lib.fipi_set_fluid_coupling(self.h, 1 if on else 0))

    def set_brownian(self, kt: float, seed: int = 0):
        """Brownian force sqrt(12 pi r mu kt / dt) g per step (kt = 0: off)."""
        _check(self.lib.fipi_set_brownian(self.h, kt, seed))

    def set_params(self, params: FipiParams):
        """New physical constants (sigma, epsilon, lambda, mobility, mu,
        densities, gravity, A, k_n) for the next steps; the state is kept."""
        _check(self.lib.fipi_set_params(self.h, ctypes.byref(params)))
        self.params = params

    def set_mass_conserving(self, on: bool = True):
        """The k = 0 mode of u . grad c taken as 0 (off: the reference's drift)."""
        _check(self.lib.fipi_set_mass_conserving(self.h, 1 if on else 0))

    def set_debug(self, what: int, value: int):
        """Test hooks of the bounded device waits (fipi_set_debug)."""
        _check(self.lib.fipi_set_debug(self.h, what, value))

    def wrap(self, p) -> np.ndarray:
        out = _f64(p, 3 * self.n).copy()
        _check(self.lib.fipi_wrap(self.h, _d(out)))
        return out

    def step_async(self, n: int = 1):
        _check(self.lib.fipi_step_async(self.h, n))

    def sync(self):
        _check(self.lib.fipi_sync(self.h))

    def stream(self) -> int:
        s = _vp()
        _check(self.lib.fipi_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def device_bytes(self) -> int:
        b = ctypes.c_size_t()
        _check(self.lib.fipi_device_bytes(self.h, ctypes.byref(b)))
        return b.value

    def mass(self) -> float:
        v = ctypes.c_double()
        _check(self.lib.fipi_mass(self.h, ctypes.byref(v)))
        return v.value

    def free_energy(self) -> float:
        v = ctypes.c_double()
        _check(self.lib.fipi_free_energy(self.h, ctypes.byref(v)))
        return v.value

    def packing_tau(self) -> float:
        v = ctypes.c_double()
        _check(self.lib.fipi_packing_tau(self.h, ctypes.byref(v)))
        return v.value

    # ---------------------------------------------------------------- instrumentation
    def set_kernel_timing(self, on: bool):
        """Per-kernel CUDA-event timing (steps then launch directly, not from graphs)."""
        _check(self.lib.fipi_set_kernel_timing(self.h, 1 if on else 0))

    def kernel_stats(self) -> list[dict]:
        n = ctypes.c_int()
        _check(self.lib.fipi_kernel_stat_count(self.h, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            name = ctypes.create_string_buffer(128)
            la, ms, by = ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
            _check(self.lib.fipi_kernel_stats(self.h, i, name, 128, ctypes.byref(la), ctypes.byref(ms),
                                              ctypes.byref(by)))
            out.append({"name": name.value.decode(), "launches": la.value, "ms": ms.value, "bytes": by.value})
        return out

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        _check(self.lib.fipi_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def write_vtk(self, what: str, path):
        """VTK file of the current state: 'phase', 'free_energy', 'u' or 'particles'."""
        code = {"phase": 0, "free_energy": 1, "u": 2, "particles": 3}[what]
        _check(self.lib.fipi_write_vtk(self.h, code, str(path).encode()))

    # ---------------------------------------------------------------- checkpoints
    def checkpoint_reserve(self, slots: int):
        _check(self.lib.fipi_checkpoint_reserve(self.h, slots))

    def checkpoint_bytes(self) -> int:
        b = ctypes.c_size_t()
        _check(self.lib.fipi_checkpoint_bytes(self.h, ctypes.byref(b)))
        return b.value

    def checkpoint_save(self, slot: int):
        _check(self.lib.fipi_checkpoint_save(self.h, slot))

    def checkpoint_load(self, slot: int):
        _check(self.lib.fipi_checkpoint_load(self.h, slot))

    def checkpoint_export(self, slot: int) -> bytes:
        """Header (64 bytes) + payload of one slot."""
        buf = ctypes.create_string_buffer(64 + self.checkpoint_bytes())
        _check(self.lib.fipi_checkpoint_export(self.h, slot, ctypes.cast(buf, _vp), len(buf)))
        return buf.raw

    def checkpoint_import(self, slot: int, blob: bytes):
        buf = ctypes.create_string_buffer(bytes(blob), len(blob))
        _check(self.lib.fipi_checkpoint_import(self.h, slot, ctypes.cast(buf, _vp), len(blob)))

    # ---------------------------------------------------------------- adjoint (FP64)
    def adjoint_seed(self, dc=None, du=None, dp=None, df_pp=None):
        """Cotangent of the current state (None = zero)."""
        _check(self.lib.fipi_adjoint_seed(self.h, _d(_f64(dc, self.V)), _d(_f64(du, 3 * self.V)),
                                          _d(_f64(dp, 3 * self.n)), _d(_f64(df_pp, 3 * self.n))))

    def adjoint_step(self, slot: int):
        _check(self.lib.fipi_adjoint_step(self.h, slot))

    def adjoint_get(self):
        """(dc, du, dp, df_pp) of the state the cotangent refers to."""
        dc, du = np.empty(self.V), np.empty(3 * self.V)
        dp, df = np.empty(3 * self.n), np.empty(3 * self.n)
        _check(self.lib.fipi_adjoint_get(self.h, _d(dc), _d(du), _d(dp) if self.n else None,
                                         _d(df) if self.n else None))
        return dc, du, dp, df

    def adjoint_get_history(self):
        """Real-field cotangents of the SBDF2 histories (c_old, f_old, conv_old)."""
        a, b, c = np.empty(self.V), np.empty(self.V), np.empty(self.V)
        _check(self.lib.fipi_adjoint_get_history(self.h, _d(a), _d(b), _d(c)))
        return a, b, c

    def adjoint_get_params(self):
        """Parameter cotangents summed over the reversed steps: a dict with
        mobility, sigma (lambda and k_n following it), lambda_, k_n,
        sigma_attach, and the per-particle cos(theta) cotangents."""
        g = ParamGrads()
        dct = np.empty(self.n)
        _check(self.lib.fipi_adjoint_get_params(self.h, ctypes.byref(g), _d(dct) if self.n else None))
        return g.as_dict(), dct

    def trajectory_forward(self, nsteps: int, stride: int = 0):
        _check(self.lib.fipi_trajectory_forward(self.h, nsteps, stride))

    def trajectory_backward(self, dc=None, du=None, dp=None, df_pp=None):
        _check(self.lib.fipi_trajectory_backward(self.h, _d(_f64(dc, self.V)), _d(_f64(du, 3 * self.V)),
                                                 _d(_f64(dp, 3 * self.n)), _d(_f64(df_pp, 3 * self.n))))

    # ---------------------------------------------------------------- fine-grained
    def fft_r2c(self, x) -> np.ndarray:
        out = np.empty(2 * self.SH)
        _check(self.lib.fipi_fft_r2c(self.h, _d(_f64(x, self.V)), _d(out)))
        return out.view(np.complex128)

    def fft_c2r(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, np.complex128).ravel()
        if X.size != self.SH:
            raise ValueError("half spectrum size mismatch")
        out = np.empty(self.V)
        _check(self.lib.fipi_fft_c2r(self.h, _d(X.view(np.float64)), _d(out)))
        return out

    def grad(self, c) -> np.ndarray:
        out = np.empty(3 * self.V)
        _check(self.lib.fipi_grad(self.h, _d(_f64(c, self.V)), _d(out)))
        return out

    def cells_build(self, p):
        nc, _ = cell_geometry(self.params)
        keys = np.empty(self.n, np.int32)
        srt = np.empty(self.n, np.int32)
        off = np.empty(int(np.prod(nc)) + 1, np.int32)
        _check(self.lib.fipi_cells_build(self.h, _d(_f64(p, 3 * self.n)), _i(keys), _i(srt), _i(off)))
        return keys, srt, off

    def f_pp(self, p, t, f_pi=None):
        out = np.empty(3 * self.n)
        tau = ctypes.c_double()
        _check(self.lib.fipi_f_pp(self.h, _d(_f64(p, 3 * self.n)), t, _d(_f64(f_pi, 3 * self.n)),
                                  _d(out), ctypes.byref(tau)))
        return out, tau.value

    def pairs(self, p):
        p = _f64(p, 3 * self.n)
        cnt = ctypes.c_int()
        _check(self.lib.fipi_pairs(self.h, _d(p), None, 0, ctypes.byref(cnt)))
        out = np.empty(2 * max(cnt.value, 1), np.int32)
        _check(self.lib.fipi_pairs(self.h, _d(p), _i(out), cnt.value, ctypes.byref(cnt)))
        return out[: 2 * cnt.value].reshape(-1, 2)

    def interpolate(self, fields, p):
        fields = _f64(fields)
        nf = fields.size // self.V
        out = np.empty(self.n * nf)
        _check(self.lib.fipi_interpolate(self.h, _d(fields), nf, _d(_f64(p, 3 * self.n)), _d(out)))
        return out.reshape(self.n, nf)

    def f_pi(self, c_loc, dcdx, r=None, cos_theta=None):
        out = np.empty(3 * self.n)
        _check(self.lib.fipi_f_pi(self.h, _d(_f64(c_loc, self.n)), _d(_f64(dcdx, 3 * self.n)),
                                  _d(_f64(r, self.n)), _d(_f64(cos_theta, self.n)), _d(out)))
        return out

    def advect(self, stage, f_pi, f_pp, r, p, p_old, u_old):
        p, p_old, u_old = (_f64(a, 3 * self.n).copy() for a in (p, p_old, u_old))
        _check(self.lib.fipi_advect(self.h, stage, _d(_f64(f_pi, 3 * self.n)), _d(_f64(f_pp, 3 * self.n)),
                                    _d(_f64(r, self.n)), _d(p), _d(p_old), _d(u_old)))
        return p, p_old, u_old

    def spread(self, p, f_pp):
        out = np.empty(3 * self.V)
        _check(self.lib.fipi_spread(self.h, _d(_f64(p, 3 * self.n)), _d(_f64(f_pp, 3 * self.n)), _d(out)))
        return out
