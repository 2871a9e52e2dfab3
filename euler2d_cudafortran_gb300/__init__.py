"""GB300-native Euler-2D explicit step (pkestene/euler2d_cudaFortran hot path).

Python host mirror of the reference's ``m_run`` module procedures, calling the
C ABI of ``libeuler2d_gb300.so`` (include/euler2d_gb300.h) through ctypes:

=====================================  =========================================
reference (serial_ref/m_run.f90)       here
=====================================  =========================================
initHydroParameters + run_init :48,150 ``HydroRun(params)``
init_implode :524                      ``HydroRun.init_implode()``
compute_dt(params, dt, useU) :248      ``HydroRun.compute_dt(useU)``
make_boundaries(params, data) :561     ``HydroRun.make_boundaries(which)``
godunov_unsplit(nStep, dt) :187        ``HydroRun.godunov_unsplit(nStep, dt)``
main.f90:53-76 loop (no I/O)           ``HydroRun.advance(nStep0, nsteps)``
saveVTK(data, iStep) :653              ``vtk.save_vtk(...)``
run_cleanup :172                       ``HydroRun.close()``
=====================================  =========================================

There is no CPU fallback: every call runs the CUDA library, and importing the
wrapper fails loudly if the library was not built.

Two builds of the library share the C ABI (``e2d_arithmetic``): ``"exact"``
(``libeuler2d_gb300.so``, no multiply-add contraction, bitwise serial_ref
arithmetic) and ``"fma"`` (``libeuler2d_gb300_fma.so``, multiply-adds fused).
Every class takes ``arith=`` to pick one; the default is ``"exact"``, or the
value of the environment variable ``E2D_ARITH``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIBS as LIB_PATHS
from .namelist import RunConfig, read_config  # noqa: F401

LIB_PATH = LIB_PATHS["exact"]
ARITH_EXACT = 0
ARITH_FMA = 1

E2D_OK = 0
E2D_ERR_INVALID_ARG = 1
E2D_ERR_CUDA = 2
E2D_ERR_OOM = 3
E2D_ERR_NUMERICS = 4
E2D_ERR_NO_DEVICE = 5
HEALTH_DT_NONFINITE = 1
HEALTH_NEG_DENSITY = 2
HEALTH_TMA_TIMEOUT = 4
RIEMANN_APPROX = 0
RIEMANN_HLLC = 2

EXPORTED_SYMBOLS = [
    "e2d_default_params", "e2d_arithmetic", "e2d_create", "e2d_destroy", "e2d_get_sizes", "e2d_set_stream", "e2d_synchronize",
    "e2d_init_implode", "e2d_init_diagonal", "e2d_upload_state", "e2d_download_state", "e2d_compute_dt",
    "e2d_make_boundaries", "e2d_godunov_unsplit", "e2d_advance", "e2d_last_advance_ms", "e2d_get_invdt",
    "e2d_get_health", "e2d_last_error", "e2d_device_state", "e2d_time_steps", "e2d_measure_fp64_peak",
    "e2d_godunov_unsplit_noalloc", "e2d_selftest_arith", "e2d_selftest_wait", "e2d_begin_download",
    "e2d_wait_download",
    "e2d_host_alloc", "e2d_host_free",
    "e2d_batch_create", "e2d_batch_destroy", "e2d_batch_init_diagonal", "e2d_batch_upload_state",
    "e2d_batch_download_state", "e2d_batch_advance", "e2d_batch_last_advance_ms", "e2d_batch_set_schedule",
    "e2d_batch_get_schedule", "e2d_batch_tune", "e2d_batch_get_health",
    "e2d_adjoint_create", "e2d_adjoint_destroy", "e2d_adjoint_objective", "e2d_adjoint_gradient",
    "e2d_adjoint_last_ms", "e2d_adjoint_layout",
    "e2d_adjoint_batch_create", "e2d_adjoint_batch_destroy", "e2d_adjoint_batch_init_diagonal",
    "e2d_adjoint_batch_upload_state", "e2d_adjoint_batch_objective", "e2d_adjoint_batch_gradient",
    "e2d_adjoint_batch_last_ms",
]


class E2DError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"euler2d_gb300 error {code}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    """struct e2d_params of include/euler2d_gb300.h."""
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("gamma0", ctypes.c_double), ("cfl", ctypes.c_double),
        ("smallr", ctypes.c_double), ("smallc", ctypes.c_double),
        ("niter_riemann", ctypes.c_int), ("iorder", ctypes.c_int), ("slope_type", ctypes.c_int),
        ("boundary_type_xmin", ctypes.c_int), ("boundary_type_xmax", ctypes.c_int),
        ("boundary_type_ymin", ctypes.c_int), ("boundary_type_ymax", ctypes.c_int),
        ("implementation_version", ctypes.c_int), ("riemann_solver", ctypes.c_int),
        ("precision", ctypes.c_int),
    ]


_libs: dict = {}


def default_arith() -> str:
    a = os.environ.get("E2D_ARITH", "exact")
    if a not in LIB_PATHS:
        raise ValueError(f"E2D_ARITH must be one of {sorted(LIB_PATHS)}, not {a!r}")
    return a


def load_library(arith: str | None = None):
    """Load one build of the CUDA library, "exact" or "fma" (raises if it has
    not been built)."""
    arith = arith or default_arith()
    if arith in _libs:
        return _libs[arith]
    if arith not in LIB_PATHS:
        raise ValueError(f"arith must be one of {sorted(LIB_PATHS)}, not {arith!r}")
    path = LIB_PATHS[arith]
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m euler2d_cudafortran_gb300.build` "
                          "(there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    vp, ip, i, d = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_double
    sig = {
        "e2d_default_params": [ctypes.POINTER(Params)],
        "e2d_arithmetic": [ip],
        "e2d_create": [ctypes.POINTER(Params), ctypes.POINTER(vp)],
        "e2d_destroy": [vp],
        "e2d_get_sizes": [vp, ip, ip, ctypes.POINTER(ctypes.c_size_t)],
        "e2d_set_stream": [vp, vp],
        "e2d_synchronize": [vp],
        "e2d_init_implode": [vp],
        "e2d_init_diagonal": [vp, d, d, d, d, d],
        "e2d_upload_state": [vp, i, vp],
        "e2d_download_state": [vp, i, vp],
        "e2d_compute_dt": [vp, i, vp],
        "e2d_make_boundaries": [vp, i],
        "e2d_godunov_unsplit": [vp, i, d],
        "e2d_advance": [vp, i, i, vp],
        "e2d_last_advance_ms": [vp, ctypes.POINTER(ctypes.c_float)],
        "e2d_time_steps": [vp, i, i, ctypes.POINTER(ctypes.c_float)],
        "e2d_measure_fp64_peak": [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
        "e2d_get_invdt": [vp, ctypes.POINTER(ctypes.c_double)],
        "e2d_get_health": [vp, ctypes.POINTER(ctypes.c_uint)],
        "e2d_device_state": [vp, i, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_size_t),
                             ctypes.POINTER(ctypes.c_size_t)],
        "e2d_godunov_unsplit_noalloc": [ctypes.POINTER(Params), vp, vp, ctypes.c_size_t, d, vp,
                                        ctypes.POINTER(ctypes.c_uint)],
        "e2d_selftest_wait": [ctypes.c_longlong, ip, ip, ctypes.POINTER(ctypes.c_longlong)],
        "e2d_begin_download": [vp, i, vp],
        "e2d_wait_download": [vp],
        "e2d_host_alloc": [ctypes.c_size_t, ctypes.POINTER(vp)],
        "e2d_host_free": [vp],
        "e2d_selftest_arith": [i, i, ctypes.c_longlong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong),
                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double)],
    }
    dp = ctypes.POINTER(ctypes.c_double)
    sig.update({
        "e2d_batch_create": [ctypes.POINTER(Params), i, ip, ip, ip, ctypes.POINTER(vp)],
        "e2d_batch_destroy": [vp],
        "e2d_batch_init_diagonal": [vp, dp, dp, dp, dp, dp],
        "e2d_batch_upload_state": [vp, i, i, vp],
        "e2d_batch_download_state": [vp, i, i, vp],
        "e2d_batch_advance": [vp, i, i, vp],
        "e2d_batch_last_advance_ms": [vp, ctypes.POINTER(ctypes.c_float)],
        "e2d_batch_set_schedule": [vp, i, i, i],
        "e2d_batch_get_schedule": [vp, ip, ip, ip, ip],
        "e2d_batch_tune": [vp, i, ctypes.c_char_p, ctypes.POINTER(ctypes.c_float)],
        "e2d_batch_get_health": [vp, i, ctypes.POINTER(ctypes.c_uint)],
        "e2d_adjoint_create": [ctypes.POINTER(Params), ctypes.POINTER(vp)],
        "e2d_adjoint_destroy": [vp],
        "e2d_adjoint_objective": [vp, vp, i, d, d, d, dp, dp],
        "e2d_adjoint_gradient": [vp, vp, i, i, d, d, d, dp, dp, dp],
        "e2d_adjoint_last_ms": [vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)],
        "e2d_adjoint_layout": [vp, ip, ip],
        "e2d_adjoint_batch_create": [ctypes.POINTER(Params), i, ip, ip, ip, ctypes.POINTER(vp)],
        "e2d_adjoint_batch_destroy": [vp],
        "e2d_adjoint_batch_init_diagonal": [vp, dp, dp, dp, dp, dp],
        "e2d_adjoint_batch_upload_state": [vp, i, vp],
        "e2d_adjoint_batch_objective": [vp, i, d, d, d, dp],
        "e2d_adjoint_batch_gradient": [vp, i, i, d, d, d, dp, dp, dp],
        "e2d_adjoint_batch_last_ms": [vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)],
    })
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.e2d_last_error.argtypes = []
    lib.e2d_last_error.restype = ctypes.c_char_p
    mode = ctypes.c_int(-1)
    lib.e2d_arithmetic(ctypes.byref(mode))
    if mode.value != {"exact": ARITH_EXACT, "fma": ARITH_FMA}[arith]:
        raise ImportError(f"{path} reports arithmetic {mode.value}, not {arith}")
    _libs[arith] = lib
    return lib


def _check(rc: int, lib=None):
    if rc != E2D_OK:
        raise E2DError(rc, (lib or load_library()).e2d_last_error().decode())


class _Handle:
    """Base of the run classes: errors are read from the library build that
    returned them."""
    _lib = None

    def _ok(self, rc: int):
        _check(rc, self._lib)


def default_params() -> Params:
    p = Params()
    _check(load_library().e2d_default_params(ctypes.byref(p)))
    return p


def params_from_config(cfg: RunConfig) -> Params:
    p = default_params()
    for k in ("nx", "ny", "gamma0", "cfl", "smallr", "smallc", "niter_riemann", "iorder", "slope_type",
              "boundary_type_xmin", "boundary_type_xmax", "boundary_type_ymin", "boundary_type_ymax",
              "riemann_solver", "precision"):
        setattr(p, k, getattr(cfg, k))
    p.implementation_version = cfg.implementationVersion
    return p


def make_params(**kw) -> Params:
    p = default_params()
    for k, v in kw.items():
        if not hasattr(p, k):
            raise TypeError(f"unknown parameter {k}")
        setattr(p, k, v)
    return p


class HydroRun(_Handle):
    """One run on the current CUDA device: u, u2 and the step's work arrays."""

    def __init__(self, params: Params | None = None, arith: str | None = None, **kw):
        self._lib = load_library(arith)
        self.params = params if params is not None else make_params(**kw)
        h = ctypes.c_void_p()
        self._ok(self._lib.e2d_create(ctypes.byref(self.params), ctypes.byref(h)))
        self._h = h
        isz, jsz, nb = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
        self._ok(self._lib.e2d_get_sizes(h, ctypes.byref(isz), ctypes.byref(jsz), ctypes.byref(nb)))
        self.isize, self.jsize, self.state_bytes = isz.value, jsz.value, nb.value
        self.dtype = np.float64 if self.params.precision == 8 else np.float32

    # -- lifecycle -------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.e2d_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state -----------------------------------------------------------
    def new_state(self) -> np.ndarray:
        return np.zeros((4, self.jsize, self.isize), dtype=self.dtype)

    def init_implode(self):
        self._ok(self._lib.e2d_init_implode(self._h))

    def init_diagonal(self, offset, rho_hi, p_hi, rho_lo, p_lo):
        self._ok(self._lib.e2d_init_diagonal(self._h, offset, rho_hi, p_hi, rho_lo, p_lo))

    def set_state(self, which: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        if a.shape != (4, self.jsize, self.isize):
            raise ValueError(f"state must have shape (4, {self.jsize}, {self.isize})")
        self._ok(self._lib.e2d_upload_state(self._h, which, a.ctypes.data_as(ctypes.c_void_p)))

    def get_state(self, which: int, out: np.ndarray | None = None) -> np.ndarray:
        """State `which` (0 = u, 1 = u2) in Fortran layout; into `out` (e.g. a
        pinned buffer) when given."""
        if out is None:
            a = self.new_state()
        else:
            if out.shape != (4, self.jsize, self.isize) or out.dtype != self.dtype or not out.flags["C_CONTIGUOUS"]:
                raise ValueError("out must be a C-contiguous state array of this run")
            a = out
        self._ok(self._lib.e2d_download_state(self._h, which, a.ctypes.data_as(ctypes.c_void_p)))
        return a

    def begin_download(self, which: int, out: np.ndarray):
        """Starts an asynchronous copy of state `which` into `out` (see
        e2d_begin_download); call wait_download() before reading `out`."""
        if out.shape != (4, self.jsize, self.isize) or out.dtype != self.dtype or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous state array of this run")
        self._pending_out = out
        self._ok(self._lib.e2d_begin_download(self._h, which, out.ctypes.data_as(ctypes.c_void_p)))

    def wait_download(self) -> np.ndarray | None:
        self._ok(self._lib.e2d_wait_download(self._h))
        out, self._pending_out = getattr(self, "_pending_out", None), None
        return out

    # -- the reference procedures -----------------------------------------
    def compute_dt(self, useU: int) -> float:
        dt = (ctypes.c_double if self.params.precision == 8 else ctypes.c_float)()
        self._ok(self._lib.e2d_compute_dt(self._h, useU, ctypes.byref(dt)))
        return dt.value

    def make_boundaries(self, which: int):
        self._ok(self._lib.e2d_make_boundaries(self._h, which))

    def godunov_unsplit(self, nStep: int, dt: float):
        self._ok(self._lib.e2d_godunov_unsplit(self._h, nStep, float(dt)))

    def advance(self, nStep0: int, nsteps: int, log: bool = True):
        buf = np.zeros(max(nsteps, 1), dtype=self.dtype) if log else None
        ptr = buf.ctypes.data_as(ctypes.c_void_p) if log else None
        self._ok(self._lib.e2d_advance(self._h, nStep0, nsteps, ptr))
        return buf[:nsteps] if log else None

    def last_advance_ms(self) -> float:
        ms = ctypes.c_float()
        self._ok(self._lib.e2d_last_advance_ms(self._h, ctypes.byref(ms)))
        return ms.value

    def time_steps(self, nStep0: int, nsteps: int) -> np.ndarray:
        """Per-step device time (ms) of nsteps steps launched one by one."""
        ms = np.zeros(nsteps, dtype=np.float32)
        self._ok(self._lib.e2d_time_steps(self._h, nStep0, nsteps,
                                        ms.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return ms

    def synchronize(self):
        self._ok(self._lib.e2d_synchronize(self._h))

    def set_stream(self, stream_ptr: int | None):
        self._ok(self._lib.e2d_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def invdt(self) -> float:
        x = ctypes.c_double()
        self._ok(self._lib.e2d_get_invdt(self._h, ctypes.byref(x)))
        return x.value

    def health(self) -> int:
        x = ctypes.c_uint()
        self._ok(self._lib.e2d_get_health(self._h, ctypes.byref(x)))
        return x.value

    def final_state(self, nsteps: int) -> np.ndarray:
        """The state after nsteps steps from u: u if nsteps is even, else u2."""
        return self.get_state(nsteps % 2)


class Batch(_Handle):
    """An ensemble of independent runs advanced together (e2d_batch_*)."""

    def __init__(self, sizes, bcs=None, params: Params | None = None, arith: str | None = None, **kw):
        self._lib = load_library(arith)
        self.params = params if params is not None else make_params(**kw)
        self.sizes = [(int(a), int(b)) for a, b in sizes]
        n = len(self.sizes)
        nx = (ctypes.c_int * n)(*[a for a, _ in self.sizes])
        ny = (ctypes.c_int * n)(*[b for _, b in self.sizes])
        bc = None
        if bcs is not None:
            flat = [int(x) for row in bcs for x in (row if hasattr(row, "__len__") else (row,) * 4)]
            bc = (ctypes.c_int * len(flat))(*flat)
        h = ctypes.c_void_p()
        self._ok(self._lib.e2d_batch_create(ctypes.byref(self.params), n, nx, ny, bc, ctypes.byref(h)))
        self._h = h
        self.nprob = n
        self.dtype = np.float64 if self.params.precision == 8 else np.float32

    def close(self):
        if getattr(self, "_h", None):
            self._lib.e2d_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_diagonal(self, offset, rho_hi, p_hi, rho_lo, p_lo):
        arrs = [np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (self.nprob,)))
                for x in (offset, rho_hi, p_hi, rho_lo, p_lo)]
        ptrs = [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in arrs]
        self._ok(self._lib.e2d_batch_init_diagonal(self._h, *ptrs))

    def get_state(self, prob: int, which: int) -> np.ndarray:
        nx, ny = self.sizes[prob]
        a = np.zeros((4, ny + 4, nx + 4), dtype=self.dtype)
        self._ok(self._lib.e2d_batch_download_state(self._h, prob, which, a.ctypes.data_as(ctypes.c_void_p)))
        return a

    def set_state(self, prob: int, which: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        self._ok(self._lib.e2d_batch_upload_state(self._h, prob, which, a.ctypes.data_as(ctypes.c_void_p)))

    def advance(self, nStep0: int, nsteps: int, log: bool = True):
        buf = np.zeros((max(nsteps, 1), self.nprob), dtype=self.dtype) if log else None
        self._ok(self._lib.e2d_batch_advance(self._h, nStep0, nsteps,
                                           buf.ctypes.data_as(ctypes.c_void_p) if log else None))
        return buf[:nsteps] if log else None

    def last_advance_ms(self) -> float:
        ms = ctypes.c_float()
        self._ok(self._lib.e2d_batch_last_advance_ms(self._h, ctypes.byref(ms)))
        return ms.value

    def set_schedule(self, variant: int, grid_mult: int, order: int):
        self._ok(self._lib.e2d_batch_set_schedule(self._h, variant, grid_mult, order))

    def schedule(self):
        v, m, o, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._ok(self._lib.e2d_batch_get_schedule(self._h, ctypes.byref(v), ctypes.byref(m), ctypes.byref(o),
                                                ctypes.byref(g)))
        return {"tile": ["32x15", "32x7"][v.value], "variant": v.value, "grid_mult": m.value,
                "order": ["problem", "largest-first"][o.value], "grid": g.value}

    def tune(self, steps: int = 3, cache_path: str | None = None) -> float:
        ms = ctypes.c_float()
        self._ok(self._lib.e2d_batch_tune(self._h, steps, cache_path.encode() if cache_path else None,
                                        ctypes.byref(ms)))
        return ms.value

    def health(self, prob: int) -> int:
        x = ctypes.c_uint()
        self._ok(self._lib.e2d_batch_get_health(self._h, prob, ctypes.byref(x)))
        return x.value

    def final_state(self, prob: int, nsteps: int) -> np.ndarray:
        return self.get_state(prob, nsteps % 2)


class Adjoint(_Handle):
    """Discrete adjoint of the FP64 HLLC step: J = sum rho^2 w(x, y) after
    nsteps steps and dJ/d(initial interior density) (e2d_adjoint_*)."""

    def __init__(self, params: Params | None = None, arith: str | None = None, **kw):
        self._lib = load_library(arith)
        kw.setdefault("riemann_solver", RIEMANN_HLLC)
        self.params = params if params is not None else make_params(**kw)
        h = ctypes.c_void_p()
        self._ok(self._lib.e2d_adjoint_create(ctypes.byref(self.params), ctypes.byref(h)))
        self._h = h
        self.nx, self.ny = self.params.nx, self.params.ny

    def close(self):
        if getattr(self, "_h", None):
            self._lib.e2d_adjoint_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _u0(u0):
        if u0 is None:
            return None, None
        a = np.ascontiguousarray(u0, dtype=np.float64)
        return a, a.ctypes.data_as(ctypes.c_void_p)

    def objective(self, nsteps, u0=None, xc=0.6, yc=0.6, sigma=0.1, dt_fixed=None) -> float:
        keep, ptr = self._u0(u0)
        J = ctypes.c_double()
        dtp = None
        if dt_fixed is not None:
            dtf = np.ascontiguousarray(dt_fixed, dtype=np.float64)
            dtp = dtf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self._ok(self._lib.e2d_adjoint_objective(self._h, ptr, nsteps, xc, yc, sigma, dtp, ctypes.byref(J)))
        return J.value

    def gradient(self, nsteps, u0=None, dt_mode=1, xc=0.6, yc=0.6, sigma=0.1):
        """Returns (J, dJ/drho0 as (ny, nx), dt of every step)."""
        keep, ptr = self._u0(u0)
        J = ctypes.c_double()
        g = np.zeros((self.ny, self.nx), dtype=np.float64)
        dts = np.zeros(nsteps, dtype=np.float64)
        self._ok(self._lib.e2d_adjoint_gradient(self._h, ptr, nsteps, dt_mode, xc, yc, sigma, ctypes.byref(J),
                                              g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                              dts.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return J.value, g, dts

    def last_ms(self):
        a, b = ctypes.c_float(), ctypes.c_float()
        self._ok(self._lib.e2d_adjoint_last_ms(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def layout(self):
        """(steps between checkpoints, tape in use) of the last gradient call;
        the first equals the step count when every state and tape were kept."""
        k, t = ctypes.c_int(), ctypes.c_int()
        self._ok(self._lib.e2d_adjoint_layout(self._h, ctypes.byref(k), ctypes.byref(t)))
        return k.value, bool(t.value)


class AdjointBatch(_Handle):
    """The discrete adjoint of an ensemble of FP64 HLLC problems of uneven
    sizes, all stages batched, one captured graph per call
    (e2d_adjoint_batch_*)."""

    def __init__(self, sizes, bcs=None, params: Params | None = None, arith: str | None = None, **kw):
        self._lib = load_library(arith)
        kw.setdefault("riemann_solver", RIEMANN_HLLC)
        self.params = params if params is not None else make_params(**kw)
        self.sizes = [(int(a), int(b)) for a, b in sizes]
        n = len(self.sizes)
        nx = (ctypes.c_int * n)(*[a for a, _ in self.sizes])
        ny = (ctypes.c_int * n)(*[b for _, b in self.sizes])
        bc = None
        if bcs is not None:
            flat = [int(x) for row in bcs for x in (row if hasattr(row, "__len__") else (row,) * 4)]
            bc = (ctypes.c_int * len(flat))(*flat)
        h = ctypes.c_void_p()
        self._ok(self._lib.e2d_adjoint_batch_create(ctypes.byref(self.params), n, nx, ny, bc, ctypes.byref(h)))
        self._h = h
        self.nprob = n

    def close(self):
        if getattr(self, "_h", None):
            self._lib.e2d_adjoint_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_diagonal(self, offset, rho_hi, p_hi, rho_lo, p_lo):
        arrs = [np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (self.nprob,)))
                for x in (offset, rho_hi, p_hi, rho_lo, p_lo)]
        ptrs = [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in arrs]
        self._ok(self._lib.e2d_adjoint_batch_init_diagonal(self._h, *ptrs))

    def set_state(self, prob, u0):
        a = np.ascontiguousarray(u0, dtype=np.float64)
        nx, ny = self.sizes[prob]
        if a.shape != (4, ny + 4, nx + 4):
            raise ValueError(f"state of problem {prob} must have shape {(4, ny + 4, nx + 4)}")
        self._ok(self._lib.e2d_adjoint_batch_upload_state(self._h, prob, a.ctypes.data_as(ctypes.c_void_p)))

    def objective(self, nsteps, xc=0.6, yc=0.6, sigma=0.1):
        J = np.zeros(self.nprob)
        self._ok(self._lib.e2d_adjoint_batch_objective(self._h, nsteps, xc, yc, sigma,
                                                     J.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return J

    def gradient(self, nsteps, dt_mode=1, xc=0.6, yc=0.6, sigma=0.1):
        """Returns (J[nprob], [dJ_p/drho0_p as (ny_p, nx_p)], dt log (nsteps, nprob))."""
        J = np.zeros(self.nprob)
        g = np.zeros(sum(a * b for a, b in self.sizes))
        dts = np.zeros((nsteps, self.nprob))
        dp = ctypes.POINTER(ctypes.c_double)
        self._ok(self._lib.e2d_adjoint_batch_gradient(self._h, nsteps, dt_mode, xc, yc, sigma, J.ctypes.data_as(dp),
                                                    g.ctypes.data_as(dp), dts.ctypes.data_as(dp)))
        grads, o = [], 0
        for nx, ny in self.sizes:
            grads.append(g[o:o + nx * ny].reshape(ny, nx))
            o += nx * ny
        return J, grads, dts

    def last_ms(self):
        a, b = ctypes.c_float(), ctypes.c_float()
        self._ok(self._lib.e2d_adjoint_batch_last_ms(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value


def measure_fp64_peak():
    """(independent DFMA/s, IEEE double divisions/s) measured on the current GPU."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(load_library().e2d_measure_fp64_peak(ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def arithmetic(arith: str | None = None) -> int:
    """ARITH_EXACT or ARITH_FMA, as the loaded build reports it."""
    lib = load_library(arith)
    m = ctypes.c_int()
    _check(lib.e2d_arithmetic(ctypes.byref(m)), lib)
    return m.value


def selftest_wait(limit_cycles: int = 1 << 24):
    """(arrived barrier completed, silent barrier completed, cycles waited on the silent one)."""
    a, b, w = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
    _check(load_library().e2d_selftest_wait(limit_cycles, ctypes.byref(a), ctypes.byref(b), ctypes.byref(w)))
    return bool(a.value), bool(b.value), w.value


def selftest_arith(op: int, mode: int, n: int, seed: int = 1, rates: bool = False):
    """Bitwise check of the integer-pipe division (op 0) / square root (op 1)
    against the hardware, or of the exponent-test pressure floor (op 2) and
    limiter sign test (op 3) against the product (and maximum), or of the
    faithful division (op 4; single precision op 6) / square root (op 5; op 7)
    to within one neighbour of the hardware result, on n inputs; returns
    (mismatches, first_bad[4], rates)."""
    bad = ctypes.c_ulonglong()
    first = (ctypes.c_double * 4)()
    em, na = ctypes.c_double(), ctypes.c_double()
    _check(load_library().e2d_selftest_arith(op, mode, n, seed, ctypes.byref(bad), first,
                                              ctypes.byref(em) if rates else None,
                                              ctypes.byref(na) if rates else None))
    return bad.value, list(first), ((em.value, na.value) if rates else None)


def run_steps(nsteps: int, params: Params | None = None, u0: np.ndarray | None = None,
              mode: str = "advance", **kw):
    """The serial_ref/main.f90 loop (no output) on the GPU.

    mode="advance": one e2d_advance call (device-resident dt, graph replay).
    mode="percall": compute_dt / godunov_unsplit per step, as main.f90 calls them.
    Returns (final_state, dt_log)."""
    with HydroRun(params, **kw) as run:
        if u0 is None:
            run.init_implode()
        else:
            run.set_state(0, u0)
        if mode == "advance":
            dts = run.advance(0, nsteps)
        else:
            dt = run.compute_dt(0)
            run.make_boundaries(0)
            dts = []
            for n in range(nsteps):
                dt = run.compute_dt(n % 2)
                run.godunov_unsplit(n, dt)
                dts.append(dt)
            dts = np.array(dts, dtype=run.dtype)
        return run.final_state(nsteps), dts
