"""ctypes wrapper around the CPU oracle (oracle/euler2d_oracle.c).

TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the CUDA path: only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module.  The product library never calls it.

Arrays are numpy arrays of shape ``(4, jsize, isize)`` in C order, which is
byte-for-byte the Fortran array ``A(isize, jsize, NBVAR)`` of
serial_ref/m_run.f90:14-18 (variables ID=rho, IP=E, IU=rho*u, IV=rho*v).
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", platform.machine() or "unknown", "liboracle.so")
_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _Params(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("gamma0", ctypes.c_double), ("cfl", ctypes.c_double),
        ("smallr", ctypes.c_double), ("smallc", ctypes.c_double),
        ("niter_riemann", ctypes.c_int), ("iorder", ctypes.c_int), ("slope_type", ctypes.c_int),
        ("bc_xmin", ctypes.c_int), ("bc_xmax", ctypes.c_int),
        ("bc_ymin", ctypes.c_int), ("bc_ymax", ctypes.c_int),
        ("riemann", ctypes.c_int),
    ]


@dataclass
class Params:
    """The &MESH/&HYDRO values of a run (serial_ref/m_run.f90:56-68)."""
    nx: int = 64
    ny: int = 64
    gamma0: float = 1.4
    cfl: float = 0.8
    smallr: float = 1e-7
    smallc: float = 1e-7
    niter_riemann: int = 10
    iorder: int = 2
    slope_type: int = 2
    bc_xmin: int = 1
    bc_xmax: int = 1
    bc_ymin: int = 1
    bc_ymax: int = 1
    riemann: int = 0  # 0 two-shock approx (reference default), 2 HLLC

    @property
    def isize(self) -> int:
        return self.nx + 4

    @property
    def jsize(self) -> int:
        return self.ny + 4

    def c(self) -> _Params:
        return _Params(self.nx, self.ny, self.gamma0, self.cfl, self.smallr, self.smallc,
                       self.niter_riemann, self.iorder, self.slope_type, self.bc_xmin,
                       self.bc_xmax, self.bc_ymin, self.bc_ymax, self.riemann)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
    return _lib


def _dtype(prec: str):
    return np.float64 if prec == "f64" else np.float32


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def _real(prec: str, x: float):
    return ctypes.c_double(x) if prec == "f64" else ctypes.c_float(x)


def new_state(p: Params, prec: str = "f64") -> np.ndarray:
    return np.zeros((4, p.jsize, p.isize), dtype=_dtype(prec))


def init_implode(p: Params, prec: str = "f64") -> np.ndarray:
    """init_implode, serial_ref/m_run.f90:524-555."""
    u = new_state(p, prec)
    getattr(lib(), f"oracle_init_implode_{prec}")(ctypes.byref(p.c()), _ptr(u))
    return u


def init_diagonal(p: Params, offset: float, rho_hi: float, p_hi: float, rho_lo: float,
                  p_lo: float, prec: str = "f64") -> np.ndarray:
    u = new_state(p, prec)
    f = getattr(lib(), f"oracle_init_diagonal_{prec}")
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_double] * 5
    f(ctypes.byref(p.c()), _ptr(u), offset, rho_hi, p_hi, rho_lo, p_lo)
    return u


def make_boundaries(p: Params, u: np.ndarray) -> None:
    prec = "f64" if u.dtype == np.float64 else "f32"
    getattr(lib(), f"oracle_make_boundaries_{prec}")(ctypes.byref(p.c()), _ptr(u))


def compute_dt(p: Params, u: np.ndarray, invdt: float = 0.0, nthreads: int = 1):
    """Returns (dt, new running max invDt)."""
    prec = "f64" if u.dtype == np.float64 else "f32"
    ctype = ctypes.c_double if prec == "f64" else ctypes.c_float
    inv = ctype(invdt)
    dt = ctype(0)
    getattr(lib(), f"oracle_compute_dt_{prec}")(ctypes.byref(p.c()), _ptr(u), ctypes.byref(inv),
                                                 ctypes.byref(dt), ctypes.c_int(nthreads))
    return dt.value, inv.value


def godunov_step(p: Params, u_in: np.ndarray, u_out: np.ndarray, dt: float, nthreads: int = 1) -> None:
    prec = "f64" if u_in.dtype == np.float64 else "f32"
    getattr(lib(), f"oracle_godunov_step_{prec}")(ctypes.byref(p.c()), _ptr(u_in), _ptr(u_out),
                                                   _real(prec, dt), ctypes.c_int(nthreads))


def run(p: Params, nsteps: int, prec: str = "f64", u0: np.ndarray | None = None, nthreads: int = 1):
    """The serial_ref/main.f90 loop without I/O.

    Returns (final_state, dt_log, u, u2): final_state is u after an even number
    of steps and u2 after an odd number (serial_ref/m_run.f90:197-201)."""
    u = init_implode(p, prec) if u0 is None else np.ascontiguousarray(u0, dtype=_dtype(prec)).copy()
    u2 = new_state(p, prec)
    ctype = ctypes.c_double if prec == "f64" else ctypes.c_float
    inv = ctype(0)
    dt_log = np.zeros(max(nsteps, 1), dtype=_dtype(prec))
    rc = getattr(lib(), f"oracle_run_{prec}")(ctypes.byref(p.c()), ctypes.c_int(nsteps), _ptr(u), _ptr(u2),
                                               ctypes.byref(inv), _ptr(dt_log), ctypes.c_int(nthreads))
    if rc != 0:
        raise MemoryError("oracle_run failed to allocate its work arrays")
    final = u if nsteps % 2 == 0 else u2
    return final, dt_log[:nsteps], u, u2


# ---- objective and its forward-mode tangent ----------------------------------

def objective(p: Params, u: np.ndarray, xc=0.6, yc=0.6, sig=0.1) -> float:
    """J = sum over interior cells of rho^2 w, w a Gaussian at cell centres."""
    f = lib().oracle_objective_f64
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    return f(ctypes.byref(p.c()), _ptr(np.ascontiguousarray(u, dtype=np.float64)), xc, yc, sig)


def run_fixed_dt(p: Params, u0: np.ndarray, dts, nthreads: int = 1):
    """The driver loop with the dt of every step given (dt frozen); final state."""
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    u2 = new_state(p)
    d = np.ascontiguousarray(dts, dtype=np.float64)
    rc = lib().oracle_run_fixed_dt_f64(ctypes.byref(p.c()), ctypes.c_int(len(d)), _ptr(u), _ptr(u2), _ptr(d),
                                      ctypes.c_int(nthreads))
    if rc != 0:
        raise MemoryError("oracle_run_fixed_dt failed")
    return u if len(d) % 2 == 0 else u2


def tangent(p: Params, u0: np.ndarray, direction: np.ndarray, nsteps: int, xc=0.6, yc=0.6, sig=0.1,
            h: float = 1e-200, nthreads: int = 1, fixed_dts=None):
    """Forward-mode derivative of J(final state) along a perturbation of the
    initial interior density: the complex-step build of the oracle run from
    u0 + i h d (d on the density plane's interior).  With fixed_dts the dt
    of every step is frozen.  Returns (J, dJ.d)."""
    uc = np.ascontiguousarray(u0, dtype=np.complex128).copy()
    uc[0, 2:-2, 2:-2] += 1j * h * direction
    u2 = np.zeros_like(uc)
    inv = np.zeros(1, dtype=np.complex128)
    dts = np.zeros(max(nsteps, 1), dtype=np.complex128)
    L = lib()
    if fixed_dts is not None:
        fd = np.ascontiguousarray(fixed_dts[:nsteps], dtype=np.float64)
        rc = L.oracle_run_fixed_dt_c128(ctypes.byref(p.c()), ctypes.c_int(nsteps), _ptr(uc), _ptr(u2), _ptr(fd),
                                        ctypes.c_int(nthreads))
    else:
        rc = L.oracle_run_c128(ctypes.byref(p.c()), ctypes.c_int(nsteps), _ptr(uc), _ptr(u2), _ptr(inv),
                               _ptr(dts), ctypes.c_int(nthreads))
    if rc != 0:
        raise MemoryError("oracle_run_c128 failed")
    final = uc if nsteps % 2 == 0 else u2
    out = np.zeros(1, dtype=np.complex128)
    f = L.oracle_objective_into_c128
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                  ctypes.c_void_p]
    f(ctypes.byref(p.c()), _ptr(final), xc, yc, sig, _ptr(out))
    return out[0].real, out[0].imag / h


# ---- pointwise routines ----------------------------------------------------

def _vec(x, prec):
    return np.ascontiguousarray(x, dtype=_dtype(prec))


def primitives(p: Params, u, prec="f64"):
    u = _vec(u, prec)
    q = np.zeros(4, _dtype(prec))
    c = (ctypes.c_double if prec == "f64" else ctypes.c_float)(0)
    getattr(lib(), f"oracle_primitives_{prec}")(ctypes.byref(p.c()), _ptr(u), _ptr(q), ctypes.byref(c))
    return q, c.value


def slopes(p: Params, q, qpx, qmx, qpy, qmy, prec="f64"):
    args = [_vec(a, prec) for a in (q, qpx, qmx, qpy, qmy)]
    dqx = np.zeros(4, _dtype(prec))
    dqy = np.zeros(4, _dtype(prec))
    getattr(lib(), f"oracle_slopes_{prec}")(ctypes.byref(p.c()), *[_ptr(a) for a in args], _ptr(dqx), _ptr(dqy))
    return dqx, dqy


def trace(p: Params, q, dqx, dqy, dtdx, dtdy, face, prec="f64"):
    q, dqx, dqy = (_vec(a, prec) for a in (q, dqx, dqy))
    qf = np.zeros(4, _dtype(prec))
    getattr(lib(), f"oracle_trace_{prec}")(ctypes.byref(p.c()), _ptr(q), _ptr(dqx), _ptr(dqy),
                                            _real(prec, dtdx), _real(prec, dtdy), ctypes.c_int(face), _ptr(qf))
    return qf


def riemann_approx(p: Params, ql, qr, prec="f64"):
    ql, qr = _vec(ql, prec), _vec(qr, prec)
    flux = np.zeros(4, _dtype(prec))
    n = ctypes.c_int(0)
    getattr(lib(), f"oracle_riemann_approx_{prec}")(ctypes.byref(p.c()), _ptr(ql), _ptr(qr), _ptr(flux), ctypes.byref(n))
    return flux, n.value


def riemann_hllc(p: Params, ql, qr, prec="f64"):
    ql, qr = _vec(ql, prec), _vec(qr, prec)
    flux = np.zeros(4, _dtype(prec))
    getattr(lib(), f"oracle_riemann_hllc_{prec}")(ctypes.byref(p.c()), _ptr(ql), _ptr(qr), _ptr(flux))
    return flux
