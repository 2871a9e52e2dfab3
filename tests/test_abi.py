"""CPU-side checks of the C ABI: the library loads, exports every function
that include/euler2d_gb300.h declares, and rejects bad arguments before it
touches a device.  No kernel is launched here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "euler2d_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(e2d_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("e2d_create", "e2d_destroy", "e2d_compute_dt", "e2d_make_boundaries", "e2d_godunov_unsplit",
              "e2d_advance", "e2d_upload_state", "e2d_download_state"):
        assert n in names


@pytest.mark.parametrize("arith", ["exact", "fma"])
def test_library_exports_every_declared_symbol(e2d, arith):
    lib = ctypes.CDLL(e2d.LIB_PATHS[arith])
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"
    assert sorted(e2d.EXPORTED_SYMBOLS) == declared_functions()


def test_each_build_reports_its_arithmetic(e2d):
    """e2d_arithmetic needs no device: the exact and the FMA builds say which
    they are, and load_library refuses a file that says otherwise."""
    assert e2d.arithmetic("exact") == e2d.ARITH_EXACT
    assert e2d.arithmetic("fma") == e2d.ARITH_FMA
    lib = e2d.load_library("exact")
    assert lib.e2d_arithmetic(None) == e2d.E2D_ERR_INVALID_ARG


def test_params_struct_layout_matches_header(e2d, tmp_path):
    """The ctypes mirror of e2d_params has the C compiler's size and offsets."""
    fields = [f[0] for f in e2d.Params._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "euler2d_gb300.h"\nint main(void){\n'
                   '  printf("%zu", sizeof(e2d_params));\n'
                   + "".join(f'  printf(" %zu", offsetof(e2d_params, {f}));\n' for f in fields)
                   + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    import subprocess
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == ctypes.sizeof(e2d.Params)
    assert out[1:] == [getattr(e2d.Params, f).offset for f in fields]
    p = e2d.default_params()
    assert p.niter_riemann == 10 and p.slope_type == 2 and p.precision == 8
    assert p.boundary_type_xmin == p.boundary_type_ymax == 1


@pytest.mark.parametrize("field,value", [
    ("nx", 1), ("ny", 0), ("implementation_version", 3), ("riemann_solver", 1), ("precision", 2),
    ("gamma0", 1.0), ("cfl", 0.0), ("smallr", 0.0), ("niter_riemann", -1),
])
def test_create_rejects_invalid_parameters(e2d, field, value):
    p = e2d.default_params()
    setattr(p, field, value)
    h = ctypes.c_void_p()
    rc = e2d.load_library().e2d_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == e2d.E2D_ERR_INVALID_ARG
    assert not h.value
    assert e2d.load_library().e2d_last_error()


def test_null_handles_are_rejected(e2d):
    lib = e2d.load_library()
    assert lib.e2d_destroy(None) == e2d.E2D_OK
    assert lib.e2d_synchronize(None) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_godunov_unsplit(None, 0, 1e-3) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_advance(None, 0, 1, None) == e2d.E2D_ERR_INVALID_ARG


def test_create_without_device_fails_cleanly(e2d):
    """On a machine without a GPU, create reports E2D_ERR_NO_DEVICE."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    p = e2d.default_params()
    p.nx = p.ny = 16
    h = ctypes.c_void_p()
    assert e2d.load_library().e2d_create(ctypes.byref(p), ctypes.byref(h)) == e2d.E2D_ERR_NO_DEVICE


def test_batch_create_rejects_invalid_arguments(e2d):
    lib = e2d.load_library()
    p = e2d.default_params()
    h = ctypes.c_void_p()
    nx = (ctypes.c_int * 2)(16, 1)
    ny = (ctypes.c_int * 2)(16, 16)
    assert lib.e2d_batch_create(ctypes.byref(p), 2, nx, ny, None, ctypes.byref(h)) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_batch_create(ctypes.byref(p), 0, nx, ny, None, ctypes.byref(h)) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_batch_destroy(None) == e2d.E2D_OK
    assert lib.e2d_batch_advance(None, 0, 1, None) == e2d.E2D_ERR_INVALID_ARG


def test_adjoint_create_rejects_invalid_arguments(e2d):
    lib = e2d.load_library()
    h = ctypes.c_void_p()
    p = e2d.make_params(nx=16, ny=16, riemann_solver=e2d.RIEMANN_APPROX)
    assert lib.e2d_adjoint_create(ctypes.byref(p), ctypes.byref(h)) == e2d.E2D_ERR_INVALID_ARG  # HLLC only
    p = e2d.make_params(nx=16, ny=16, riemann_solver=e2d.RIEMANN_HLLC, precision=4)
    assert lib.e2d_adjoint_create(ctypes.byref(p), ctypes.byref(h)) == e2d.E2D_ERR_INVALID_ARG  # FP64 only
    p = e2d.make_params(nx=16, ny=16, riemann_solver=e2d.RIEMANN_HLLC)
    nx = (ctypes.c_int * 2)(16, 1)
    ny = (ctypes.c_int * 2)(16, 16)
    assert lib.e2d_adjoint_batch_create(ctypes.byref(p), 2, nx, ny, None, ctypes.byref(h)) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_adjoint_batch_create(ctypes.byref(p), 0, nx, ny, None, ctypes.byref(h)) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_adjoint_destroy(None) == e2d.E2D_OK
    assert lib.e2d_adjoint_batch_destroy(None) == e2d.E2D_OK
    J = ctypes.c_double()
    assert lib.e2d_adjoint_batch_objective(None, 10, 0.6, 0.6, 0.1, ctypes.byref(J)) == e2d.E2D_ERR_INVALID_ARG
    k, t = ctypes.c_int(), ctypes.c_int()
    assert lib.e2d_adjoint_layout(None, ctypes.byref(k), ctypes.byref(t)) == e2d.E2D_ERR_INVALID_ARG


def test_async_download_and_selftest_reject_invalid_arguments(e2d):
    lib = e2d.load_library()
    buf = ctypes.create_string_buffer(64)
    assert lib.e2d_begin_download(None, 0, buf) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_wait_download(None) == e2d.E2D_ERR_INVALID_ARG
    p = ctypes.c_void_p()
    assert lib.e2d_host_alloc(0, ctypes.byref(p)) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_host_alloc(64, None) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_host_free(None) == e2d.E2D_OK
    a, b = ctypes.c_int(), ctypes.c_int()
    assert lib.e2d_selftest_wait(0, ctypes.byref(a), ctypes.byref(b), None) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_selftest_wait(1 << 40, ctypes.byref(a), ctypes.byref(b), None) == e2d.E2D_ERR_INVALID_ARG
    assert lib.e2d_selftest_wait(1000, None, ctypes.byref(b), None) == e2d.E2D_ERR_INVALID_ARG
