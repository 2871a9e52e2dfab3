"""The Godunov step that allocates no device memory.

e2d_godunov_unsplit_noalloc serves callers that cannot call cudaMalloc: host
codes whose device arrays come from another allocator or memory pool, and
frameworks that hand the time step only its input and output arrays and
forbid allocation on that path.  Its work arrays live in one static device
array of E2D_NOALLOC_SCRATCH_BYTES shared by every call.  These tests check
that two calls in a row (the second reusing whatever the first left in the
static array) give the same states as the regular per-call step
e2d_godunov_unsplit, and that grids too large for the static array are
refused before any device work.
"""
import ctypes

import numpy as np
import pytest

REL_L1_TOL = 1e-12  # the parity tolerance of the other GPU tests (bitwise is expected)


def _interior(a):
    return a[:, 2:-2, 2:-2]


def _rel_l1(a, b):
    a, b = _interior(a), _interior(b)
    return max(float(np.abs(a[v] - b[v]).sum() / np.abs(b[v]).sum()) for v in range(4))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [8, 4])
def test_noalloc_step_matches_regular_step_two_calls(e2d, precision):
    torch = pytest.importorskip("torch")
    p = e2d.make_params(nx=96, ny=80, gamma0=1.4, cfl=0.8, riemann_solver=e2d.RIEMANN_HLLC,
                        implementation_version=0, precision=precision)
    lib = e2d.load_library()
    stream = torch.cuda.Stream()
    with e2d.HydroRun(p) as ref, e2d.HydroRun(p) as buf:
        # the existing entry point, called as serial_ref/main.f90 calls it
        ref.init_implode()
        ref.compute_dt(0)
        ref.make_boundaries(0)
        dt0 = ref.compute_dt(0)
        ref.godunov_unsplit(0, dt0)
        dt1 = ref.compute_dt(1)
        ref.godunov_unsplit(1, dt1)
        want1, want2 = ref.get_state(1), ref.get_state(0)

        # the no-allocation step on device arrays owned by another run
        buf.set_stream(stream.cuda_stream)
        buf.init_implode()
        pu, pu2 = ctypes.c_void_p(), ctypes.c_void_p()
        pitch = ctypes.c_size_t()
        assert lib.e2d_device_state(buf._h, 0, ctypes.byref(pu), ctypes.byref(pitch), None) == 0
        assert lib.e2d_device_state(buf._h, 1, ctypes.byref(pu2), None, None) == 0
        sp = ctypes.c_void_p(stream.cuda_stream)
        rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), pu, pu2, pitch.value, dt0, sp)
        assert rc == 0, lib.e2d_last_error().decode()
        got1 = buf.get_state(1)
        rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), pu2, pu, pitch.value, dt1, sp)
        assert rc == 0, lib.e2d_last_error().decode()
        got2 = buf.get_state(0)

    assert _rel_l1(got1, want1) <= REL_L1_TOL
    assert _rel_l1(got2, want2) <= REL_L1_TOL
    assert np.array_equal(_interior(got1), _interior(want1))
    assert np.array_equal(_interior(got2), _interior(want2))


def test_noalloc_rejects_grids_beyond_its_scratch(e2d):
    """4096^2 FP64 needs ~1.6 GB of work arrays: refused with a clear error,
    before any CUDA call (the pointers are never touched)."""
    lib = e2d.load_library()
    p = e2d.make_params(nx=4096, ny=4096, precision=8)
    fake_in, fake_out = ctypes.c_void_p(0x1000), ctypes.c_void_p(0x2000)
    rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), fake_in, fake_out, 4100, 1e-4, None)
    assert rc == e2d.E2D_ERR_INVALID_ARG
    assert b"too large" in lib.e2d_last_error()
