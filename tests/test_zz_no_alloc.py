"""The Godunov step that allocates no device memory.

e2d_godunov_unsplit_noalloc serves callers that cannot call cudaMalloc: host
codes whose device arrays come from another allocator or memory pool, and
frameworks that hand the time step only its input and output arrays and
forbid allocation on that path.  Its work arrays live in one static device
array of E2D_NOALLOC_SCRATCH_BYTES shared by every call.  These tests check
that two calls in a row (the second reusing whatever the first left in the
static array) give the same states as the regular per-call step
e2d_godunov_unsplit -- on the library's own arrays and on arrays the caller
allocated with a wider row pitch --, that the output's ghost cells are left
alone, that the numerical health flags reach the caller, and that bad
arguments (grids too large for the static array, a bad dt, overlapping
arrays, a pitch beyond INT_MAX) are refused before any device work.
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
@pytest.mark.parametrize("arith", ["exact", "fma"])
@pytest.mark.parametrize("precision", [8, 4])
def test_noalloc_step_matches_regular_step_two_calls(e2d, precision, arith):
    torch = pytest.importorskip("torch")
    p = e2d.make_params(nx=96, ny=80, gamma0=1.4, cfl=0.8, riemann_solver=e2d.RIEMANN_HLLC,
                        implementation_version=0, precision=precision)
    lib = e2d.load_library(arith)
    stream = torch.cuda.Stream()
    with e2d.HydroRun(p, arith=arith) as ref, e2d.HydroRun(p, arith=arith) as buf:
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
        rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), pu, pu2, pitch.value, dt0, sp, None)
        assert rc == 0, lib.e2d_last_error().decode()
        got1 = buf.get_state(1)
        rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), pu2, pu, pitch.value, dt1, sp, None)
        assert rc == 0, lib.e2d_last_error().decode()
        got2 = buf.get_state(0)

    # the exact build: bitwise; the FMA build's two paths (fused step, stored
    # fluxes) round differently: the FP64 bar of the other tests, and 1e-5 in FP32
    tol = REL_L1_TOL if (arith == "exact" or precision == 8) else 1e-5
    assert _rel_l1(got1, want1) <= tol
    assert _rel_l1(got2, want2) <= tol
    if arith == "exact":
        assert np.array_equal(_interior(got1), _interior(want1))
        assert np.array_equal(_interior(got2), _interior(want2))


def test_noalloc_rejects_grids_beyond_its_scratch(e2d):
    """4096^2 FP64 needs ~1.6 GB of work arrays: refused with a clear error,
    before any CUDA call (the pointers are never touched)."""
    lib = e2d.load_library()
    p = e2d.make_params(nx=4096, ny=4096, precision=8)
    fake_in, fake_out = ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1000 + 2 ** 40)
    rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), fake_in, fake_out, 4100, 1e-4, None, None)
    assert rc == e2d.E2D_ERR_INVALID_ARG
    assert b"too large" in lib.e2d_last_error()


@pytest.mark.parametrize("dt", [0.0, -1e-4, float("nan"), float("inf")])
def test_noalloc_rejects_a_bad_dt(e2d, dt):
    lib = e2d.load_library()
    p = e2d.make_params(nx=64, ny=64, precision=8)
    rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), ctypes.c_void_p(0x100000), ctypes.c_void_p(0x10000000),
                                         68, dt, None, None)
    assert rc == e2d.E2D_ERR_INVALID_ARG
    assert b"dt" in lib.e2d_last_error()


def test_noalloc_rejects_overlapping_or_oversized_layouts(e2d):
    """Overlapping state arrays and a pitch beyond INT_MAX are refused (fake
    pointers: nothing is dereferenced)."""
    lib = e2d.load_library()
    p = e2d.make_params(nx=64, ny=64, precision=8)
    state_bytes = 4 * 68 * 68 * 8
    base = 0x10000000
    for off in (0, 8, state_bytes - 8):
        rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), ctypes.c_void_p(base), ctypes.c_void_p(base + off),
                                             68, 1e-4, None, None)
        assert rc == e2d.E2D_ERR_INVALID_ARG, off
        assert b"overlap" in lib.e2d_last_error() or b"null" in lib.e2d_last_error()
    rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), ctypes.c_void_p(base), ctypes.c_void_p(base + 2 ** 40),
                                         2 ** 31, 1e-4, None, None)
    assert rc == e2d.E2D_ERR_INVALID_ARG
    assert b"INT_MAX" in lib.e2d_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny,extra", [(70, 52, 13), (700, 610, 5)], ids=["70x52", "700x610-carried"])
def test_noalloc_on_caller_arrays_with_a_wider_pitch(e2d, nx, ny, extra):
    """Arrays the caller allocated (torch) with a row pitch wider than nx+4:
    two calls give the regular step's interiors bit for bit, and the output's
    ghost cells keep what the caller put there.  At 700 x 610 the regular
    (fused) step it is compared with walks runs of its 902 tiles with the
    carried ring rows, while this step stores fluxes: two independent
    formulations of the same arithmetic."""
    torch = pytest.importorskip("torch")
    p = e2d.make_params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann_solver=e2d.RIEMANN_HLLC, precision=8)
    lib = e2d.load_library()
    with e2d.HydroRun(p) as ref:
        ref.init_implode()
        u0 = ref.get_state(0)
        ref.compute_dt(0)
        ref.make_boundaries(0)
        dt0 = ref.compute_dt(0)
        ref.godunov_unsplit(0, dt0)
        dt1 = ref.compute_dt(1)
        ref.godunov_unsplit(1, dt1)
        want1, want2 = ref.get_state(1), ref.get_state(0)
    pitch = nx + 4 + extra
    a = torch.full((4, ny + 4, pitch), -7.0, dtype=torch.float64, device="cuda")
    b = torch.full((4, ny + 4, pitch), -7.0, dtype=torch.float64, device="cuda")
    a[:, :, :nx + 4] = torch.from_numpy(u0).cuda()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    flags = ctypes.c_uint(99)
    rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), ctypes.c_void_p(a.data_ptr()),
                                         ctypes.c_void_p(b.data_ptr()), pitch, dt0, ctypes.c_void_p(stream),
                                         ctypes.byref(flags))
    assert rc == 0, lib.e2d_last_error().decode()
    assert flags.value == 0
    got1 = b[:, :, :nx + 4].cpu().numpy()
    ghosts = b.clone()
    ghosts[:, 2:-2, 2:nx + 2] = -7.0
    assert bool((ghosts == -7.0).all()), "the output's ghost cells and row padding must be left alone"
    rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), ctypes.c_void_p(b.data_ptr()),
                                         ctypes.c_void_p(a.data_ptr()), pitch, dt1, ctypes.c_void_p(stream), None)
    assert rc == 0, lib.e2d_last_error().decode()
    torch.cuda.synchronize()
    got2 = a[:, :, :nx + 4].cpu().numpy()
    assert np.array_equal(_interior(got1), _interior(want1))
    assert np.array_equal(_interior(got2), _interior(want2))


@pytest.mark.gpu
def test_noalloc_reports_a_negative_density(e2d):
    """A state with a negative density is stepped (the reference floors it)
    and the health flag reaches the caller through `health`; the next clean
    call reports no flag (the word is cleared per call)."""
    torch = pytest.importorskip("torch")
    nx = ny = 32
    p = e2d.make_params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, precision=8)
    lib = e2d.load_library()
    u = np.zeros((4, ny + 4, nx + 4))
    u[0] = 1.0
    u[1] = 2.5
    bad = u.copy()
    bad[0, 10:12, 10:12] = -1.0
    a = torch.from_numpy(bad).cuda()
    b = torch.zeros_like(a)
    flags = ctypes.c_uint(0)
    rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), ctypes.c_void_p(a.data_ptr()),
                                         ctypes.c_void_p(b.data_ptr()), nx + 4, 1e-3, None, ctypes.byref(flags))
    assert rc == 0, lib.e2d_last_error().decode()
    assert flags.value & e2d.HEALTH_NEG_DENSITY
    a.copy_(torch.from_numpy(u))
    rc = lib.e2d_godunov_unsplit_noalloc(ctypes.byref(p), ctypes.c_void_p(a.data_ptr()),
                                         ctypes.c_void_p(b.data_ptr()), nx + 4, 1e-3, None, ctypes.byref(flags))
    assert rc == 0, lib.e2d_last_error().decode()
    assert flags.value == 0
