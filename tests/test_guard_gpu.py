"""Guard bands: out-of-bounds writes show up as changed padding.

compute-sanitizer is closed on the GPU pool, so bounds are also checked this
way.  A state is stored with rows padded from isize to a pitch that is a
multiple of 32 elements; the padding of u and u2 is filled with a sentinel
bit pattern (a signalling NaN) before the steps.  After steps of every
implementation version, both arithmetic builds and both precisions --
through e2d_advance (graphs) and through the per-call sequence -- every
padding word must still hold the sentinel (no kernel wrote past the end of
a row) and no health flag may be raised (no kernel read it into a result).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SENTINEL64 = np.uint64(0x7FF4DEADBEEF0001)  # a signalling-NaN pattern no step computes
SENTINEL32 = np.uint32(0x7FA0BEEF)


def _state_view(torch, run, which):
    """A torch view (no copy) of state `which` of the run on the device, as
    raw words of the element size: (4 planes, rows, pitch)."""
    ptr, pitch, plane = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.c_size_t()
    assert run._lib.e2d_device_state(run._h, which, ctypes.byref(ptr), ctypes.byref(pitch),
                                     ctypes.byref(plane)) == 0
    wide = run.params.precision == 8

    class _Device:
        __cuda_array_interface__ = {"shape": (4 * plane.value,), "typestr": "<i8" if wide else "<i4",
                                    "data": (ptr.value, False), "version": 3}

    t = torch.as_tensor(_Device(), device="cuda")
    return t.view(4, plane.value // pitch.value, pitch.value), pitch.value


@pytest.mark.parametrize("arith", ["exact", "fma"])
@pytest.mark.parametrize("prec", [8, 4], ids=["f64", "f32"])
@pytest.mark.parametrize("version", [0, 1, 2])
@pytest.mark.parametrize("mode", ["advance", "percall"])
def test_row_padding_is_never_written(e2d, arith, prec, version, mode):
    torch = pytest.importorskip("torch")
    nx, ny = 70, 45  # isize 74: rows padded to 96 elements
    p = e2d.make_params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann_solver=e2d.RIEMANN_HLLC, precision=prec,
                        implementation_version=version, boundary_type_xmax=2, boundary_type_ymin=3)
    sentinel = int(SENTINEL64.view(np.int64)) if prec == 8 else int(SENTINEL32.view(np.int32))
    with e2d.HydroRun(p, arith=arith) as run:
        run.init_implode()
        views = []
        for which in (0, 1):
            v, pitch = _state_view(torch, run, which)
            assert pitch > run.isize
            v[:, :, run.isize:] = sentinel
            views.append(v)
        torch.cuda.synchronize()
        if mode == "advance":
            run.advance(0, 9)
        else:
            run.compute_dt(0)
            run.make_boundaries(0)
            for n in range(9):
                run.godunov_unsplit(n, run.compute_dt(n % 2))
        run.synchronize()
        for v in views:
            pad = v[:, :, run.isize:]
            assert bool((pad == sentinel).all()), "a kernel wrote into the row padding"
        assert run.health() == 0
