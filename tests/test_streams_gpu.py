"""Where the work runs: on a stream the caller owns (e2d_set_stream), and
step by step with per-step events (e2d_time_steps, the path the benchmark's
roofline times).  Both must leave bit for bit the states and running CFL
maximum of the library's default path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(E, version=0, prec=8):
    return E.make_params(nx=96, ny=80, gamma0=1.4, cfl=0.8, riemann_solver=E.RIEMANN_HLLC,
                         implementation_version=version, precision=prec, boundary_type_xmax=2, boundary_type_ymin=3,
                         boundary_type_ymax=3)


@pytest.mark.parametrize("version", [0, 1, 2])
def test_caller_stream_gives_the_same_states(e2d, version):
    torch = pytest.importorskip("torch")
    p = _params(e2d, version)
    with e2d.HydroRun(p) as a:
        a.init_implode()
        da = a.advance(0, 12)
        a.make_boundaries(0)
        ua = a.final_state(12)
    s = torch.cuda.Stream()
    with e2d.HydroRun(p) as b:
        b.set_stream(s.cuda_stream)
        b.init_implode()
        db = b.advance(0, 7)  # graph captured on the caller's stream
        for n in range(7, 12):  # then the reference's per-call loop on it
            db = np.append(db, b.compute_dt(n % 2))
            b.godunov_unsplit(n, db[-1])
        # The per-call steps leave the ghosts of their output to the next
        # make_boundaries (serial_ref/m_run.f90:224); the fused advance writes them in
        # the update: fill them on both runs before comparing whole arrays.
        b.make_boundaries(0)
        s.synchronize()
        ub = b.final_state(12)
        b.set_stream(None)
    assert np.array_equal(ua, ub)
    assert np.array_equal(da, db)


@pytest.mark.parametrize("prec", [8, 4], ids=["f64", "f32"])
def test_time_steps_leaves_the_advance_state(e2d, prec):
    p = _params(e2d, 0, prec)
    with e2d.HydroRun(p) as a:
        a.init_implode()
        a.advance(0, 3)
        a.advance(3, 9)
        ua, inv_a = a.final_state(12), a.invdt()
    with e2d.HydroRun(p) as b:
        b.init_implode()
        b.advance(0, 3)
        ms = b.time_steps(3, 9)
        ub, inv_b = b.final_state(12), b.invdt()
        assert np.all(ms > 0)
        b.advance(12, 2)  # carries on from the timed steps
        assert b.health() == 0
    assert np.array_equal(ua, ub)
    assert inv_a == inv_b


@pytest.mark.parametrize("prec", [8, 4], ids=["f64", "f32"])
def test_percall_steps_see_an_uploaded_state(e2d, prec):
    """The per-call step keeps the primitives of its states between calls; a
    state written from the host in between must be the one the next step
    reads (same bits as a run that starts from it)."""
    p = _params(e2d, 0, prec)
    dt = 2e-4
    with e2d.HydroRun(p) as a:
        a.init_implode()
        for n in range(5):
            a.godunov_unsplit(n, dt)
        mid = a.get_state(1)
        mid[0, 2:-2, 2:-2] *= 1.01
        a.set_state(1, mid)
        a.make_boundaries(1)
        for n in range(5, 10):
            a.godunov_unsplit(n, dt)
        a.make_boundaries(0)
        ua = a.get_state(0)
    with e2d.HydroRun(p) as b:
        b.init_implode()
        b.set_state(1, mid)
        b.make_boundaries(1)
        for n in range(5, 10):
            b.godunov_unsplit(n, dt)
        b.make_boundaries(0)
        ub = b.get_state(0)
    assert np.array_equal(ua, ub)


@pytest.mark.parametrize("size", [(96, 80), (700, 610)], ids=["96x80", "700x610-carried"])
@pytest.mark.parametrize("prec", [8, 4], ids=["f64", "f32"])
def test_kept_primitives_change_no_bit(e2d, monkeypatch, prec, size):
    """implementationVersion 0 keeps the primitives of its states beside them
    (each step writes its output's); with E2D_KEEP_PRIMS=0 every step
    converts its box instead.  Both give the same states and dt -- at 700 x
    610 also with the persistent kernel's carried ring rows (902 tiles), on
    primitive and on conservative boxes."""
    nx, ny = size
    p = e2d.make_params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann_solver=e2d.RIEMANN_HLLC, precision=prec,
                        boundary_type_xmax=2, boundary_type_ymin=3, boundary_type_ymax=3)
    runs = []
    for keep in ("1", "0"):
        monkeypatch.setenv("E2D_KEEP_PRIMS", keep)
        with e2d.HydroRun(p) as r:
            r.init_implode()
            dts = r.advance(0, 9)
            for n in range(9, 13):
                dts = np.append(dts, r.compute_dt(n % 2))
                r.godunov_unsplit(n, dts[-1])
            r.make_boundaries(1)
            runs.append((r.get_state(1), dts))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])


@pytest.mark.parametrize("prec", [8, 4], ids=["f64", "f32"])
@pytest.mark.parametrize("nx", [96, 33], ids=["even", "odd"])
def test_pinned_host_arrays_copy_like_pageable_ones(e2d, prec, nx):
    """Upload and download through pinned (mapped) host memory, which the
    library copies with a kernel reading or writing the host rows directly,
    move the same bytes as through pageable memory (the 2D copy), for even
    and odd row lengths; rows of a pinned array past the state are left
    alone."""
    torch = pytest.importorskip("torch")
    p = e2d.make_params(nx=nx, ny=40, gamma0=1.4, cfl=0.8, riemann_solver=e2d.RIEMANN_HLLC, precision=prec)
    dt = np.float64 if prec == 8 else np.float32
    rng = np.random.default_rng(5)
    with e2d.HydroRun(p) as run:
        shape = (4, run.jsize, run.isize)
        src = rng.uniform(0.5, 2.0, size=shape).astype(dt)
        pinned = torch.empty(int(np.prod(shape)) + 64, dtype=torch.float64 if prec == 8 else torch.float32,
                             pin_memory=True).numpy()
        pinned[:] = -3.0
        pin_state = pinned[: np.prod(shape)].reshape(shape)
        pin_state[...] = src
        run.set_state(0, pin_state)          # pinned upload
        run.set_state(1, src)                # pageable upload
        a = run.get_state(0)                 # pageable download
        pin_state[...] = 0.0
        run.get_state(1, out=pin_state)      # pinned download
        assert np.array_equal(a, src)
        assert np.array_equal(pin_state, src)
        assert np.all(pinned[np.prod(shape):] == -3.0)
