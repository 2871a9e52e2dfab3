"""Parity of the CUDA step (through the C ABI) with the CPU oracle.

The oracle restates serial_ref; the library is built with -fmad=false and IEEE
division/square root, so the bar here is stricter than the 1e-12 relative L1
per conservative variable (and 1e-14 relative dt) of the specification: the
interior states and the dt sequences must be bitwise identical.  Where a case
differs, the assertion message reports the relative L1 difference.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1
REL_L1_TOL = 1e-12   # specification: relative L1 per conservative variable
DT_REL_TOL = 1e-14   # specification: dt relative


def interior(a):
    return a[:, 2:-2, 2:-2]


def rel_l1(a, b):
    a, b = interior(a).astype(np.float64), interior(b).astype(np.float64)
    return [float(np.abs(a[v] - b[v]).sum() / max(np.abs(b[v]).sum(), 1e-300)) for v in range(4)]


def assert_same(gpu, ref, dts_gpu, dts_ref, what):
    l1 = rel_l1(gpu, ref)
    assert max(l1) <= REL_L1_TOL, f"{what}: relative L1 per variable {l1}"
    dtr = np.max(np.abs(dts_gpu.astype(np.float64) - dts_ref) / np.abs(dts_ref)) if len(dts_ref) else 0.0
    assert dtr <= DT_REL_TOL, f"{what}: dt relative difference {dtr}"
    assert np.array_equal(interior(gpu), interior(ref)), f"{what}: not bitwise identical (rel L1 {l1})"
    assert np.array_equal(dts_gpu, dts_ref), f"{what}: dt sequence not bitwise identical"


SMALL = [
    dict(nx=64, ny=64, nsteps=40, bc=(1, 1, 1, 1)),
    dict(nx=33, ny=17, nsteps=30, bc=(1, 1, 1, 1)),
    dict(nx=48, ny=40, nsteps=30, bc=(2, 2, 2, 2)),
    dict(nx=40, ny=48, nsteps=31, bc=(3, 3, 3, 3)),
    dict(nx=50, ny=30, nsteps=25, bc=(1, 2, 3, 1)),
]


def _params(E, O, c, version, riemann, prec=8):
    bc = c["bc"]
    pe = E.make_params(nx=c["nx"], ny=c["ny"], gamma0=1.4, cfl=0.8, implementation_version=version,
                       riemann_solver=riemann, precision=prec, boundary_type_xmin=bc[0], boundary_type_xmax=bc[1],
                       boundary_type_ymin=bc[2], boundary_type_ymax=bc[3])
    po = O.Params(nx=c["nx"], ny=c["ny"], gamma0=1.4, cfl=0.8, riemann=riemann, bc_xmin=bc[0], bc_xmax=bc[1],
                  bc_ymin=bc[2], bc_ymax=bc[3])
    return pe, po


@pytest.mark.parametrize("case", SMALL, ids=lambda c: f"{c['nx']}x{c['ny']}-bc{''.join(map(str, c['bc']))}")
@pytest.mark.parametrize("version", [0, 1, 2])
@pytest.mark.parametrize("riemann", [0, 2], ids=["approx", "hllc"])
@pytest.mark.parametrize("mode", ["advance", "percall"])
def test_small_grids_bitwise(e2d, oracle, case, version, riemann, mode):
    pe, po = _params(e2d, oracle, case, version, riemann)
    ref, dts_ref, _, _ = oracle.run(po, case["nsteps"], nthreads=NTHREADS)
    gpu, dts = e2d.run_steps(case["nsteps"], pe, mode=mode)
    assert_same(gpu, ref, dts, dts_ref, f"v{version} riemann={riemann} {mode}")


TINY = [
    dict(nx=2, ny=2, nsteps=9, bc=(1, 1, 1, 1)),
    dict(nx=3, ny=2, nsteps=9, bc=(2, 3, 1, 2)),
    dict(nx=2, ny=5, nsteps=9, bc=(3, 3, 3, 3)),
    dict(nx=300, ny=3, nsteps=15, bc=(1, 2, 3, 1)),
    dict(nx=3, ny=200, nsteps=15, bc=(2, 1, 1, 3)),
]


@pytest.mark.parametrize("case", TINY, ids=lambda c: f"{c['nx']}x{c['ny']}-bc{''.join(map(str, c['bc']))}")
@pytest.mark.parametrize("version", [0, 1, 2])
@pytest.mark.parametrize("prec", [8, 4], ids=["f64", "f32"])
def test_minimal_and_skinny_grids_bitwise(e2d, oracle, case, version, prec):
    """The smallest grid the reference allows (one ghost source cell for
    several ghosts) and grids a few cells wide, where every tile is partial."""
    pe, po = _params(e2d, oracle, case, version, 2, prec)
    ref, dts_ref, _, _ = oracle.run(po, case["nsteps"], prec="f64" if prec == 8 else "f32", nthreads=NTHREADS)
    gpu, dts = e2d.run_steps(case["nsteps"], pe)
    assert_same(gpu, ref, dts, dts_ref, f"v{version} prec={prec}")


@pytest.mark.parametrize("riemann", [2, 0], ids=["hllc", "approx"])
def test_plain_256_500_steps(e2d, oracle, riemann):
    """The plain-method case: 256x256, FP64, gamma 1.4, CFL 0.8, MC slopes,
    reflective walls, 500 steps, diagonal discontinuity."""
    c = dict(nx=256, ny=256, bc=(1, 1, 1, 1))
    pe, po = _params(e2d, oracle, c, 0, riemann)
    ref, dts_ref, _, _ = oracle.run(po, 500, nthreads=NTHREADS)
    gpu, dts = e2d.run_steps(500, pe)
    assert_same(gpu, ref, dts, dts_ref, "256^2 x 500")


def test_percall_matches_reference_driver_including_ghosts(e2d, oracle):
    """compute_dt / godunov_unsplit called per step, as serial_ref/main.f90
    calls them: both arrays u and u2, ghosts and corners included, match."""
    c = dict(nx=40, ny=24, bc=(1, 2, 1, 3))
    pe, po = _params(e2d, oracle, c, 0, 0)
    _, dts_ref, u_ref, u2_ref = oracle.run(po, 13, nthreads=NTHREADS)
    with e2d.HydroRun(pe) as run:
        run.init_implode()
        run.compute_dt(0)
        run.make_boundaries(0)
        dts = []
        for n in range(13):
            dt = run.compute_dt(n % 2)
            run.godunov_unsplit(n, dt)
            dts.append(dt)
        assert np.array_equal(run.get_state(0), u_ref)
        assert np.array_equal(run.get_state(1), u2_ref)
        assert np.array_equal(np.array(dts), dts_ref)


def test_running_max_dt_across_calls(e2d, oracle):
    """compute_dt keeps the maximum of every invDt it has seen (the SAVEd
    invDt of serial_ref/m_run.f90:257): a calmer state does not raise dt."""
    c = dict(nx=32, ny=32, bc=(1, 1, 1, 1))
    pe, po = _params(e2d, oracle, c, 0, 0)
    u = oracle.init_implode(po)
    hot = u.copy()
    hot[2, 10, 10] = 50.0  # large momentum in one interior cell
    dt0, inv0 = oracle.compute_dt(po, u)
    dt1, inv1 = oracle.compute_dt(po, hot, inv0)
    dt2, inv2 = oracle.compute_dt(po, u, inv1)
    assert dt1 < dt0 and dt2 == dt1
    with e2d.HydroRun(pe) as run:
        run.set_state(0, u)
        run.set_state(1, hot)
        assert run.compute_dt(0) == dt0
        assert run.compute_dt(1) == dt1
        assert run.compute_dt(0) == dt2
        assert run.invdt() == inv2


def test_dt_excludes_last_interior_row_and_column(e2d, oracle):
    c = dict(nx=32, ny=32, bc=(1, 1, 1, 1))
    pe, po = _params(e2d, oracle, c, 0, 0)
    u = oracle.init_implode(po)
    last = u.copy()
    last[2, 20, c["nx"] + 1] = 80.0   # last interior column: ignored by compute_dt
    first = u.copy()
    first[2, 20, 2] = 80.0            # first interior column: counted
    with e2d.HydroRun(pe) as run:
        run.set_state(0, last)
        d_last = run.compute_dt(0)
    with e2d.HydroRun(pe) as run:
        run.set_state(0, first)
        d_first = run.compute_dt(0)
    assert d_last == oracle.compute_dt(po, last)[0] == oracle.compute_dt(po, u)[0]
    assert d_first == oracle.compute_dt(po, first)[0] < d_last


@pytest.mark.parametrize("version", [0, 2])
def test_fp32_build(e2d, oracle, version):
    """FP32 (fp_kind = sp_kind): bitwise against the FP32 oracle; its error
    against the FP64 oracle is reported in the assertion message bound."""
    c = dict(nx=96, ny=96, bc=(1, 1, 1, 1))
    pe, po = _params(e2d, oracle, c, version, 2, prec=4)
    ref32, dts32, _, _ = oracle.run(po, 100, prec="f32", nthreads=NTHREADS)
    gpu, dts = e2d.run_steps(100, pe)
    assert gpu.dtype == np.float32
    assert np.array_equal(interior(gpu), interior(ref32))
    assert np.array_equal(dts, dts32)
    ref64, _, _, _ = oracle.run(po, 100, prec="f64", nthreads=NTHREADS)
    err = rel_l1(gpu, ref64)
    assert max(err) < 1e-3, f"FP32 vs FP64 relative L1 {err}"


def test_full_size_2048_matches_oracle(e2d, oracle):
    """2048^2, FP64, HLLC, implementationVersion 0: 100 steps against the
    multicore oracle (bitwise), plus the exact x<->y symmetry of the problem."""
    c = dict(nx=2048, ny=2048, bc=(1, 1, 1, 1))
    pe, po = _params(e2d, oracle, c, 0, 2)
    n = 100 if NTHREADS >= 16 else 10
    ref, dts_ref, _, _ = oracle.run(po, n, nthreads=NTHREADS)
    gpu, dts = e2d.run_steps(n, pe)
    assert_same(gpu, ref, dts, dts_ref, "2048^2")
    rho = interior(gpu)[0]
    assert np.array_equal(rho, rho.T)
    assert np.array_equal(interior(gpu)[2], interior(gpu)[3].T)


def test_health_flags_clean_run(e2d):
    with e2d.HydroRun(nx=64, ny=64, gamma0=1.4) as run:
        run.init_implode()
        run.advance(0, 20)
        assert run.health() == 0


def test_health_flags_negative_density(e2d):
    """A state with a negative conservative density is computed (the
    reference floors it) and flagged."""
    with e2d.HydroRun(nx=32, ny=32, gamma0=1.4) as run:
        u = run.new_state()
        u[0] = 1.0
        u[1] = 2.5
        u[0, 10:12, 10:12] = -1.0
        run.set_state(0, u)
        run.advance(0, 1)
        assert run.health() & e2d.HEALTH_NEG_DENSITY


SCHEMES = [
    dict(slope_type=0, riemann=2),                          # first order (zero slopes)
    dict(slope_type=0, riemann=0),
    dict(slope_type=1, riemann=0),                          # minmod
    dict(niter_riemann=0, riemann=0),                       # two-shock solver without Newton iterations
    dict(niter_riemann=1, riemann=0),
    dict(gamma0=5.0 / 3.0, cfl=0.5, riemann=2),
    dict(gamma0=5.0 / 3.0, cfl=0.5, riemann=0),
    dict(smallr=1e-3, smallc=1e-2, riemann=2),              # floors that bite in the low state
    dict(smallr=1e-3, smallc=1e-2, riemann=0),
]


@pytest.mark.parametrize("scheme", SCHEMES, ids=lambda d: "-".join(f"{k}{v:.4g}" if isinstance(v, float) else
                                                                  f"{k}{v}" for k, v in d.items()))
@pytest.mark.parametrize("version", [0, 1, 2])
@pytest.mark.parametrize("prec", [8, 4], ids=["f64", "f32"])
def test_scheme_parameters_bitwise(e2d, oracle, scheme, version, prec):
    """Every &HYDRO parameter the step reads: slope_type, niter_riemann,
    gamma0, cfl, smallr, smallc, with both Riemann solvers."""
    kw = dict(scheme)
    riemann = kw.pop("riemann")
    nx, ny, n = 64, 48, 20
    pe = e2d.make_params(nx=nx, ny=ny, implementation_version=version, riemann_solver=riemann, precision=prec,
                         boundary_type_xmin=1, boundary_type_xmax=2, boundary_type_ymin=3, boundary_type_ymax=3,
                         **{"gamma0": 1.4, "cfl": 0.8, **kw})
    po = oracle.Params(nx=nx, ny=ny, riemann=riemann, bc_xmin=1, bc_xmax=2, bc_ymin=3, bc_ymax=3,
                       **{"gamma0": 1.4, "cfl": 0.8, **kw})
    ref, dts_ref, _, _ = oracle.run(po, n, prec="f64" if prec == 8 else "f32", nthreads=NTHREADS)
    gpu, dts = e2d.run_steps(n, pe)
    assert_same(gpu, ref, dts, dts_ref, f"{scheme} v{version} prec={prec}")
