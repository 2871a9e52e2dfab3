"""The full-size cells of the 2048^2 / 4096^2 workload against the oracle, and
the multiply-add (FMA) build of the library against the oracle.

Workload (serial_ref/m_run.f90:187-243 driven by serial_ref/main.f90:66-76):
diagonal discontinuity, gamma 1.4, CFL 0.8, MC slopes, HLLC flux, reflective
walls, 100 steps, at 2048^2 and 4096^2, FP64 and FP32, implementationVersion
0 (fused) and 1 (stored primitives and face states).

* The exact build (no contraction) must give the oracle's bits in every cell
  and the oracle's dt sequence, FP64 against the FP64 oracle and FP32 against
  the FP32 oracle.
* The FMA build must stay within the specified bar against the FP64 oracle:
  relative L1 difference per conservative variable at most 1e-12, dt within
  1e-14 relative.
* Each FP32 build states its error against the FP64 oracle (bounded here by
  1e-5 relative L1 per variable and 1e-5 relative dt).

Oracle runs are shared between the tests of this file (one run per grid,
precision and step count).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1
FULL = NTHREADS >= 16          # 100 oracle steps at 4096^2 take ~15 s on 16 cores
REL_L1_TOL = 1e-12             # specification: relative L1 per conservative variable
DT_REL_TOL = 1e-14             # specification: dt relative
FP32_TOL = 1e-5                # FP32 against the FP64 oracle (measured ~3e-7)

_cache = {}


def interior(a):
    return a[:, 2:-2, 2:-2]


def rel_l1(a, b):
    a, b = interior(a).astype(np.float64), interior(b).astype(np.float64)
    return [float(np.abs(a[v] - b[v]).sum() / max(np.abs(b[v]).sum(), 1e-300)) for v in range(4)]


def dt_rel(d, dref):
    d, dref = np.asarray(d, np.float64), np.asarray(dref, np.float64)
    return float(np.max(np.abs(d - dref) / np.abs(dref)))


def steps_for(nx):
    return 100 if FULL else (10 if nx <= 2048 else 4)


def oracle_run(O, nx, prec, nsteps, riemann=2):
    key = (nx, prec, nsteps, riemann)
    if key not in _cache:
        po = O.Params(nx=nx, ny=nx, gamma0=1.4, cfl=0.8, riemann=riemann)
        ref, dts, _, _ = O.run(po, nsteps, prec="f64" if prec == 8 else "f32", nthreads=NTHREADS)
        _cache[key] = (ref, dts)  # ~1 GB in all: the 4096^2 FP64 state is 538 MB
    return _cache[key]


def gpu_run(E, nx, prec, version, nsteps, arith, riemann=2):
    p = E.make_params(nx=nx, ny=nx, gamma0=1.4, cfl=0.8, implementation_version=version, riemann_solver=riemann,
                      precision=prec)
    return E.run_steps(nsteps, p, arith=arith)


@pytest.mark.parametrize("nx,prec,version", [
    (2048, 8, 1),
    (4096, 8, 0), (4096, 8, 1),
    (2048, 4, 0), (2048, 4, 1),
    (4096, 4, 0), (4096, 4, 1),
], ids=lambda x: str(x))
def test_exact_build_bitwise_at_full_size(e2d, oracle, nx, prec, version):
    """Exact build: every interior cell and the dt sequence equal the
    oracle's bits (FP64 against the FP64 oracle, FP32 against the FP32
    oracle) after 100 steps."""
    n = steps_for(nx)
    ref, dts_ref = oracle_run(oracle, nx, prec, n)
    gpu, dts = gpu_run(e2d, nx, prec, version, n, "exact")
    assert np.array_equal(interior(gpu), interior(ref)), f"rel L1 {rel_l1(gpu, ref)}"
    assert np.array_equal(dts, dts_ref), f"dt relative difference {dt_rel(dts, dts_ref)}"


@pytest.mark.parametrize("nx", [2048, 4096])
@pytest.mark.parametrize("arith", ["exact", "fma"])
def test_fp32_error_against_fp64_oracle(e2d, oracle, nx, arith):
    """The FP32 build's error against the FP64 oracle after 100 steps:
    relative L1 per variable and the largest relative dt difference."""
    n = steps_for(nx)
    ref, dts_ref = oracle_run(oracle, nx, 8, n)
    gpu, dts = gpu_run(e2d, nx, 4, 0, n, arith)
    l1, dr = rel_l1(gpu, ref), dt_rel(dts, dts_ref)
    assert max(l1) < FP32_TOL and dr < FP32_TOL, f"FP32 {arith} vs FP64 oracle: rel L1 {l1}, dt {dr}"


@pytest.mark.parametrize("nx,version", [(2048, 0), (2048, 1), (4096, 0), (4096, 1)], ids=lambda x: str(x))
def test_fma_build_full_size_within_tolerance(e2d, oracle, nx, version):
    """FMA build, FP64, 100 steps: relative L1 per variable <= 1e-12 and dt
    within 1e-14 relative of the FP64 oracle."""
    n = steps_for(nx)
    ref, dts_ref = oracle_run(oracle, nx, 8, n)
    gpu, dts = gpu_run(e2d, nx, 8, version, n, "fma")
    l1, dr = rel_l1(gpu, ref), dt_rel(dts, dts_ref)
    assert max(l1) <= REL_L1_TOL, f"{nx}^2 v{version}: relative L1 per variable {l1}"
    assert dr <= DT_REL_TOL, f"{nx}^2 v{version}: dt relative difference {dr}"


@pytest.mark.parametrize("riemann", [2, 0], ids=["hllc", "approx"])
@pytest.mark.parametrize("version", [0, 1, 2])
def test_fma_build_plain_256_500_steps(e2d, oracle, riemann, version):
    """The plain-method case (256^2, FP64, 500 steps) with the FMA build,
    both Riemann solvers, every implementation version."""
    ref, dts_ref = oracle_run(oracle, 256, 8, 500, riemann)
    gpu, dts = gpu_run(e2d, 256, 8, version, 500, "fma", riemann)
    l1, dr = rel_l1(gpu, ref), dt_rel(dts, dts_ref)
    assert max(l1) <= REL_L1_TOL, f"v{version} riemann={riemann}: relative L1 per variable {l1}"
    assert dr <= DT_REL_TOL, f"v{version} riemann={riemann}: dt relative difference {dr}"


SMALL = [
    dict(nx=64, ny=64, nsteps=40, bc=(1, 1, 1, 1)),
    dict(nx=33, ny=17, nsteps=30, bc=(1, 1, 1, 1)),
    dict(nx=50, ny=30, nsteps=25, bc=(1, 2, 3, 1)),
    dict(nx=3, ny=200, nsteps=15, bc=(2, 1, 1, 3)),
]


@pytest.mark.parametrize("case", SMALL, ids=lambda c: f"{c['nx']}x{c['ny']}-bc{''.join(map(str, c['bc']))}")
@pytest.mark.parametrize("version", [0, 1, 2])
@pytest.mark.parametrize("riemann", [0, 2], ids=["approx", "hllc"])
@pytest.mark.parametrize("mode", ["advance", "percall"])
def test_fma_build_small_grids(e2d, oracle, case, version, riemann, mode):
    bc = case["bc"]
    pe = e2d.make_params(nx=case["nx"], ny=case["ny"], gamma0=1.4, cfl=0.8, implementation_version=version,
                         riemann_solver=riemann, boundary_type_xmin=bc[0], boundary_type_xmax=bc[1],
                         boundary_type_ymin=bc[2], boundary_type_ymax=bc[3])
    po = oracle.Params(nx=case["nx"], ny=case["ny"], gamma0=1.4, cfl=0.8, riemann=riemann, bc_xmin=bc[0],
                       bc_xmax=bc[1], bc_ymin=bc[2], bc_ymax=bc[3])
    ref, dts_ref, _, _ = oracle.run(po, case["nsteps"], nthreads=NTHREADS)
    gpu, dts = e2d.run_steps(case["nsteps"], pe, mode=mode, arith="fma")
    l1, dr = rel_l1(gpu, ref), dt_rel(dts, dts_ref)
    assert max(l1) <= REL_L1_TOL and dr <= DT_REL_TOL, f"rel L1 {l1}, dt {dr}"


def test_fma_build_reports_its_arithmetic(e2d):
    assert e2d.arithmetic("exact") == e2d.ARITH_EXACT
    assert e2d.arithmetic("fma") == e2d.ARITH_FMA


@pytest.mark.parametrize("mode", ["advance", "percall"])
@pytest.mark.parametrize("arith", ["exact", "fma"])
def test_carried_tiles_on_a_ragged_grid(e2d, oracle, arith, mode):
    """A grid with more tiles than the persistent grid has CTAs (1000 x 777:
    32 x 52 tiles of 32 x 15, the last row and column ragged), so that every
    CTA walks a run of tiles that crosses from one column of tiles to the
    next, and tiles take over the ring rows and y-face row of the tile below
    (the persistent kernel's carry); reflective and outflow walls in x,
    periodic in y.  The exact build
    must give the oracle's bits, the FMA build stay within the specified bar;
    both with the primitives kept (advance) and through the reference's
    per-call loop."""
    nx, ny, n = 1000, 777, 12
    bc = (1, 2, 3, 3)
    po = oracle.Params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann=2, bc_xmin=bc[0], bc_xmax=bc[1],
                       bc_ymin=bc[2], bc_ymax=bc[3])
    u0 = oracle.init_diagonal(po, 0.43, 1.0, 1.0, 0.125, float(np.float32(0.14)))
    ref, dts_ref, _, _ = oracle.run(po, n, u0=u0, nthreads=NTHREADS)
    p = e2d.make_params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann_solver=e2d.RIEMANN_HLLC,
                        boundary_type_xmin=bc[0], boundary_type_xmax=bc[1], boundary_type_ymin=bc[2],
                        boundary_type_ymax=bc[3])
    got, dts = e2d.run_steps(n, p, u0=u0, mode=mode, arith=arith)
    if arith == "exact":
        assert np.array_equal(interior(got), interior(ref))
        assert np.array_equal(np.asarray(dts), dts_ref)
    else:
        assert max(rel_l1(got, ref)) <= REL_L1_TOL
        assert dt_rel(dts, dts_ref) <= DT_REL_TOL
