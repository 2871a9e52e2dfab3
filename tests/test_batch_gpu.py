"""The batched ensemble: every problem of a batch is bitwise identical to the
same problem advanced alone (states and dt sequence), whatever the schedule."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(40, 40), (130, 96), (64, 33), (17, 80), (96, 96), (200, 24)]
BCS = [[1, 1, 1, 1], [2, 2, 2, 2], [1, 2, 3, 1], [3, 3, 3, 3], [2, 1, 1, 2], [1, 1, 2, 2]]
OFFSET = [0.5, 0.3, 0.7, 0.45, 0.62, 0.38]
RHO_HI = [1.0, 0.2, 0.9, 0.5, 0.1, 0.7]
P_HI = [1.0, 0.3, 0.15, 0.8, 0.4, 0.9]
RHO_LO = [0.125, 0.9, 0.1, 0.35, 0.6, 0.25]
P_LO = [float(np.float32(0.14)), 0.1, 0.95, 0.2, 0.5, 0.33]


def single_run(E, k, nsteps, prec, riemann):
    bc = BCS[k]
    p = E.make_params(nx=SIZES[k][0], ny=SIZES[k][1], gamma0=1.4, cfl=0.8, riemann_solver=riemann,
                      precision=prec, boundary_type_xmin=bc[0], boundary_type_xmax=bc[1],
                      boundary_type_ymin=bc[2], boundary_type_ymax=bc[3])
    with E.HydroRun(p) as run:
        run.init_diagonal(OFFSET[k], RHO_HI[k], P_HI[k], RHO_LO[k], P_LO[k])
        dts = run.advance(0, nsteps)
        return run.final_state(nsteps), dts


def make_batch(E, prec, riemann):
    b = E.Batch(SIZES, BCS, gamma0=1.4, cfl=0.8, riemann_solver=riemann, precision=prec)
    b.init_diagonal(OFFSET, RHO_HI, P_HI, RHO_LO, P_LO)
    return b


@pytest.mark.parametrize("schedule", [(0, 1, 0), (0, 2, 1), (1, 1, 1), (1, 4, 0), (0, 0, 1)],
                         ids=["32x15-x1-order", "32x15-x2-lpt", "32x7-x1-lpt", "32x7-x4-order", "32x15-pertile-lpt"])
@pytest.mark.parametrize("riemann", [2, 0], ids=["hllc", "approx"])
def test_batch_equals_single_runs(e2d, schedule, riemann):
    n = 25
    with make_batch(e2d, 8, riemann) as b:
        b.set_schedule(*schedule)
        dts = b.advance(0, n)
        for k in range(len(SIZES)):
            ref, ref_dts = single_run(e2d, k, n, 8, riemann)
            got = b.final_state(k, n)
            assert np.array_equal(got[:, 2:-2, 2:-2], ref[:, 2:-2, 2:-2]), f"problem {k}"
            assert np.array_equal(dts[:, k], ref_dts), f"problem {k} dt"
            assert b.health(k) == 0


def test_batch_fp32_equals_single_runs(e2d):
    n = 20
    with make_batch(e2d, 4, 2) as b:
        b.advance(0, 7)
        b.advance(7, n - 7)  # two calls: running maxima and ping-pong carry over
        for k in range(len(SIZES)):
            ref, _ = single_run(e2d, k, n, 4, 2)
            assert np.array_equal(b.final_state(k, n)[:, 2:-2, 2:-2], ref[:, 2:-2, 2:-2])


def test_autotuner_restores_states_and_reuses_cache(e2d, tmp_path):
    cache = str(tmp_path / "tune.txt")
    with make_batch(e2d, 8, 2) as b:
        before = [b.get_state(k, 0) for k in range(len(SIZES))]
        ms = b.tune(steps=2, cache_path=cache)
        assert ms > 0
        for k in range(len(SIZES)):
            assert np.array_equal(b.get_state(k, 0), before[k])
        chosen = b.schedule()
        # the tuned batch still matches the single runs
        b.advance(0, 10)
        ref, _ = single_run(e2d, 1, 10, 8, 2)
        assert np.array_equal(b.final_state(1, 10)[:, 2:-2, 2:-2], ref[:, 2:-2, 2:-2])
    with make_batch(e2d, 8, 2) as b2:
        b2.tune(steps=2, cache_path=cache)  # answered from the cache
        assert b2.schedule()["variant"] == chosen["variant"]
        assert b2.schedule()["grid_mult"] == chosen["grid_mult"]


def test_seeded_ensemble_first_steps(e2d):
    """The 64-problem seeded ensemble: a few steps, compared with single runs
    for a handful of its problems."""
    from euler2d_cudafortran_gb300.ensemble import diagonal_ensemble
    ens = diagonal_ensemble()
    with e2d.Batch(ens.sizes, ens.bcs, gamma0=1.4, cfl=0.8, riemann_solver=2) as b:
        b.init_diagonal(ens.offset, ens.rho_hi, ens.p_hi, ens.rho_lo, ens.p_lo)
        dts = b.advance(0, 4)
        for k in (0, 17, 63):
            bc = ens.bcs[k]
            p = e2d.make_params(nx=ens.sizes[k][0], ny=ens.sizes[k][1], gamma0=1.4, cfl=0.8, riemann_solver=2,
                                boundary_type_xmin=bc[0], boundary_type_xmax=bc[1], boundary_type_ymin=bc[2],
                                boundary_type_ymax=bc[3])
            with e2d.HydroRun(p) as run:
                run.init_diagonal(ens.offset[k], ens.rho_hi[k], ens.p_hi[k], ens.rho_lo[k], ens.p_lo[k])
                rdts = run.advance(0, 4)
                assert np.array_equal(b.final_state(k, 4)[:, 2:-2, 2:-2], run.final_state(4)[:, 2:-2, 2:-2])
                assert np.array_equal(dts[:, k], rdts)


@pytest.mark.parametrize("prec", [8, 4], ids=["f64", "f32"])
def test_fma_batch_matches_the_oracle(e2d, oracle, prec):
    """The FMA build's ensemble step against the oracle, problem by problem:
    FP64 within the specified 1e-12 relative L1 per variable and 1e-14
    relative dt; FP32 within 1e-5 of the FP32 oracle (rounding differences of
    the fused multiply-adds)."""
    n = 25
    l1_tol, dt_tol = (1e-12, 1e-14) if prec == 8 else (1e-5, 1e-5)
    with e2d.Batch(SIZES, BCS, gamma0=1.4, cfl=0.8, riemann_solver=2, precision=prec, arith="fma") as b:
        b.init_diagonal(OFFSET, RHO_HI, P_HI, RHO_LO, P_LO)
        dts = b.advance(0, n)
        for k, ((nx, ny), bc) in enumerate(zip(SIZES, BCS)):
            po = oracle.Params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann=2, bc_xmin=bc[0], bc_xmax=bc[1],
                               bc_ymin=bc[2], bc_ymax=bc[3])
            u0 = oracle.init_diagonal(po, OFFSET[k], RHO_HI[k], P_HI[k], RHO_LO[k], P_LO[k],
                                      prec="f64" if prec == 8 else "f32")
            ref, dts_ref, _, _ = oracle.run(po, n, prec="f64" if prec == 8 else "f32", u0=u0)
            got = b.final_state(k, n)[:, 2:-2, 2:-2].astype(np.float64)
            want = ref[:, 2:-2, 2:-2].astype(np.float64)
            l1 = [float(np.abs(got[v] - want[v]).sum() / np.abs(want[v]).sum()) for v in range(4)]
            dr = float(np.max(np.abs(dts[:, k].astype(np.float64) - dts_ref) / dts_ref))
            assert max(l1) <= l1_tol and dr <= dt_tol, f"problem {k}: rel L1 {l1}, dt {dr}"
            assert b.health(k) == 0


@pytest.mark.parametrize("schedule", [(0, 1, 0), (1, 2, 1)], ids=["32x15-x1-order", "32x7-x2-lpt"])
def test_carried_runs_across_problems_match_the_oracle(e2d, oracle, schedule):
    """An ensemble with many more tiles than CTAs (2244 tiles of 32 x 15 over
    the persistent grid), so that each CTA walks a run of tiles up the
    columns of a problem and on into the next problem, the tiles taking over
    the ring rows and y-face row of the tile below: each problem bitwise
    equal to the oracle (states and dt), exact build."""
    sizes = [(1000, 777), (333, 600), (640, 96)]
    bcs = [[1, 2, 3, 3], [2, 2, 1, 1], [3, 3, 2, 1]]
    init = ([0.43, 0.6, 0.5], [1.0, 0.3, 0.8], [1.0, 0.9, 0.4], [0.125, 0.7, 0.2],
            [float(np.float32(0.14)), 0.2, 0.6])
    n = 8
    with e2d.Batch(sizes, bcs, gamma0=1.4, cfl=0.8, riemann_solver=2) as b:
        b.set_schedule(*schedule)
        b.init_diagonal(*init)
        dts = b.advance(0, n)
        for k, ((nx, ny), bc) in enumerate(zip(sizes, bcs)):
            po = oracle.Params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann=2, bc_xmin=bc[0], bc_xmax=bc[1],
                               bc_ymin=bc[2], bc_ymax=bc[3])
            u0 = oracle.init_diagonal(po, *(x[k] for x in init))
            ref, dts_ref, _, _ = oracle.run(po, n, u0=u0, nthreads=os.cpu_count() or 1)
            assert np.array_equal(b.final_state(k, n)[:, 2:-2, 2:-2], ref[:, 2:-2, 2:-2]), f"problem {k}"
            assert np.array_equal(dts[:, k], dts_ref), f"problem {k}"
            assert b.health(k) == 0
