"""Seeded random sweeps against the oracle.

Thirty configurations drawn from one seed: grid sides from 2 to 200 in each
direction, the wall type of every face (reflective, outflow, periodic), a
diagonal initial state with random offset, densities and pressures, and
random scheme parameters (Riemann solver, slope type, gamma, CFL, Newton
iterations).  Every implementation version must reproduce the oracle's
states and dt sequence bit for bit.  Eight more configurations check the
adjoint gradient against the oracle's forward-mode tangent."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1


def draw(rng):
    nx, ny = (int(rng.choice([rng.integers(2, 9), rng.integers(9, 201)])) for _ in range(2))
    bc = [int(x) for x in rng.integers(1, 4, 4)]
    c = dict(nx=nx, ny=ny, bc=bc, riemann=int(rng.choice([0, 2])), slope_type=int(rng.choice([0, 1, 2, 2])),
             gamma0=float(rng.choice([1.4, 5.0 / 3.0, 1.3])), cfl=float(rng.choice([0.8, 0.5, 0.3])),
             niter_riemann=int(rng.choice([10, 10, 3, 0])), offset=float(rng.uniform(0.2, 0.8)),
             rho_hi=float(10 ** rng.uniform(-1, 0)), p_hi=float(10 ** rng.uniform(-1, 0)),
             rho_lo=float(10 ** rng.uniform(-1, 0)), p_lo=float(10 ** rng.uniform(-1, 0)),
             nsteps=int(rng.integers(3, 16)))
    return c


CASES = [draw(np.random.default_rng(20261203 + k)) for k in range(30)]


def _params(E, O, c, version, prec=8):
    bc = c["bc"]
    pe = E.make_params(nx=c["nx"], ny=c["ny"], gamma0=c["gamma0"], cfl=c["cfl"], niter_riemann=c["niter_riemann"],
                       slope_type=c["slope_type"], implementation_version=version, riemann_solver=c["riemann"],
                       precision=prec, boundary_type_xmin=bc[0], boundary_type_xmax=bc[1],
                       boundary_type_ymin=bc[2], boundary_type_ymax=bc[3])
    po = O.Params(nx=c["nx"], ny=c["ny"], gamma0=c["gamma0"], cfl=c["cfl"], niter_riemann=c["niter_riemann"],
                  slope_type=c["slope_type"], riemann=c["riemann"], bc_xmin=bc[0], bc_xmax=bc[1], bc_ymin=bc[2],
                  bc_ymax=bc[3])
    return pe, po


@pytest.mark.parametrize("k", range(len(CASES)))
def test_random_configuration_bitwise(e2d, oracle, k):
    c = CASES[k]
    for prec in (8, 4):
        for version in (0, 1, 2):
            pe, po = _params(e2d, oracle, c, version, prec)
            prec_s = "f64" if prec == 8 else "f32"
            u0 = oracle.init_diagonal(po, c["offset"], c["rho_hi"], c["p_hi"], c["rho_lo"], c["p_lo"], prec=prec_s)
            ref, dts_ref, _, _ = oracle.run(po, c["nsteps"], prec=prec_s, u0=u0, nthreads=NTHREADS)
            gpu, dts = e2d.run_steps(c["nsteps"], pe, u0=u0)
            assert np.array_equal(gpu[:, 2:-2, 2:-2], ref[:, 2:-2, 2:-2]), (c, version, prec)
            assert np.array_equal(dts, dts_ref), (c, version, prec)


ADJ = [c for c in (draw(np.random.default_rng(777 + k)) for k in range(40)) if c["nx"] >= 8 and c["ny"] >= 8][:8]


@pytest.mark.parametrize("k", range(len(ADJ)))
@pytest.mark.parametrize("dt_mode", [0, 1], ids=["dt-frozen", "dt-through-max"])
def test_random_adjoint_matches_tangent(e2d, oracle, k, dt_mode):
    c = dict(ADJ[k], riemann=2)  # the adjoint is defined for the HLLC flux
    pe, po = _params(e2d, oracle, c, 0)
    u0 = oracle.init_diagonal(po, c["offset"], c["rho_hi"], c["p_hi"], c["rho_lo"], c["p_lo"])
    u0[0, 2:-2, 2:-2] *= 1.0 + 0.01 * np.random.default_rng(k).standard_normal((c["ny"], c["nx"]))
    with e2d.Adjoint(pe) as A:
        J, g, dts = A.gradient(c["nsteps"], u0, dt_mode=dt_mode)
    d = np.random.default_rng(100 + k).normal(size=(c["ny"], c["nx"]))
    Jt, dJt = oracle.tangent(po, u0, d, c["nsteps"], nthreads=NTHREADS, fixed_dts=dts if dt_mode == 0 else None)
    assert abs(J - Jt) <= 1e-13 * abs(Jt)
    assert abs(float(np.sum(g * d)) - dJt) <= 1e-9 * abs(dJt), (c, float(np.sum(g * d)), dJt)


def _rel_l1(gpu, ref, gamma0):
    """Relative L1 difference per conservative variable (interior cells).  A
    momentum is measured against at least the momentum of the same gas moving
    at Mach 0.01, 0.01 * rho c with rho c ~ sqrt(gamma (gamma - 1) rho E): a
    short run on a skinny grid can leave the gas nearly at rest (momenta
    ~1e-6 of rho c), and the relative difference of such a nearly vanishing
    variable measures rounding noise of the pressure terms that feed it
    (absolute differences ~1e-16), not the step."""
    a, b = gpu[:, 2:-2, 2:-2].astype(np.float64), ref[:, 2:-2, 2:-2].astype(np.float64)
    mscale = 0.01 * float(np.sqrt(gamma0 * (gamma0 - 1.0) * np.abs(b[0] * b[1])).sum())
    floors = [0.0, 0.0, mscale, mscale]
    return [float(np.abs(a[v] - b[v]).sum() / max(np.abs(b[v]).sum(), floors[v], 1e-300)) for v in range(4)]


@pytest.mark.parametrize("k", range(len(CASES)))
def test_random_configuration_fma_build(e2d, oracle, k):
    """The same thirty configurations with the build that fuses multiply-adds:
    FP64 within 1e-12 relative L1 per variable and 1e-14 relative dt of the
    oracle, FP32 within 1e-4 (L1) and 1e-5 (dt) of the FP32 oracle, every
    implementation version."""
    c = CASES[k]
    for prec, (l1_tol, dt_tol) in ((8, (1e-12, 1e-14)), (4, (1e-4, 1e-5))):
        for version in (0, 1, 2):
            pe, po = _params(e2d, oracle, c, version, prec)
            prec_s = "f64" if prec == 8 else "f32"
            u0 = oracle.init_diagonal(po, c["offset"], c["rho_hi"], c["p_hi"], c["rho_lo"], c["p_lo"], prec=prec_s)
            ref, dts_ref, _, _ = oracle.run(po, c["nsteps"], prec=prec_s, u0=u0, nthreads=NTHREADS)
            gpu, dts = e2d.run_steps(c["nsteps"], pe, u0=u0, arith="fma")
            l1 = _rel_l1(gpu, ref, c["gamma0"])
            dr = float(np.max(np.abs(dts.astype(np.float64) - dts_ref) / np.abs(dts_ref)))
            assert max(l1) <= l1_tol and dr <= dt_tol, (c, version, prec, l1, dr)


@pytest.mark.parametrize("k", range(len(ADJ)))
@pytest.mark.parametrize("dt_mode", [0, 1], ids=["dt-frozen", "dt-through-max"])
def test_random_adjoint_fma_build_matches_tangent(e2d, oracle, k, dt_mode):
    """The adjoint of the build with fused multiply-adds on the same random
    configurations (density modulated by 1 % random noise: no ties for the
    two arithmetics to break differently) against the oracle's tangent, to
    1e-7 relative."""
    c = dict(ADJ[k], riemann=2)
    pe, po = _params(e2d, oracle, c, 0)
    u0 = oracle.init_diagonal(po, c["offset"], c["rho_hi"], c["p_hi"], c["rho_lo"], c["p_lo"])
    u0[0, 2:-2, 2:-2] *= 1.0 + 0.01 * np.random.default_rng(k).standard_normal((c["ny"], c["nx"]))
    with e2d.Adjoint(pe, arith="fma") as A:
        J, g, dts = A.gradient(c["nsteps"], u0, dt_mode=dt_mode)
    d = np.random.default_rng(100 + k).normal(size=(c["ny"], c["nx"]))
    Jt, dJt = oracle.tangent(po, u0, d, c["nsteps"], nthreads=NTHREADS, fixed_dts=dts if dt_mode == 0 else None)
    assert abs(J - Jt) <= 1e-12 * abs(Jt)
    assert abs(float(np.sum(g * d)) - dJt) <= 1e-7 * abs(dJt), (c, float(np.sum(g * d)), dJt)
