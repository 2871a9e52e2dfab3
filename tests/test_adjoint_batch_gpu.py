"""The batched adjoint: every problem of an ensemble gets the gradient the
single-problem adjoint gives it (same dt sequence bit for bit; J and the
gradient to round-off, since both accumulate with atomics), and the gradient
agrees with the CPU forward-mode tangent of the oracle."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NTHREADS = os.cpu_count() or 1
SIZES = [(48, 40), (64, 64), (33, 70), (80, 24)]
BCS = [[1, 1, 1, 1], [2, 2, 2, 2], [1, 2, 2, 1], [2, 1, 1, 2]]
OFFSET = [0.5, 0.35, 0.62, 0.45]
RHO_HI = [1.0, 0.4, 0.9, 0.3]
P_HI = [1.0, 0.5, 0.2, 0.8]
RHO_LO = [0.125, 0.9, 0.15, 0.6]
P_LO = [float(np.float32(0.14)), 0.2, 0.7, 0.25]


def single_params(E, O, k):
    nx, ny = SIZES[k]
    bc = BCS[k]
    pe = E.make_params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann_solver=E.RIEMANN_HLLC,
                       boundary_type_xmin=bc[0], boundary_type_xmax=bc[1],
                       boundary_type_ymin=bc[2], boundary_type_ymax=bc[3])
    po = O.Params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann=2, bc_xmin=bc[0], bc_xmax=bc[1],
                  bc_ymin=bc[2], bc_ymax=bc[3])
    u0 = O.init_diagonal(po, OFFSET[k], RHO_HI[k], P_HI[k], RHO_LO[k], P_LO[k])
    return pe, po, u0


def make_batch(E):
    b = E.AdjointBatch(SIZES, BCS, gamma0=1.4, cfl=0.8)
    b.init_diagonal(OFFSET, RHO_HI, P_HI, RHO_LO, P_LO)
    return b


def rel_l1(a, b):
    return float(np.sum(np.abs(a - b)) / max(np.sum(np.abs(b)), 1e-300))


@pytest.mark.parametrize("dt_mode", [0, 1], ids=["dt-frozen", "dt-through-max"])
def test_batch_adjoint_equals_single_problem_adjoints(e2d, oracle, dt_mode):
    n = 23  # K = 5: a ragged last segment
    with make_batch(e2d) as b:
        J, grads, dts = b.gradient(n, dt_mode=dt_mode)
        Jf = b.objective(n)
        J2, grads2, _ = b.gradient(n, dt_mode=dt_mode)  # graph replay
    for k in range(len(SIZES)):
        pe, po, u0 = single_params(e2d, oracle, k)
        with e2d.Adjoint(pe) as A:
            Js, gs, dts_s = A.gradient(n, u0, dt_mode=dt_mode)
        assert np.array_equal(dts[:, k], dts_s), f"problem {k}: dt sequence"
        assert abs(J[k] - Js) <= 1e-13 * abs(Js), (k, J[k], Js)
        assert abs(Jf[k] - Js) <= 1e-13 * abs(Js), (k, Jf[k], Js)
        assert rel_l1(grads[k], gs) <= 1e-11, (k, rel_l1(grads[k], gs))
        assert rel_l1(grads2[k], gs) <= 1e-11
        assert np.any(grads[k] != 0.0)


def test_batch_adjoint_matches_forward_mode_tangent(e2d, oracle):
    n = 17
    with make_batch(e2d) as b:
        J, grads, _ = b.gradient(n, dt_mode=1)
    rng = np.random.default_rng(5)
    for k in (0, 2):
        _, po, u0 = single_params(e2d, oracle, k)
        d = rng.normal(size=(SIZES[k][1], SIZES[k][0]))
        Jt, dJt = oracle.tangent(po, u0, d, n, nthreads=NTHREADS)
        assert abs(J[k] - Jt) <= 1e-13 * abs(Jt)
        assert abs(float(np.sum(grads[k] * d)) - dJt) <= 1e-9 * abs(dJt), (k, float(np.sum(grads[k] * d)), dJt)


def test_batch_adjoint_uploaded_state(e2d, oracle):
    """A state uploaded for one problem replaces its diagonal initial state."""
    n = 9
    with make_batch(e2d) as b:
        _, po, _ = single_params(e2d, oracle, 1)
        u0 = oracle.init_implode(po)
        u0[0, 2:-2, 2:-2] *= 1.0 + 0.01 * np.random.default_rng(3).standard_normal((po.ny, po.nx))
        b.set_state(1, u0)
        J, grads, _ = b.gradient(n, dt_mode=1)
    pe, _, _ = single_params(e2d, oracle, 1)
    with e2d.Adjoint(pe) as A:
        Js, gs, _ = A.gradient(n, u0, dt_mode=1)
    assert abs(J[1] - Js) <= 1e-13 * abs(Js)
    assert rel_l1(grads[1], gs) <= 1e-11


def test_batch_tape_gives_the_recomputed_gradient(e2d, monkeypatch):
    """With the tape (written by the recomputation, the recomputation then
    following each segment's reverse sweep) and without it (E2D_NO_TAPE=1:
    the reverse recomputes, the recomputation overlaps it), the gradients
    agree to round-off."""
    n = 23  # K = 5: a ragged last segment, four recomputed segments
    with make_batch(e2d) as b:
        J1, g1, d1 = b.gradient(n, dt_mode=1)
    monkeypatch.setenv("E2D_NO_TAPE", "1")
    with make_batch(e2d) as b:
        J2, g2, d2 = b.gradient(n, dt_mode=1)
    assert np.array_equal(d1, d2)
    for k in range(len(SIZES)):
        assert abs(J1[k] - J2[k]) <= 1e-13 * abs(J2[k])
        assert np.any(g1[k] != 0.0)
        assert rel_l1(g1[k], g2[k]) <= 1e-12, (k, rel_l1(g1[k], g2[k]))


@pytest.mark.parametrize("dt_mode", [0, 1], ids=["dt-frozen", "dt-through-max"])
def test_fma_batch_adjoint_equals_single_problem_adjoints(e2d, oracle, dt_mode):
    """The build with fused multiply-adds: each problem's gradient from the
    batch equals its single-problem adjoint's (to round-off) on states
    modulated by 1 % random noise (no ties for the two paths' roundings to
    break differently)."""
    n = 23
    rng = np.random.default_rng(31)
    states = []
    for k in range(len(SIZES)):
        _, po, u0 = single_params(e2d, oracle, k)
        u0 = u0.copy()
        u0[0, 2:-2, 2:-2] *= 1.0 + 0.01 * rng.standard_normal((po.ny, po.nx))
        states.append(u0)
    with e2d.AdjointBatch(SIZES, BCS, gamma0=1.4, cfl=0.8, arith="fma") as b:
        for k, u0 in enumerate(states):
            b.set_state(k, u0)
        J, grads, dts = b.gradient(n, dt_mode=dt_mode)
    for k in range(len(SIZES)):
        pe, _, _ = single_params(e2d, oracle, k)
        with e2d.Adjoint(pe, arith="fma") as A:
            Js, gs, dts_s = A.gradient(n, states[k], dt_mode=dt_mode)
        assert float(np.max(np.abs(dts[:, k] - dts_s) / dts_s)) <= 1e-14, f"problem {k}: dt sequence"
        assert abs(J[k] - Js) <= 1e-12 * abs(Js), (k, J[k], Js)
        assert rel_l1(grads[k], gs) <= 1e-9, (k, rel_l1(grads[k], gs))
        assert np.any(grads[k] != 0.0)
