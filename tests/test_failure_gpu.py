"""Failure detection without a GPU fault.

Every wait in the library is bounded: the step kernels' TMA wait gives up
after about a second, raises health flag 4 and returns, so a lost transfer
cannot hang the GPU.  Here the same bounded wait is run on an mbarrier that
nothing arrives on (a flag nothing sets, no copy in flight): it must give up
after its limit, report it, and leave the context usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_stays_usable(e2d, oracle):
    limit = 1 << 22  # about 2 ms of SM cycles
    arrived, silent, waited = e2d.selftest_wait(limit)
    assert arrived is True
    assert silent is False
    assert limit < waited < 64 * limit
    # the context still runs the step, bitwise as before
    p = e2d.make_params(nx=40, ny=32, gamma0=1.4, cfl=0.8, riemann_solver=e2d.RIEMANN_HLLC)
    gpu, dts = e2d.run_steps(6, p)
    ref, dts_ref, _, _ = oracle.run(oracle.Params(nx=40, ny=32, riemann=2), 6)
    assert np.array_equal(gpu[:, 2:-2, 2:-2], ref[:, 2:-2, 2:-2]) and np.array_equal(dts, dts_ref)


def test_bounded_wait_rejects_bad_limits(e2d):
    with pytest.raises(e2d.E2DError):
        e2d.selftest_wait(0)
