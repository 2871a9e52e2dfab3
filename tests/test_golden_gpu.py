"""The CUDA path against the committed oracle fixtures (tests/golden/*.npz,
written by tests/golden/make_golden.py): every implementation version must
reproduce each fixture's interior state and dt sequence bit for bit."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(f for f in os.listdir(GOLDEN) if f.startswith("oracle_") and f.endswith(".npz"))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("version", [0, 1, 2])
def test_cuda_path_reproduces_fixture(e2d, name, version):
    z = np.load(os.path.join(GOLDEN, name))
    m = {k[2:]: z[k].item() for k in z.files if k.startswith("p_")}
    prec = 8 if str(z["prec"]) == "f64" else 4
    n = int(z["nsteps"])
    p = e2d.make_params(nx=m["nx"], ny=m["ny"], gamma0=m["gamma0"], cfl=m["cfl"], smallr=m["smallr"],
                        smallc=m["smallc"], niter_riemann=m["niter_riemann"], iorder=m["iorder"],
                        slope_type=m["slope_type"], boundary_type_xmin=m["bc_xmin"],
                        boundary_type_xmax=m["bc_xmax"], boundary_type_ymin=m["bc_ymin"],
                        boundary_type_ymax=m["bc_ymax"], riemann_solver=m["riemann"],
                        implementation_version=version, precision=prec)
    with e2d.HydroRun(p) as run:
        run.init_implode()
        dts = run.advance(0, n)
        got = run.final_state(n)
    ref = z["state"]
    assert np.array_equal(got[:, 2:-2, 2:-2], ref[:, 2:-2, 2:-2]), name
    assert np.array_equal(dts, z["dts"]), name
