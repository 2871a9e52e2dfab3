"""NVTX ranges of the C ABI carry the reference's names and nesting.

serial_ref opens NVTX ranges godunov_compute (0), compute_dt (1),
convertToPrimitives (2), computeAndStoreFluxes (3), updateHydro (4) and
make_boundaries (5) (serial_ref/m_run.f90:195,264,336,387,502,571).  The
library opens the same ranges around the same work.  A small injection
library (tests/nvtx_recorder.c, loaded through NVTX_INJECTION64_PATH as
profilers are) records them in a child process.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.fixture(scope="module")
def recorder(tmp_path_factory):
    out = tmp_path_factory.mktemp("nvtx") / "libnvtx_recorder.so"
    subprocess.run(["gcc", "-shared", "-fPIC", "-O1", "-I", os.path.join(CUDA, "include"), "-o", str(out),
                    os.path.join(ROOT, "tests", "nvtx_recorder.c")], check=True)
    return str(out)


def record(recorder, tmp_path, code):
    path = tmp_path / "ranges.txt"
    env = dict(os.environ, NVTX_INJECTION64_PATH=recorder, E2D_NVTX_RECORD=str(path))
    subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, check=True, timeout=300)
    return path.read_text().split("\n")[:-1] if path.exists() else []


def test_entry_points_open_the_reference_ranges(e2d, recorder, tmp_path):
    """Each procedure's range opens and closes even when the call is refused
    (a null handle: no device needed)."""
    code = (
        "import ctypes, euler2d_cudafortran_gb300 as E\n"
        "lib = E.load_library('exact')\n"
        "d = ctypes.c_double()\n"
        "assert lib.e2d_compute_dt(None, 0, ctypes.byref(d)) == E.E2D_ERR_INVALID_ARG\n"
        "assert lib.e2d_make_boundaries(None, 0) == E.E2D_ERR_INVALID_ARG\n"
        "assert lib.e2d_godunov_unsplit(None, 0, 1e-3) == E.E2D_ERR_INVALID_ARG\n"
    )
    assert record(recorder, tmp_path, code) == [
        "push compute_dt", "pop", "push make_boundaries", "pop", "push godunov_compute", "pop"]


@pytest.mark.gpu
def test_stored_fluxes_step_nests_the_stage_ranges(e2d, recorder, tmp_path):
    """The stored-fluxes step (implementationVersion 2) called as
    serial_ref/main.f90 calls it: godunov_compute holds make_boundaries,
    convertToPrimitives, computeAndStoreFluxes and updateHydro in the order of
    serial_ref/m_run.f90:224-239."""
    code = (
        "import euler2d_cudafortran_gb300 as E\n"
        "with E.HydroRun(nx=64, ny=64, gamma0=1.4, implementation_version=2) as r:\n"
        "    r.init_implode()\n"
        "    dt = r.compute_dt(0)\n"
        "    r.godunov_unsplit(0, dt)\n"
        "    r.synchronize()\n"
    )
    got = record(recorder, tmp_path, code)
    assert got == ["push compute_dt", "pop",
                   "push godunov_compute",
                   "push make_boundaries", "pop", "push convertToPrimitives", "pop",
                   "push computeAndStoreFluxes", "pop", "push updateHydro", "pop",
                   "pop"], got
