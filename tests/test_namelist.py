"""The parameter-file readers (Python and the C++ driver) on namelist files
laid out like the reference's test.nml: &RUN, &MESH, &HYDRO, optional
&OTHER (implementationVersion) and the trailing &GB300 group."""
import json
import os
import subprocess

import pytest

from euler2d_cudafortran_gb300 import namelist

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def test_reference_groups_only():
    cfg = namelist.read_config(os.path.join(GOLDEN, "run_reference_groups.nml"))
    assert (cfg.nx, cfg.ny, cfg.nStepmax, cfg.nOutput) == (256, 256, 500, 100)
    assert cfg.gamma0 == 1.4 and cfg.cfl == 0.8 and cfg.smallr == 1e-7
    assert cfg.implementationVersion == 0 and cfg.riemann_solver == 0 and cfg.precision == 8


def test_extended_groups():
    cfg = namelist.read_config(os.path.join(GOLDEN, "run_hllc_fp32.nml"))
    assert (cfg.nx, cfg.ny) == (256, 128)
    assert (cfg.boundary_type_xmin, cfg.boundary_type_xmax, cfg.boundary_type_ymin) == (1, 2, 3)
    assert cfg.gamma0 == 1.4  # Fortran d exponent
    assert cfg.slope_type == 2  # real in the cuf/stdpar variants
    assert cfg.implementationVersion == 1 and cfg.riemann_solver == 2 and cfg.precision == 4


def test_unknown_key_is_an_error(tmp_path):
    p = tmp_path / "bad.nml"
    p.write_text("&RUN\nnStepmax=1\n/\n&MESH\nnx=8\nny=8\nbogus=3\n/\n&HYDRO\ngamma0=1.4\n/\n")
    with pytest.raises(namelist.NamelistError):
        namelist.read_config(str(p))


def test_bad_implementation_version(tmp_path):
    p = tmp_path / "bad.nml"
    p.write_text("&RUN\nnStepmax=1\n/\n&MESH\nnx=8\nny=8\n/\n&HYDRO\ngamma0=1.4\n/\n&OTHER\nimplementationVersion=3\n/\n")
    with pytest.raises(namelist.NamelistError):
        namelist.read_config(str(p))


@pytest.mark.parametrize("name", ["run_reference_groups.nml", "run_hllc_fp32.nml"])
def test_cpp_driver_reads_the_same_values(e2d, name):
    """The C++ HydroRun driver and the Python reader agree on every value."""
    from euler2d_cudafortran_gb300 import build
    if not os.path.exists(build.EXE):
        build.build()
    path = os.path.join(GOLDEN, name)
    out = subprocess.run([build.EXE, path, "--parse-only"], capture_output=True, text=True, check=True).stdout
    got = json.loads(out)
    cfg = namelist.read_config(path)
    for k, v in got.items():
        assert getattr(cfg, k) == v, k
