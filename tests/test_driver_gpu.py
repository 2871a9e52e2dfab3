"""The C++ HydroRun driver end to end (the device-resident loop and the
reference's per-call loop), and the asynchronous output path.

The driver's default output is asynchronous (device snapshot in stream
order, copy on a second stream, VTK file written by a worker thread while
the next steps run); --sync-io downloads and writes in the step loop as
serial_ref/main.f90 does.  Both must write byte-identical files, and the
last file must hold the oracle's final state."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NML = """&RUN
tEnd=10.0
nStepmax=23
nOutput=5
/
&MESH
nx=48
ny=40
boundary_type_xmin=1
boundary_type_xmax=2
boundary_type_ymin=1
boundary_type_ymax=3
/
&HYDRO
gamma0=1.4
cfl=0.8
smallr=1e-7
smallc=1e-7
niter_riemann=10
iorder=2
slope_type=2
/
"""


def run_driver(exe, nml, outdir, *flags):
    os.makedirs(outdir, exist_ok=True)
    out = subprocess.run([exe, nml, "--binary-vtk", "--outdir", outdir, *flags], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "Perf" in out.stdout
    return sorted(os.listdir(outdir))


def read_binary_vti(path, nx, ny):
    raw = open(path, "rb").read()
    start = raw.index(b"<AppendedData encoding=\"raw\">")
    data = raw[raw.index(b"_", start) + 1:]
    fields = []
    o = 0
    for _ in range(4):
        n = int(np.frombuffer(data[o:o + 4], dtype=np.uint32)[0])
        fields.append(np.frombuffer(data[o + 4:o + 4 + n], dtype=np.float64).reshape(ny, nx))
        o += 4 + n
    return np.stack(fields)


def test_async_and_sync_output_identical(e2d, oracle, tmp_path):
    from euler2d_cudafortran_gb300 import build
    nml = tmp_path / "test.nml"
    nml.write_text(NML)
    a = run_driver(build.EXE, str(nml), str(tmp_path / "async"))
    s = run_driver(build.EXE, str(nml), str(tmp_path / "sync"), "--sync-io")
    assert a == s and len(a) == 6  # steps 0, 5, 10, 15, 20 and the final 23
    c = run_driver(build.EXE, str(nml), str(tmp_path / "percall"), "--percall")
    assert c == a
    for name in a:
        assert (tmp_path / "async" / name).read_bytes() == (tmp_path / "sync" / name).read_bytes(), name
        assert (tmp_path / "percall" / name).read_bytes() == (tmp_path / "sync" / name).read_bytes(), name
    # serial_ref/main.f90:81 writes u at the end: after 23 steps that is u after step 22
    po = oracle.Params(nx=48, ny=40, gamma0=1.4, cfl=0.8, riemann=0, bc_xmin=1, bc_xmax=2, bc_ymin=1, bc_ymax=3)
    _, _, u, _ = oracle.run(po, 23)
    got = read_binary_vti(str(tmp_path / "async" / a[-1]), 48, 40)
    assert np.array_equal(got, u[:, 2:-2, 2:-2])


def test_begin_download_snapshots_in_stream_order(e2d):
    p = e2d.make_params(nx=96, ny=80, riemann_solver=e2d.RIEMANN_HLLC)
    with e2d.HydroRun(p) as run:
        run.init_implode()
        run.advance(0, 10, log=False)
        ref = run.get_state(0)
        out = run.new_state()
        run.begin_download(0, out)
        run.advance(10, 6, log=False)  # overwrites u while the copy may still be in flight
        got = run.wait_download()
        assert np.array_equal(got, ref)
        assert not np.array_equal(run.get_state(0), ref)


def test_fma_driver_within_tolerance_of_the_oracle(e2d, oracle, tmp_path):
    """The same driver linked to the build with fused multiply-adds
    (-leuler2d_gb300_fma): the same files, the final state within 1e-12
    relative L1 per variable of the oracle's."""
    from euler2d_cudafortran_gb300 import build
    nml = tmp_path / "test.nml"
    nml.write_text(NML)
    a = run_driver(build.EXES["fma"], str(nml), str(tmp_path / "fma"))
    assert len(a) == 6
    po = oracle.Params(nx=48, ny=40, gamma0=1.4, cfl=0.8, riemann=0, bc_xmin=1, bc_xmax=2, bc_ymin=1, bc_ymax=3)
    _, _, u, _ = oracle.run(po, 23)
    got = read_binary_vti(str(tmp_path / "fma" / a[-1]), 48, 40)
    want = u[:, 2:-2, 2:-2]
    l1 = [float(np.abs(got[v] - want[v]).sum() / np.abs(want[v]).sum()) for v in range(4)]
    assert max(l1) <= 1e-12, l1
