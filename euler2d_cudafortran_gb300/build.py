"""Build of the native parts: the CUDA library (sm_103a) and the C++ HydroRun driver.

Everything is built in-tree under ``euler2d_cudafortran_gb300/_build/<machine>/``
(``platform.machine()``: ``x86_64``, ``aarch64``) with plain ``nvcc``/``g++``
invocations run in parallel (no cmake), so the same recipe works on x86-64
(cross-compiling the device code) and on the aarch64 GPU host, and objects of
one host architecture are never reused on the other.

Two builds of the same sources share one C ABI:

``libeuler2d_gb300.so`` (arithmetic "exact")
    ``-fmad=false`` stops the compiler from contracting a multiply and an add
    into one FMA, and ``-prec-div=true -prec-sqrt=true -ftz=false`` keep IEEE
    round-to-nearest division and square root in single precision (double is
    always IEEE).  Host code gets ``-ffp-contract=off`` for the same reason.
    With these, every operation of the step rounds as in the reference's
    Fortran build (serial_ref, gfortran without contraction), and results are
    bitwise those of the oracle.

``libeuler2d_gb300_fma.so`` (arithmetic "fma")
    ``-fmad=true``: a multiplication feeding an addition is one fused
    multiply-add, one rounding instead of two and one FP64 issue slot instead
    of two -- what nvfortran's ``-O3 -cuda`` / ``-stdpar=gpu`` builds of the
    reference do by default (cuf/Makefile:22, stdpar/Makefile:8).  Double
    division and square root are faithfully rounded (the correctly rounded
    result or one of its two neighbours; single precision stays IEEE); results
    agree with the oracle to the specified 1e-12 relative L1 per variable and
    1e-14 relative dt, not bit for bit.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
DRIVER = os.path.join(HERE, "driver")
OUT = os.path.join(HERE, "_build", platform.machine() or "unknown")
LIB_NAMES = {"exact": "libeuler2d_gb300.so", "fma": "libeuler2d_gb300_fma.so"}
LIBS = {k: os.path.join(OUT, v) for k, v in LIB_NAMES.items()}
LIB = LIBS["exact"]
EXE = os.path.join(OUT, "euler2d_gb300")
EXES = {"exact": EXE, "fma": os.path.join(OUT, "euler2d_gb300_fma")}  # the driver linked to each build

CUDA_SOURCES = ["abi.cu", "k_sweeps.cu", "k_fused.cu", "k_probe.cu", "noalloc.cu", "k_selftest.cu", "k_batch.cu",
                "abi_batch.cu", "k_adjoint.cu", "abi_adjoint.cu", "abi_adjoint_batch.cu"]
DRIVER_SOURCES = ["main.cpp", "namelist.cpp", "vtk.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
                 "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", os.path.join(ROOT, "include")]
VARIANT_FLAGS = {"exact": ["-fmad=false"], "fma": ["-fmad=true", "-DE2D_FMA=1"]}
NVCC_FLAGS = COMMON + VARIANT_FLAGS["exact"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags: list[str] | None = None,
          variants: tuple[str, ...] = ("exact", "fma")) -> str:
    """Compile the CUDA libraries (both arithmetic variants by default) and the
    driver; returns the path of the exact library."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "euler2d_gb300.h"))
    jobs, links = [], []
    for var in variants:
        odir = os.path.join(OUT, var)
        os.makedirs(odir, exist_ok=True)
        flags = COMMON + VARIANT_FLAGS[var] + (extra_flags or [])
        objs = []
        for src in CUDA_SOURCES:
            s = os.path.join(CSRC, src)
            o = os.path.join(odir, src.replace(".cu", ".o"))
            objs.append(o)
            if _stale(o, [s] + headers + [__file__]):
                jobs.append([nvcc] + flags + ["-c", s, "-o", o])
        links.append((LIBS[var], objs))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    for lib, objs in links:
        if _stale(lib, objs):
            _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs)
    drv = [os.path.join(DRIVER, f) for f in DRIVER_SOURCES]
    for var in variants:
        exe, lib = EXES[var], LIBS[var]
        if all(os.path.exists(d) for d in drv) and _stale(exe, drv + [lib, os.path.join(DRIVER, "namelist.h")]):
            libname = LIB_NAMES[var][3:-3]  # libX.so -> X
            _run(["g++", "-O2", "-std=c++17", "-pthread", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                  "-o", exe] + drv + ["-L", OUT, "-l" + libname, "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
