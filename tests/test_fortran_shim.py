"""The Fortran drop-in module, parsed (no Fortran compiler exists here).

euler2d_cudafortran_gb300/fortran/m_euler2d_gb300.f90 holds the ISO_C_BINDING
interface of the C ABI (module m_euler2d_gb300_abi) and an m_run module with
the procedures serial_ref/main.f90 calls.  No Fortran compiler is installed
on any machine of this build, so the module is checked by parsing it with
numpy's Fortran front end (f2py's crackfortran):

* every bind(C) interface names a function of include/euler2d_gb300.h, with
  the same number of arguments, scalars passed by value where C takes them
  by value and by reference where C takes a pointer to one, pointers as type(c_ptr), value where C takes a pointer, handles
  returned through an argument (C: T**) as type(c_ptr) by reference, the
  parameter struct by reference, and an integer(c_int) result;
* the bind(C) type e2d_params has the C struct's fields, in its order, with
  c_int / c_double kinds;
* m_run exposes the procedures and argument lists of serial_ref/m_run.f90
  that serial_ref/main.f90:36-86 calls (initHydroParameters :48,
  printHydroParameters, run_init :150, compute_dt(hydroParams, dt, useU)
  :248, make_boundaries(hydroParams, data) :561, godunov_unsplit(nStep, dt)
  :187, saveVTK(data, iStep) :653, run_cleanup :172) and the module
  variables it reads (u, u2, hydroParams, nStepmax, tEnd, nOutput).
"""
import contextlib
import io
import os
import re
import warnings

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "euler2d_cudafortran_gb300", "fortran", "m_euler2d_gb300.f90")
HEADER = os.path.join(ROOT, "include", "euler2d_gb300.h")


@pytest.fixture(scope="module")
def modules():
    cf = pytest.importorskip("numpy.f2py.crackfortran")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        with contextlib.redirect_stdout(io.StringIO()), contextlib.redirect_stderr(io.StringIO()):
            mods = cf.crackfortran([SHIM])
    return {m["name"]: m for m in mods}


def c_functions():
    """name -> list of parameter declarations of include/euler2d_gb300.h."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(?:int|const char\*)\s+(e2d_\w+)\s*\(([^)]*)\)\s*;", text):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(1)] = params
    return out


def interfaces(mod):
    for block in mod["body"]:
        if block.get("block") == "interface":
            for f in block.get("body", []):
                if f.get("block") == "function":
                    yield f


def test_bind_c_interfaces_match_the_header(modules):
    cfuns = c_functions()
    seen = []
    for f in interfaces(modules["m_euler2d_gb300_abi"]):
        name = f["name"]
        bind = f.get("bindlang", {}).get(name, {})
        assert bind.get("lang") == "c" and bind.get("name") == name, f"{name}: not bind(C, name=\"{name}\")"
        assert name in cfuns, f"{name} is not declared in include/euler2d_gb300.h"
        cparams = cfuns[name]
        assert len(f["args"]) == len(cparams), (name, f["args"], cparams)
        assert f["vars"][name]["typespec"] == "integer", f"{name}: result must be integer(c_int)"
        for a, cp in zip(f["args"], cparams):
            v = f["vars"][a]
            pointer = "*" in cp
            if v["typespec"] == "type" and v.get("typename") == "c_ptr":
                if "**" in cp:  # a handle returned through the argument: type(c_ptr), intent(out)
                    assert "value" not in v.get("attrspec", []), (name, a, cp)
                else:
                    assert pointer and "value" in v.get("attrspec", []), (name, a, cp)
            elif v["typespec"] == "type":  # a bind(C) derived type, passed by reference
                assert pointer and "value" not in v.get("attrspec", []), (name, a, cp)
                assert v.get("typename") == "e2d_params" and "e2d_params" in cp, (name, a, cp)
            else:
                # a scalar: by value where C takes a value, by reference where C takes a pointer
                assert pointer == ("value" not in v.get("attrspec", [])), (name, a, cp)
                kind = v.get("kindselector", {}).get("kind")
                want = "c_int" if re.match(r"int\b", cp) else "c_double"
                assert kind == want, (name, a, cp, kind)
        seen.append(name)
    for must in ("e2d_create", "e2d_destroy", "e2d_compute_dt", "e2d_make_boundaries", "e2d_godunov_unsplit",
                 "e2d_upload_state", "e2d_download_state", "e2d_advance"):
        assert must in seen


def test_params_type_matches_the_c_struct(modules, e2d):
    types = [b for b in modules["m_euler2d_gb300_abi"]["body"] if b.get("block") == "type"]
    assert len(types) == 1 and types[0]["name"] == "e2d_params"
    t = types[0]
    fields = t["sortvars"]
    assert fields == [f[0] for f in e2d.Params._fields_]
    for name, ctype in e2d.Params._fields_:
        want = "c_double" if ctype.__name__ == "c_double" else "c_int"
        assert t["vars"][name]["kindselector"]["kind"] == want, name


def test_m_run_keeps_the_reference_procedures(modules):
    run = modules["m_run"]
    procs = {b["name"]: b.get("args", []) for b in run["body"] if b.get("block") == "subroutine"}
    want = {
        "inithydroparameters": [], "printhydroparameters": [], "run_init": [], "run_cleanup": [],
        "compute_dt": ["params", "dt", "useu"], "make_boundaries": ["params", "data"],
        "godunov_unsplit": ["nstep", "dt"], "savevtk": ["data", "istep"],
    }
    for name, args in want.items():
        assert name in procs, f"m_run lacks {name}"
        assert len(procs[name]) == len(args), (name, procs[name])
    for var in ("u", "u2", "hydroparams", "nstepmax", "tend", "noutput"):
        assert var in run["vars"], f"m_run lacks the module variable {var}"
