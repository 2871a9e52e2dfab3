"""Reader for the reference's Fortran namelist parameter file (test.nml).

The groups and keys are those of serial_ref/m_run.f90:71-73 (&RUN, &MESH,
&HYDRO), the cuf variant's &OTHER implementationVersion
(cuf/m_HydroParameters.cuf:90), and a trailing &GB300 group for the keys this
implementation adds (riemann_solver, precision).  Because Fortran reads the
groups by name in file order, a file with the extra trailing group is still
readable by the reference binaries.

Values of keys absent from the file keep the defaults of the reference
(niter_riemann=10 and boundary types 1, serial_ref/m_run.f90:62-68).  Like a
Fortran namelist read, an unknown key inside a known group is an error.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

_GROUP_KEYS = {
    "run": {"tend", "nstepmax", "noutput"},
    "mesh": {"nx", "ny", "boundary_type_xmin", "boundary_type_xmax", "boundary_type_ymin", "boundary_type_ymax"},
    "hydro": {"gamma0", "cfl", "smallr", "smallc", "niter_riemann", "iorder", "slope_type"},
    "other": {"implementationversion"},
    "gb300": {"riemann_solver", "precision"},
}


class NamelistError(ValueError):
    pass


@dataclass
class RunConfig:
    """Everything the HydroRun driver reads from the parameter file."""
    tEnd: float = 0.0
    nStepmax: int = 0
    nOutput: int = 1
    nx: int = 0
    ny: int = 0
    boundary_type_xmin: int = 1
    boundary_type_xmax: int = 1
    boundary_type_ymin: int = 1
    boundary_type_ymax: int = 1
    gamma0: float = 1.666
    cfl: float = 0.8
    smallr: float = 1e-7
    smallc: float = 1e-7
    niter_riemann: int = 10
    iorder: int = 2
    slope_type: int = 2
    implementationVersion: int = 0
    riemann_solver: int = 0
    precision: int = 8
    groups: list = field(default_factory=list)


def _parse_value(tok: str):
    t = tok.strip()
    low = t.lower()
    if low in (".true.", "t", ".t."):
        return True
    if low in (".false.", "f", ".f."):
        return False
    if (t.startswith("'") and t.endswith("'")) or (t.startswith('"') and t.endswith('"')):
        return t[1:-1]
    # Fortran exponent letters d/q mean double/quad precision
    num = re.sub(r"(?<=[0-9.])[dDqQ](?=[+-]?[0-9])", "e", t)
    try:
        if re.fullmatch(r"[+-]?[0-9]+", num):
            return int(num)
        return float(num)
    except ValueError as e:
        raise NamelistError(f"cannot parse value {tok!r}") from e


def parse_namelist(text: str) -> dict:
    """Parse every &group ... / block into {group: {key: value}} (lower-case)."""
    # strip comments (! to end of line, outside quotes)
    lines = []
    for line in text.splitlines():
        out, q = [], None
        for ch in line:
            if q:
                out.append(ch)
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
                out.append(ch)
            elif ch == "!":
                break
            else:
                out.append(ch)
        lines.append("".join(out))
    body = "\n".join(lines)
    groups = {}
    for m in re.finditer(r"[&$]([A-Za-z_][A-Za-z0-9_]*)(.*?)(?:/|[&$]end\b)", body, re.S | re.I):
        name = m.group(1).lower()
        content = m.group(2)
        items = {}
        for km in re.finditer(r"([A-Za-z_][A-Za-z0-9_%]*)\s*=\s*([^=]*?)(?=(?:,?\s*[A-Za-z_][A-Za-z0-9_%]*\s*=)|\s*$)",
                              content, re.S):
            key = km.group(1).lower()
            val = km.group(2).strip().rstrip(",").strip()
            items[key] = _parse_value(val)
        groups[name] = items
    return groups


_RIEMANN_NAMES = {"approx": 0, "hllc": 2, "0": 0, "2": 2}


def read_config(path: str) -> RunConfig:
    """initHydroParameters' namelist read (serial_ref/m_run.f90:87-92)."""
    with open(path) as f:
        groups = parse_namelist(f.read())
    for g in ("run", "mesh", "hydro"):
        if g not in groups:
            raise NamelistError(f"namelist group &{g.upper()} missing from {path}")
    cfg = RunConfig(groups=list(groups))
    for g, items in groups.items():
        allowed = _GROUP_KEYS.get(g)
        if allowed is None:
            continue
        for k, v in items.items():
            if k not in allowed:
                raise NamelistError(f"unknown key {k!r} in namelist group &{g.upper()}")
            if k == "tend":
                cfg.tEnd = float(v)
            elif k == "nstepmax":
                cfg.nStepmax = int(v)
            elif k == "noutput":
                cfg.nOutput = int(v)
            elif k == "implementationversion":
                cfg.implementationVersion = int(v)
            elif k == "riemann_solver":
                key = str(v).lower()
                if key not in _RIEMANN_NAMES:
                    raise NamelistError(f"riemann_solver must be 'approx' or 'hllc', got {v!r}")
                cfg.riemann_solver = _RIEMANN_NAMES[key]
            elif k in ("gamma0", "cfl", "smallr", "smallc"):
                setattr(cfg, k, float(v))
            else:
                setattr(cfg, k, int(v))
    if cfg.implementationVersion not in (0, 1, 2):
        raise NamelistError("The implementation version parameter should 0, 1 or 2 !!! "
                            "Check your namelist file, section OTHER")
    if cfg.precision not in (4, 8):
        raise NamelistError("precision must be 4 or 8")
    return cfg
