"""Writes the oracle's regression fixtures tests/golden/oracle_*.npz.

Each fixture holds the parameters, the step count, the precision, the final
state (u after an even number of steps, u2 after an odd one; ghosts
included) and the dt sequence of a run from init_implode.  They pin the
oracle against later changes (tests/test_oracle.py) and give the CUDA path
a committed known answer (tests/test_golden_gpu.py).  The reference itself
ships no fixtures and cannot be compiled here (Fortran), so these are the
oracle's outputs, not the reference's.

Usage: python tests/golden/make_golden.py   (from the repository root)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

CASES = {
    # the reference's own default solver, reflective walls
    "oracle_approx_f64_32x24_12": (dict(nx=32, ny=24, riemann=0), 12, "f64"),
    # HLLC with mixed wall types (reflective, outflow, periodic)
    "oracle_hllc_f64_24x40_11_bc1231": (dict(nx=24, ny=40, riemann=2, bc_xmin=1, bc_xmax=2, bc_ymin=3,
                                             bc_ymax=1), 11, "f64"),
    # single precision (fp_kind = sp_kind)
    "oracle_approx_f32_32x32_8": (dict(nx=32, ny=32, riemann=0), 8, "f32"),
    # minmod slopes (slope_type 1), outflow
    "oracle_hllc_f64_40x40_9_minmod": (dict(nx=40, ny=40, riemann=2, slope_type=1, bc_xmin=2, bc_xmax=2,
                                            bc_ymin=2, bc_ymax=2), 9, "f64"),
}


def main():
    for name, (kw, nsteps, prec) in CASES.items():
        p = O.Params(gamma0=1.4, cfl=0.8, **kw)
        final, dts, _, _ = O.run(p, nsteps, prec=prec)
        meta = {f"p_{k}": v for k, v in vars(p).items()}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), state=final, dts=dts, nsteps=nsteps,
                            prec=prec, **meta)
        print(name, final.shape, dts[-1])


if __name__ == "__main__":
    main()
