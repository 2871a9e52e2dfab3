"""Seeded ensembles of independent diagonal-interface problems.

The batched workload: square grids with sides drawn uniformly from
{128, 192, ..., 1024}, a diagonal interface at an offset uniform in
[0.3, 0.7], densities and pressures on both sides log-uniform in [0.1, 1],
and reflective (1) or outflow (2) walls at random (one type per problem), all
from one seed.  The high (upper-right) side of the interface is the
"right" state, the low side the "left" state.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Ensemble:
    sizes: list          # [(nx, ny)]
    bcs: list            # [[xmin, xmax, ymin, ymax]]
    offset: np.ndarray
    rho_hi: np.ndarray
    p_hi: np.ndarray
    rho_lo: np.ndarray
    p_lo: np.ndarray

    @property
    def cells(self) -> int:
        return int(sum(a * b for a, b in self.sizes))


def diagonal_ensemble(nprob: int = 64, seed: int = 12345, sides=tuple(range(128, 1025, 64))) -> Ensemble:
    rng = np.random.default_rng(seed)
    side = rng.choice(np.asarray(sides), size=nprob)
    logu = lambda: 10.0 ** rng.uniform(-1.0, 0.0, size=nprob)  # noqa: E731
    offset = rng.uniform(0.3, 0.7, size=nprob)
    rho_lo, rho_hi, p_lo, p_hi = logu(), logu(), logu(), logu()
    bc = rng.choice(np.array([1, 2]), size=nprob)
    return Ensemble(sizes=[(int(s), int(s)) for s in side], bcs=[[int(b)] * 4 for b in bc], offset=offset,
                    rho_hi=rho_hi, p_hi=p_hi, rho_lo=rho_lo, p_lo=p_lo)
