"""Shared test helpers: run the same seeded block through the CPU oracle and
the CUDA path through the C ABI."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from mhdvlct import ic

SOLVERS = {"hlle": O.HLLE, "hllc": O.HLLC, "hlld": O.HLLD}
RECONS = {"nn": O.NN, "plm": O.PLM, "plm_athena": O.PLM_ATHENA}


def oracle_block(state, n, g, widths, mhd=True, de=False):
    b = O.Block(n, g, widths, mhd=mhd, dual_energy=de)
    for k, v in state.items():
        key = ic.ORACLE_NAME[k]
        if key in b.f:
            b.f[key][...] = v
    return b


def oracle_params(solver="hlld", recon="plm", de=False, euler=False,
                  theta=1.5, courant=0.3, eta=0.001, dfloor=1e-200,
                  pfloor=1e-200):
    return O.params(riemann=SOLVERS[solver], recon=RECONS[recon],
                    mhd=(solver != "hllc"), dual_energy=de, euler=euler,
                    eta=eta, theta_limiter=theta, courant=courant,
                    density_floor=dfloor, pressure_floor=pfloor)


def rel_l1(a, b):
    """sum |a - b| / sum |b| (0 when both vanish)."""
    den = np.sum(np.abs(b))
    num = np.sum(np.abs(a - b))
    return 0.0 if den == 0 and num == 0 else num / max(den, 1e-300)
