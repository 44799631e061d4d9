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


# ------------------------------------------------------------ mesh refresh
HYDRO_SLOTS = (0, 1, 2, 3, 4, 5, 9, 13)  # rho, v, etot, eint, pressure, passive_0
MHD_SLOTS = HYDRO_SLOTS + (6, 7, 8, 17, 18, 19)


def mesh_blocks(nblocks, n, g, slots, dtype, seed, rho_pow2=False):
    """Per block a dict slot -> array in Cello's layout: random active cells
    (density positive; a power of two when rho_pow2), NaN ghosts."""
    rng = np.random.default_rng(seed)
    m = [x + 2 * g for x in n]
    out = []
    for _ in range(nblocks):
        b = {}
        for s in slots:
            shp = [m[2], m[1], m[0]]
            if s >= 17:
                shp[2 - (s - 17)] += 1
            a = np.full(shp, np.nan, dtype=dtype)
            # numpy axis k holds the spatial axis 2 - k; faces add one along theirs
            act = tuple(slice(g, g + n[2 - k] + (1 if s >= 17 and 2 - k == s - 17 else 0))
                        for k in range(3))
            if s == 0:
                v = (2.0 ** rng.integers(-3, 4, size=a[act].shape) if rho_pow2
                     else 0.5 + rng.random(a[act].shape))
            else:
                v = rng.standard_normal(a[act].shape)
            a[act] = v.astype(dtype)
            b[s] = a
        out.append(b)
    return out
