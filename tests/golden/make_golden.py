#!/usr/bin/env python3
"""Generate tests/golden/golden.json and golden_density.npz from the
reference's own VL+CT code.

The reference sources are compiled, unmodified, behind a shim by
`make -C oracle` into oracle/_ref/libvlct_ref.so.  That needs the Enzo-E
source tree, so this script runs only where the tree exists.  Per case it
records:
  - the SHA-256 of the seeded input (tests/golden/golden_input.py);
  - the reference dt (`EnzoMethodMHDVlct::timestep`, as a float hex string);
  - the SHA-256 of every field after the timestep call and one
    `EnzoMethodMHDVlct::compute` step of that dt;
  - the density after the step as a raw array;
  - for hydro cases, the SHA-256 of every boundary-flux array the step
    stores for flux correction (store_fluxes_for_corrections).

Usage:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
from golden_input import CASES, G, N, WIDTHS, digest, golden_input  # noqa: E402

FC_QUANTITIES = (0, 1, 2, 3, 4)
FC_QUANTITIES_DE = (0, 1, 2, 3, 4, 5)

ORACLE_NAME = {"density": "rho", "velocity_x": "vx", "velocity_y": "vy",
               "velocity_z": "vz", "total_energy": "etot",
               "internal_energy": "eint", "bfield_x": "bx", "bfield_y": "by",
               "bfield_z": "bz", "bfieldi_x": "bfx", "bfieldi_y": "bfy",
               "bfieldi_z": "bfz", "pressure": "pressure"}
SOLVER = {"hlle": O.HLLE, "hllc": O.HLLC, "hlld": O.HLLD}
RECON = {"nn": O.NN, "plm": O.PLM, "plm_athena": O.PLM_ATHENA}


def oracle_block(state, mhd, de):
    b = O.Block(N, G, WIDTHS, mhd=mhd, dual_energy=de)
    for k, v in state.items():
        b.f[ORACLE_NAME[k]][...] = v
    return b


def case_params(solver, recon, de, scheme, theta):
    return O.params(riemann=SOLVER[solver], recon=RECON[recon], mhd=solver != "hllc",
                    dual_energy=de, euler=scheme == "euler", theta_limiter=theta,
                    courant=1.0 if scheme == "euler" else 0.3)


def main():
    if O.ref_lib() is None:
        sys.exit("oracle/_ref/libvlct_ref.so is missing: run `make -C oracle` "
                 "where the Enzo-E tree is present")
    out = {"n": list(N), "ghost": G, "widths": list(WIDTHS),
           "generator": "tests/golden/make_golden.py (reference sources via oracle/_ref)",
           "cases": {}}
    dens = {}
    for name, solver, recon, de, scheme, theta, seed in CASES:
        mhd = solver != "hllc"
        state = golden_input(N, G, seed, mhd=mhd, dual_energy=de)
        rec = {"solver": solver, "recon": recon, "dual_energy": de,
               "time_scheme": scheme, "theta": theta, "seed": seed,
               "input_sha256": {k: digest(v) for k, v in sorted(state.items())}}
        b = oracle_block(state, mhd, de)
        prm = case_params(solver, recon, de, scheme, theta)
        dt = O.timestep(prm, b, ref=True)
        if mhd:
            O.step(prm, b, dt, ref=True)
        else:
            # hydro: the step also stores the boundary fluxes for flux
            # correction (EnzoMethodMHDVlct.cpp:250-330)
            qs = FC_QUANTITIES_DE if de else FC_QUANTITIES
            fc = O.step_fc(prm, b, dt, qs, ref=True)
            rec["fc_quantities"] = list(qs)
            rec["fc_sha256"] = {f"{ax}{side}{q}": digest(a)
                                for (ax, side, q), a in sorted(fc.items())}
        rec["dt"] = float(dt).hex()
        rec["output_sha256"] = {k: digest(b.f[ORACLE_NAME[k]]) for k in sorted(state)}
        out["cases"][name] = rec
        dens[name] = b.f["rho"].copy()
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "golden_density.npz"), **dens)
    print(f"wrote {len(out['cases'])} cases")


if __name__ == "__main__":
    main()
