#!/usr/bin/env python3
"""Generate tests/golden/golden_edge.json from the reference's own VL+CT code
on the edge-case inputs of golden_edge_input.py (degenerate HLLD states,
active floors, the dual-energy switch at a Mach-10 jump).

The reference sources are compiled, unmodified, behind a shim by
`make -C oracle` into oracle/_ref/libvlct_ref.so, so this script runs only
where the Enzo-E tree exists.  Per case it records the SHA-256 of the input
and of every field after `EnzoMethodMHDVlct::timestep` and one `compute` of
that dt, the dt as a float hex string, and -- computed here in numpy from the
input, with the nearest-neighbour states of the first stage -- how many
faces and cells reach each branch the case is built for, so that the
fixture documents that the branch is really taken.

Usage:  python tests/golden/make_golden_edge.py
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
from golden_input import GAMMA, WIDTHS, digest  # noqa: E402
from golden_edge_input import EDGE_CASES, G, N  # noqa: E402
from make_golden import ORACLE_NAME, RECON, SOLVER  # noqa: E402

SMALL = 1e-8  # EnzoRiemannHLLD.hpp:20


def _hlld_x_branches(s):
    """Count the x-faces (nearest-neighbour states of the input) where HLLD
    takes its degenerate branches: |rho s (s - s_M) - B_x^2| < 1e-8 p* on the
    left star state (EnzoRiemannHLLD.hpp:203) and 0.5 B_x^2 < 1e-8 p* (:263)."""
    g = GAMMA
    rho, p = s["density"], None
    b2 = s["bfield_x"] ** 2 + s["bfield_y"] ** 2 + s["bfield_z"] ** 2
    ke = 0.5 * rho * (s["velocity_x"] ** 2 + s["velocity_y"] ** 2 + s["velocity_z"] ** 2)
    p = (g - 1.0) * (rho * s["total_energy"] - ke - 0.5 * b2)
    bxi = s["bfieldi_x"][:, :, 1:-1]
    L = (slice(None), slice(None), slice(0, -1))
    R = (slice(None), slice(None), slice(1, None))
    rl, rr, pl, pr = rho[L], rho[R], p[L], p[R]
    ul, ur = s["velocity_x"][L], s["velocity_x"][R]

    def cfast(r, pp, bj, bk):
        B2 = bxi * bxi + bj * bj + bk * bk
        cs2, va2, va2c = g * pp / r, B2 / r, bxi * bxi / r
        q = cs2 + va2
        return np.sqrt(0.5 * (va2 + cs2 + np.sqrt(q * q - 4.0 * cs2 * va2c)))

    cfl = cfast(rl, pl, s["bfield_y"][L], s["bfield_z"][L])
    cfr = cfast(rr, pr, s["bfield_y"][R], s["bfield_z"][R])
    s0 = np.minimum(ul - cfl, ur - cfr)
    s4 = np.maximum(ul + cfl, ur + cfr)
    ptl = pl + 0.5 * (bxi * bxi + s["bfield_y"][L] ** 2 + s["bfield_z"][L] ** 2)
    ptr = pr + 0.5 * (bxi * bxi + s["bfield_y"][R] ** 2 + s["bfield_z"][R] ** 2)
    sdl, sdr = s0 - ul, s4 - ur
    s2 = (sdr * rr * ur - sdl * rl * ul + (ptl - ptr)) / (sdr * rr - sdl * rl)
    ptst = 0.5 * ((ptl + rl * sdl * (s2 - ul)) + (ptr + rr * sdr * (s2 - ur)))
    star = np.abs(rl * sdl * (s0 - s2) - bxi * bxi) < SMALL * ptst
    dstar = 0.5 * bxi * bxi < SMALL * ptst
    return {"x_faces": int(star.size), "left_star_bt0": int(star.sum()),
            "double_star_bx0": int(dstar.sum())}


def _coverage(name, s, de, eta, dfloor, pfloor):
    cov = {}
    if "bfield_x" in s and "degenerate" in name:
        cov.update(_hlld_x_branches(s))
    if dfloor > 1e-100:
        cov["cells_below_density_floor"] = int((s["density"] < dfloor).sum())
    if de:
        v2 = s["velocity_x"] ** 2 + s["velocity_y"] ** 2 + s["velocity_z"] ** 2
        e_int = s["internal_energy"]
        cs2 = GAMMA * (GAMMA - 1.0) * e_int
        cov["cells_cs2_below_eta_v2"] = int((cs2 < eta * v2).sum())
        cov["cells_cs2_above_eta_v2"] = int((cs2 >= eta * v2).sum())
        cov["cells_pressure_below_floor"] = int(
            ((GAMMA - 1.0) * s["density"] * e_int < pfloor).sum())
    return cov


def case_params(solver, recon, de, eta, dfloor, pfloor):
    return O.params(riemann=SOLVER[solver], recon=RECON[recon], mhd=solver != "hllc",
                    dual_energy=de, eta=eta, theta_limiter=1.5, courant=0.3,
                    density_floor=dfloor, pressure_floor=pfloor)


def main():
    if O.ref_lib() is None:
        sys.exit("oracle/_ref/libvlct_ref.so is missing: run `make -C oracle` "
                 "where the Enzo-E tree is present")
    out = {"n": list(N), "ghost": G, "widths": list(WIDTHS),
           "generator": "tests/golden/make_golden_edge.py (reference sources via oracle/_ref)",
           "cases": {}}
    dens = {}
    for name, solver, recon, de, eta, dfloor, pfloor, build in EDGE_CASES:
        mhd = solver != "hllc"
        state = build()
        rec = {"solver": solver, "recon": recon, "dual_energy": de, "eta": eta,
               "density_floor": dfloor, "pressure_floor": pfloor,
               "input_sha256": {k: digest(v) for k, v in sorted(state.items())},
               "coverage": _coverage(name, state, de, eta, dfloor, pfloor)}
        b = O.Block(N, G, WIDTHS, mhd=mhd, dual_energy=de)
        for k, v in state.items():
            b.f[ORACLE_NAME[k]][...] = v
        prm = case_params(solver, recon, de, eta, dfloor, pfloor)
        dt = O.timestep(prm, b, ref=True)
        O.step(prm, b, dt, ref=True)
        rec["dt"] = float(dt).hex()
        rec["output_sha256"] = {k: digest(b.f[ORACLE_NAME[k]]) for k in sorted(state)}
        out["cases"][name] = rec
        dens[name] = b.f["rho"].copy()
        print(name, rec["coverage"])
    with open(os.path.join(HERE, "golden_edge.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "golden_edge_density.npz"), **dens)
    print(f"wrote {len(out['cases'])} cases")


if __name__ == "__main__":
    main()
