#!/usr/bin/env python3
"""Generate tests/golden/fast_wave.json from the reference's own VL+CT code:
the plain-method configuration (fast_wave_input.py: one 32^3 periodic block,
HLLD + PLM with the default limiter, CFL 0.4, FP64) run for one wave period
with Cello's cycle (timestep, clip to the stop time, periodic refresh, step).

The reference sources are compiled, unmodified, behind a shim by
`make -C oracle` into oracle/_ref/libvlct_ref.so, which needs the Enzo-E
source tree; so this script runs only where the tree exists.  It records the
SHA-256 of the input and of every field after the run, the number of cycles,
and the density's L1 distance from the initial state.  It also checks that
the restated oracle reproduces the reference's run bit for bit.

Usage:  python tests/golden/make_golden_fast_wave.py
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
from fast_wave_input import G, N, PERIOD, fast_wave_input  # noqa: E402
from golden_input import digest  # noqa: E402

ORACLE_NAME = {"density": "rho", "velocity_x": "vx", "velocity_y": "vy",
               "velocity_z": "vz", "total_energy": "etot", "bfield_x": "bx",
               "bfield_y": "by", "bfield_z": "bz", "bfieldi_x": "bfx",
               "bfieldi_y": "bfy", "bfieldi_z": "bfz", "pressure": "pressure"}
COURANT = 0.4


def params():
    return O.params(riemann=O.HLLD, recon=O.PLM, mhd=True, courant=COURANT,
                    theta_limiter=1.5, gamma=5.0 / 3.0)


def run(state, widths, ref):
    b = O.Block(N, G, widths)
    for k, v in state.items():
        b.f[ORACLE_NAME[k]][...] = v
    cycles = O.evolve_periodic(params(), b, PERIOD, ref=ref)
    return b, cycles


def main():
    if O.ref_lib() is None:
        sys.exit("oracle/_ref/libvlct_ref.so is missing: run `make -C oracle` "
                 "where the Enzo-E tree is present")
    state, widths = fast_wave_input()
    ref, cycles = run(state, widths, ref=True)
    mine, cycles_o = run(state, widths, ref=False)
    assert cycles == cycles_o
    for k, o in ORACLE_NAME.items():
        assert np.array_equal(ref.f[o], mine.f[o]), k
    act = (slice(G, G + N),) * 3
    l1 = float(np.mean(np.abs(ref.f["rho"][act] - state["density"][act])))
    out = {"generator": "tests/golden/make_golden_fast_wave.py (reference sources via "
                        "oracle/_ref)",
           "n": N, "ghost": G, "widths": list(widths), "courant": COURANT,
           "solver": "hlld", "recon": "plm", "theta": 1.5, "stop_time": PERIOD.hex(),
           "cycles": cycles,
           "input_sha256": {k: digest(v) for k, v in sorted(state.items())},
           "output_sha256": {k: digest(ref.f[o]) for k, o in sorted(ORACLE_NAME.items())},
           "density_l1_vs_initial": l1}
    with open(os.path.join(HERE, "fast_wave.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(f"{cycles} cycles; density L1 vs initial {l1:.3e}")


if __name__ == "__main__":
    main()
