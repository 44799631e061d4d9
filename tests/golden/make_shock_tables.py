#!/usr/bin/env python3
"""Copy the reference's 1D shock-tube solution tables into npz fixtures.

The reference's shock-tube regression tests compare a run against tabulated
1D solutions shipped with its input decks:
  input/vlct/MHD_shock_tube/rj2a_shock_tube_t0.2_res256.csv
  input/vlct/dual_energy_shock_tube/sod_shock_tube_t0.25_res128.csv
Those files exist only where the Enzo-E tree does, so this script stores each
table's columns, verbatim, as tests/golden/<name>.npz (with the source path
and its SHA-256) for the tests that run elsewhere.

Usage:  python tests/golden/make_shock_tables.py [ENZO_E_ROOT]
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES = {
    "rj2a_t0.2_res256": "input/vlct/MHD_shock_tube/rj2a_shock_tube_t0.2_res256.csv",
    "sod_t0.25_res128": "input/vlct/dual_energy_shock_tube/sod_shock_tube_t0.25_res128.csv",
}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    for name, rel in TABLES.items():
        path = os.path.join(root, rel)
        raw = open(path, "rb").read()
        lines = [ln for ln in raw.decode().splitlines() if ln and not ln.startswith("#")]
        cols = lines[0].split(",")
        data = np.array([[float(v) for v in ln.split(",")] for ln in lines[1:]])
        np.savez(os.path.join(HERE, f"{name}.npz"), source=rel,
                 sha256=hashlib.sha256(raw).hexdigest(), columns=np.array(cols),
                 **{c: data[:, i] for i, c in enumerate(cols)})
        print(name, data.shape, cols)


if __name__ == "__main__":
    main()
