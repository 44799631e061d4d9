#!/usr/bin/env python3
"""TEST INFRASTRUCTURE: exact floating-point operations per zone-update of the
VL+CT cycle, counted by the op-counting build of the oracle
(oracle/_ref/liboracle_count.so: vlct_oracle.cpp with every floating type
replaced by the counting scalar of flop_count.h).

The counted cycle is the benchmark's: one 32^3 block (+3 ghosts) of the
turbulent-box recipe (HLLD + PLM, gamma 5/3, CFL 0.4, rms Mach 2), its
timestep over the whole ghosted block and one VL+CT step (both stages, every
value the reference defines, ghost ring included), divided by the 32^3
active zones.  Adds, subtracts, multiplies, divides and square roots count
one floating-point operation each; comparisons, min/max and absolute values
are reported apart.  The result goes to profiles/flops_per_zone.json, which
bench.py reads for the compute side of its roofline.

Usage:  python oracle/count_flops.py
"""
import ctypes
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# this file's own directory would shadow the oracle package by its module
sys.path = [ROOT, os.path.join(ROOT, "enzo-e_gb300")] + [
    p for p in sys.path if os.path.abspath(p or ".") != HERE]

from oracle import oracle as O  # noqa: E402
from mhdvlct import ic  # noqa: E402

KINDS = ("add_sub", "mul", "div", "sqrt", "compare", "min_max", "abs")


def counting_lib():
    subprocess.check_call(["make", "-s", "-C", HERE, "_ref/liboracle_count.so"])
    L = ctypes.CDLL(os.path.join(HERE, "_ref", "liboracle_count.so"))
    L.oracle_step.argtypes = [ctypes.POINTER(O.OracleParams), ctypes.POINTER(O.OracleBlock),
                              ctypes.c_double]
    L.oracle_step.restype = ctypes.c_int
    L.oracle_timestep.argtypes = [ctypes.POINTER(O.OracleParams), ctypes.POINTER(O.OracleBlock)]
    L.oracle_timestep.restype = ctypes.c_double
    L.oracle_op_counts.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]
    return L


def count(L, solver, recon, mhd, de, n=32):
    blocks, w = ic.turbulent_box(N=n, nb=1, g=3, seed=1, mach=2.0, dual_energy=de)
    b = O.Block(n, 3, w, mhd=mhd, dual_energy=de)
    for k, v in blocks[0].items():
        if ic.ORACLE_NAME.get(k) in b.f:
            b.f[ic.ORACLE_NAME[k]][...] = v
    prm = O.params(riemann=solver, recon=recon, mhd=mhd, dual_energy=de, courant=0.4)
    ops = (ctypes.c_ulonglong * 7)()
    L.oracle_op_counts(None, 1)
    cs = b.cstruct()
    dt = L.oracle_timestep(ctypes.byref(prm), ctypes.byref(cs))
    L.oracle_op_counts(ops, 1)
    ts = list(ops)
    O.fill_ghosts_periodic(b)
    cs = b.cstruct()
    assert L.oracle_step(ctypes.byref(prm), ctypes.byref(cs), dt) == 0
    L.oracle_op_counts(ops, 1)
    st = list(ops)
    zones = n ** 3

    def per_zone(c):
        d = {k: v / zones for k, v in zip(KINDS, c)}
        d["flops"] = sum(c[:4]) / zones
        return d
    return {"timestep": per_zone(ts), "step": per_zone(st),
            "flops_per_zone_update": (sum(ts[:4]) + sum(st[:4])) / zones}


def main():
    L = counting_lib()
    out = {"generator": "oracle/count_flops.py (op-counting build of the oracle)",
           "workload": "one 32^3 block (+3 ghosts) of the turbulent-box recipe, CFL 0.4: "
                       "timestep over the ghosted block + one VL+CT step, per active zone",
           "counting": "add/sub, mul, div, sqrt = 1 flop each; compare, min/max, abs apart",
           "configs": {}}
    for name, solver, recon, mhd, de in (("hlld_plm", O.HLLD, O.PLM, True, False),
                                         ("hlld_plm_de", O.HLLD, O.PLM, True, True),
                                         ("hllc_plm_hydro", O.HLLC, O.PLM, False, False)):
        out["configs"][name] = count(L, solver, recon, mhd, de)
        print(name, out["configs"][name]["flops_per_zone_update"])
    path = os.path.join(ROOT, "profiles", "flops_per_zone.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
