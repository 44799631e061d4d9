"""The oracle's gravity source against the reference's own VL+CT code
(compiled here behind the shim; skipped where the Enzo-E tree is absent):
bit for bit, applied on the full-dt stage of vl only."""
import numpy as np
import pytest

from oracle import oracle as O
from helpers import oracle_params

import sys, os
sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from golden_input import G, N, WIDTHS, golden_input  # noqa: E402

ONAME = {"density": "rho", "velocity_x": "vx", "velocity_y": "vy", "velocity_z": "vz",
         "total_energy": "etot", "internal_energy": "eint", "bfield_x": "bx",
         "bfield_y": "by", "bfield_z": "bz", "bfieldi_x": "bfx", "bfieldi_y": "bfy",
         "bfieldi_z": "bfz", "pressure": "pressure"}


def _blocks(mhd, de, seed):
    st = golden_input(N, G, seed, mhd=mhd, dual_energy=de)
    rng = np.random.default_rng(seed + 100)
    out = []
    acc = None
    for _ in range(2):
        b = O.Block(N, G, WIDTHS, mhd=mhd, dual_energy=de, gravity=True)
        for k, v in st.items():
            if ONAME[k] in b.f:
                b.f[ONAME[k]][...] = v
        if acc is None:
            acc = [0.3 * (rng.random(b.f["rho"].shape) - 0.5) for _ in range(3)]
        for k, a in zip(("ax", "ay", "az"), acc):
            b.f[k][...] = a
        out.append(b)
    return out


@pytest.mark.skipif(O.ref_lib() is None, reason="reference sources not built here")
@pytest.mark.parametrize("solver,de,euler", [("hlld", False, False), ("hllc", True, False),
                                             ("hlld", True, False), ("hllc", False, True)])
def test_oracle_gravity_matches_reference(solver, de, euler):
    mhd = solver != "hllc"
    a, b = _blocks(mhd, de, 13)
    prm = oracle_params(solver, "plm", de=de, euler=euler, courant=1.0 if euler else 0.3)
    dt = O.timestep(prm, a)
    assert O.timestep(prm, b, ref=True) == dt
    O.step(prm, a, dt)
    O.step(prm, b, dt, ref=True)
    for k in a.f:
        assert np.array_equal(a.f[k], b.f[k]), k


def test_gravity_changes_vl_not_euler():
    for euler, expect_change in ((False, True), (True, False)):
        a, _ = _blocks(False, False, 17)
        c = O.Block(N, G, WIDTHS, mhd=False)
        for k in c.f:
            c.f[k][...] = a.f[k]
        prm = oracle_params("hllc", "plm", euler=euler, courant=1.0 if euler else 0.3)
        dt = O.timestep(prm, a)
        O.timestep(prm, c)
        O.step(prm, a, dt)
        O.step(prm, c, dt)
        changed = not np.array_equal(a.f["vx"], c.f["vx"])
        assert changed == expect_change
