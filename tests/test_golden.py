"""The oracle pinned against the committed golden fixtures (tests/golden/),
which tests/golden/make_golden.py made by running the reference's own VL+CT
sources (compiled unmodified behind a shim) on seeded inputs.  The oracle
must reproduce the reference's dt and every output field bit for bit."""
import json
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from golden_input import CASES, G, N, WIDTHS, digest, golden_input  # noqa: E402
from helpers import oracle_block, oracle_params  # noqa: E402

GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))
DENS = np.load(os.path.join(HERE, "golden", "golden_density.npz"))


def test_fixture_covers_every_case():
    assert sorted(GOLD["cases"]) == sorted(c[0] for c in CASES)
    assert tuple(GOLD["n"]) == N and GOLD["ghost"] == G


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_reference_golden(case):
    name, solver, recon, de, scheme, theta, seed = case
    rec = GOLD["cases"][name]
    mhd = solver != "hllc"
    state = golden_input(N, G, seed, mhd=mhd, dual_energy=de)
    # the seeded input is the same bits everywhere
    assert {k: digest(v) for k, v in state.items()} == rec["input_sha256"]
    b = oracle_block(state, N, G, WIDTHS, mhd=mhd, de=de)
    prm = oracle_params(solver, recon, de=de, euler=scheme == "euler", theta=theta,
                        courant=1.0 if scheme == "euler" else 0.3)
    dt = O.timestep(prm, b)
    assert dt.hex() == rec["dt"]
    O.step(prm, b, dt)
    got = {k: digest(b.f[O_NAME[k]]) for k in rec["output_sha256"]}
    assert got == rec["output_sha256"]
    assert np.array_equal(b.f["rho"], DENS[name])


O_NAME = {"density": "rho", "velocity_x": "vx", "velocity_y": "vy",
          "velocity_z": "vz", "total_energy": "etot", "internal_energy": "eint",
          "bfield_x": "bx", "bfield_y": "by", "bfield_z": "bz", "bfieldi_x": "bfx",
          "bfieldi_y": "bfy", "bfieldi_z": "bfz", "pressure": "pressure"}


def test_oracle_rejects_euler_with_constrained_transport():
    state = golden_input(N, G, 1, mhd=True)
    b = oracle_block(state, N, G, WIDTHS, mhd=True)
    prm = oracle_params("hlld", "nn", euler=True, courant=1.0)
    with pytest.raises(RuntimeError):
        O.step(prm, b, 1e-3)


FC_CASES = [c for c in CASES if "fc_sha256" in GOLD["cases"][c[0]]]


@pytest.mark.parametrize("case", FC_CASES, ids=[c[0] for c in FC_CASES])
def test_oracle_boundary_fluxes_match_reference_golden(case):
    """store_fluxes_for_corrections: the dt/dx-scaled fluxes through the
    active boundary faces equal the reference's bit for bit."""
    name, solver, recon, de, scheme, theta, seed = case
    rec = GOLD["cases"][name]
    state = golden_input(N, G, seed, mhd=False, dual_energy=de)
    b = oracle_block(state, N, G, WIDTHS, mhd=False, de=de)
    prm = oracle_params(solver, recon, de=de, euler=scheme == "euler", theta=theta,
                        courant=1.0 if scheme == "euler" else 0.3)
    dt = O.timestep(prm, b)
    fc = O.step_fc(prm, b, dt, tuple(rec["fc_quantities"]))
    got = {f"{ax}{side}{q}": digest(a) for (ax, side, q), a in sorted(fc.items())}
    assert got == rec["fc_sha256"]
    assert np.array_equal(b.f["rho"], DENS[name])


def test_oracle_flux_correction_rejects_mhd():
    state = golden_input(N, G, 1, mhd=True)
    b = oracle_block(state, N, G, WIDTHS, mhd=True)
    with pytest.raises(RuntimeError):
        O.step_fc(oracle_params("hlld", "plm"), b, 1e-3)


# ------------------------------------------------------------ edge cases
from golden_edge_input import EDGE_CASES, N as EN, G as EG  # noqa: E402

EDGE = json.load(open(os.path.join(HERE, "golden", "golden_edge.json")))
EDGE_DENS = np.load(os.path.join(HERE, "golden", "golden_edge_density.npz"))


def test_edge_fixture_covers_every_case_and_branch():
    assert sorted(EDGE["cases"]) == sorted(c[0] for c in EDGE_CASES)
    for name, rec in EDGE["cases"].items():
        cov = rec["coverage"]
        # each case reaches the branches it is built for (counted on the input)
        if "degenerate" in name:
            assert cov["left_star_bt0"] > 0 and cov["double_star_bx0"] > 0, name
        if "vacuum" in name:
            assert cov["cells_below_density_floor"] > 0, name
        if rec["dual_energy"]:
            assert cov["cells_cs2_below_eta_v2"] > 0 and cov["cells_cs2_above_eta_v2"] > 0, name


@pytest.mark.parametrize("case", EDGE_CASES, ids=[c[0] for c in EDGE_CASES])
def test_oracle_matches_reference_edge_golden(case):
    """Degenerate HLLD states, active floors at the reference decks' values
    and the dual-energy switch both ways: the oracle reproduces the
    reference's dt and every field bit for bit, and the result is finite."""
    name, solver, recon, de, eta, dfloor, pfloor, build = case
    rec = EDGE["cases"][name]
    mhd = solver != "hllc"
    state = build()
    assert {k: digest(v) for k, v in state.items()} == rec["input_sha256"]
    b = oracle_block(state, EN, EG, WIDTHS, mhd=mhd, de=de)
    prm = oracle_params(solver, recon, de=de, eta=eta, dfloor=dfloor, pfloor=pfloor)
    dt = O.timestep(prm, b)
    assert dt.hex() == rec["dt"]
    O.step(prm, b, dt)
    got = {k: digest(b.f[O_NAME[k]]) for k in rec["output_sha256"]}
    assert got == rec["output_sha256"]
    assert np.array_equal(b.f["rho"], EDGE_DENS[name])
    assert all(np.isfinite(b.f[O_NAME[k]]).all() for k in rec["output_sha256"])
