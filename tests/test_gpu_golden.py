"""The CUDA path, through the C ABI, against the golden fixtures made by the
reference's own VL+CT sources (tests/golden/): the FP64 form reproduces the
reference's dt and every output field bit for bit; the FP32 form stays within
1e-5 relative L1 of the reference's FP64 density and 1e-6 of its dt."""
import json
import os
import sys

import numpy as np
import pytest
import torch

from mhdvlct import block as B

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from golden_input import CASES, G, N, WIDTHS, digest, golden_input  # noqa: E402
from helpers import rel_l1  # noqa: E402

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))
DENS = np.load(os.path.join(HERE, "golden", "golden_density.npz"))


def _run(case, dtype):
    name, solver, recon, de, scheme, theta, seed = case
    mhd = solver != "hllc"
    state = golden_input(N, G, seed, mhd=mhd, dual_energy=de)
    meth = B.EnzoMethodMHDVlct(
        mhd_choice="constrained_transport" if mhd else "no_bfield",
        riemann_solver=solver, reconstruct_method=recon, time_scheme=scheme,
        dual_energy=de, theta_limiter=theta)
    blk = B.Block(N, G, WIDTHS, mhd=mhd, dual_energy=de, dtype=dtype)
    blk.load_numpy(state)
    dt = meth.timestep(blk)
    meth.compute(blk, dt)
    torch.cuda.synchronize()
    return dt, blk.to_numpy()


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fp64_matches_reference_golden_bit_exact(case):
    rec = GOLD["cases"][case[0]]
    dt, out = _run(case, torch.float64)
    assert dt.hex() == rec["dt"]
    got = {k: digest(out[k]) for k in rec["output_sha256"]}
    assert got == rec["output_sha256"]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fp32_within_tolerance_of_reference_golden(case):
    rec = GOLD["cases"][case[0]]
    dt, out = _run(case, torch.float32)
    dt_ref = float.fromhex(rec["dt"])
    assert abs(dt - dt_ref) / dt_ref < 1e-6
    assert rel_l1(out["density"].astype(np.float64), DENS[case[0]]) <= 1e-5


FC_CASES = [c for c in CASES if "fc_sha256" in GOLD["cases"][c[0]]]


@pytest.mark.parametrize("case", FC_CASES, ids=[c[0] for c in FC_CASES])
def test_fp64_boundary_fluxes_match_reference_golden(case):
    name, solver, recon, de, scheme, theta, seed = case
    rec = GOLD["cases"][name]
    state = golden_input(N, G, seed, mhd=False, dual_energy=de)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver=solver,
                               reconstruct_method=recon, time_scheme=scheme,
                               dual_energy=de, theta_limiter=theta)
    blk = B.Block(N, G, WIDTHS, mhd=False, dual_energy=de, dtype=torch.float64)
    blk.load_numpy(state)
    dt = meth.timestep(blk)
    fc = meth.compute_store_fluxes(blk, dt, tuple(rec["fc_quantities"]))
    torch.cuda.synchronize()
    got = {f"{ax}{side}{q}": digest(t.cpu().numpy()) for (ax, side, q), t in sorted(fc.items())}
    assert got == rec["fc_sha256"]
    assert digest(blk.to_numpy()["density"]) == rec["output_sha256"]["density"]


# ------------------------------------------------------------ edge cases
from golden_edge_input import EDGE_CASES, N as EN, G as EG  # noqa: E402

EDGE = json.load(open(os.path.join(HERE, "golden", "golden_edge.json")))
EDGE_DENS = np.load(os.path.join(HERE, "golden", "golden_edge_density.npz"))


def _run_edge(case, dtype):
    name, solver, recon, de, eta, dfloor, pfloor, build = case
    mhd = solver != "hllc"
    state = build()
    meth = B.EnzoMethodMHDVlct(
        mhd_choice="constrained_transport" if mhd else "no_bfield",
        riemann_solver=solver, reconstruct_method=recon, dual_energy=de,
        dual_energy_eta=eta, density_floor=dfloor, pressure_floor=pfloor)
    blk = B.Block(EN, EG, WIDTHS, mhd=mhd, dual_energy=de, dtype=dtype)
    blk.load_numpy(state)
    dt = meth.timestep(blk)
    meth.compute(blk, dt)
    torch.cuda.synchronize()
    return dt, blk.to_numpy()


@pytest.mark.parametrize("case", EDGE_CASES, ids=[c[0] for c in EDGE_CASES])
def test_fp64_matches_reference_edge_golden_bit_exact(case):
    """Degenerate HLLD states, active floors and the dual-energy switch at a
    Mach-10 jump: the CUDA FP64 path reproduces the reference bit for bit."""
    rec = EDGE["cases"][case[0]]
    dt, out = _run_edge(case, torch.float64)
    assert dt.hex() == rec["dt"]
    got = {k: digest(out[k]) for k in rec["output_sha256"]}
    assert got == rec["output_sha256"]
