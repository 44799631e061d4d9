"""The oracle's passive-scalar advection against the reference's own VL+CT
code (compiled here behind the shim; skipped where the Enzo-E tree is
absent): bit for bit, scalars in conserved form converted to mass fractions,
reconstructed like the primitives, upwinded with the density flux and updated
as start-of-step + dU (EnzoIntegrationQuanUpdate.cpp:242-270)."""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O
from helpers import oracle_params

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from golden_input import G, N, WIDTHS, golden_input  # noqa: E402

ONAME = {"density": "rho", "velocity_x": "vx", "velocity_y": "vy", "velocity_z": "vz",
         "total_energy": "etot", "internal_energy": "eint", "bfield_x": "bx",
         "bfield_y": "by", "bfield_z": "bz", "bfieldi_x": "bfx", "bfieldi_y": "bfy",
         "bfieldi_z": "bfz", "pressure": "pressure"}


def _blocks(mhd, de, seed, npass=2):
    st = golden_input(N, G, seed, mhd=mhd, dual_energy=de)
    rng = np.random.default_rng(seed + 7)
    out, pas = [], None
    for _ in range(2):
        b = O.Block(N, G, WIDTHS, mhd=mhd, dual_energy=de, npassive=npass)
        for k, v in st.items():
            if ONAME[k] in b.f:
                b.f[ONAME[k]][...] = v
        if pas is None:
            pas = [b.f["rho"] * rng.random(b.f["rho"].shape) for _ in range(npass)]
        for k in range(npass):
            b.f[f"pass{k}"][...] = pas[k]
        out.append(b)
    return out


CASES = [("hlld", "plm", False, False), ("hllc", "plm", True, False),
         ("hlle", "nn", False, False), ("hllc", "plm_athena", False, True)]


@pytest.mark.skipif(O.ref_lib() is None, reason="reference sources not built here")
@pytest.mark.parametrize("solver,recon,de,euler", CASES)
def test_oracle_passive_matches_reference(solver, recon, de, euler):
    a, b = _blocks(solver != "hllc", de, 23)
    prm = oracle_params(solver, recon, de=de, euler=euler, courant=1.0 if euler else 0.3)
    dt = O.timestep(prm, a)
    assert O.timestep(prm, b, ref=True) == dt
    O.step(prm, a, dt)
    O.step(prm, b, dt, ref=True)
    for k in a.f:
        assert np.array_equal(a.f[k], b.f[k]), k


def test_passive_scalar_mass_is_advected():
    """The scalar's total (conserved) changes only through the boundary
    fluxes: a uniform mass fraction stays uniform in the interior."""
    a, _ = _blocks(False, False, 29, npass=1)
    a.f["pass0"][...] = 0.25 * a.f["rho"]
    prm = oracle_params("hllc", "plm")
    dt = O.timestep(prm, a)
    O.step(prm, a, dt)
    g = G
    act = (slice(g, g + N[2]), slice(g, g + N[1]), slice(g, g + N[0]))
    np.testing.assert_allclose(a.f["pass0"][act] / a.f["rho"][act], 0.25, rtol=1e-12)


@pytest.mark.skipif(O.ref_lib() is None, reason="reference sources not built here")
@pytest.mark.parametrize("recon,de", [("plm", False), ("nn", True)])
def test_oracle_passive_boundary_fluxes_match_reference(recon, de):
    """store_fluxes_for_corrections with the passive scalars in the
    flux-correction group: the reference keys FluxData by field name and
    stores every field of the group (EnzoMethodMHDVlct.cpp:265-272), so each
    scalar's conserved-form boundary flux is saved beside the hydro ones."""
    a, b = _blocks(False, de, 29, npass=3)
    prm = oracle_params("hllc", recon, de=de, courant=0.3)
    dt = O.timestep(prm, a)
    assert O.timestep(prm, b, ref=True) == dt
    qs = (0, 1, 2, 3, 4) + ((5,) if de else ()) + (6, 7, 8)
    fa = O.step_fc(prm, a, dt, quantities=qs)
    fb = O.step_fc(prm, b, dt, quantities=qs, ref=True)
    assert fa.keys() == fb.keys()
    for key in fa:
        assert np.array_equal(fa[key], fb[key]), key
        if key[2] >= 6:
            assert np.count_nonzero(fa[key]) > 0, key
    for k in a.f:
        assert np.array_equal(a.f[k], b.f[k]), k


def test_oracle_step_fc_rejects_missing_scalar():
    a, _ = _blocks(False, False, 31, npass=1)
    prm = oracle_params("hllc", "plm", courant=0.3)
    with pytest.raises(RuntimeError):
        O.step_fc(prm, a, 1e-3, quantities=(0, 7))
