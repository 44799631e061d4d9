"""Flux correction at coarse-fine faces on the CPU (Cello's "flux_correct"
Method after a VL+CT step that stored its boundary fluxes):

  - the oracle's coarsening of a finer block's face fluxes equals the
    reference's own FaceFluxes::coarsen (src/Cello/data_FaceFluxes.cpp),
    compiled here, bit for bit, for every axis, side and child quarter;
  - a static-mesh-refinement run of the oracle (mesh refresh, step with
    stored fluxes, flux correction; periodic, hydro) conserves mass,
    momentum and total energy to round-off, as the reference's SMR VL
    regression (FluxCorrect-SMR-VL, min_digits about 16 in FP64) expects,
    and without the correction it does not.
"""
import itertools

import numpy as np
import pytest

from oracle import oracle as O
from mhdvlct import capi, mesh as M

N3 = (8, 6, 4)


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("face", [0, 1])
def test_coarsen_matches_reference(axis, face):
    if O.refresh_ref_lib() is None:
        pytest.skip("reference sources not built here")
    a_in = 1 if axis == 0 else 0
    a_out = 1 if axis == 2 else 2
    ni, no = N3[a_in], N3[a_out]
    rng = np.random.default_rng(7 * axis + face)
    for ci, co in itertools.product((0, 1), repeat=2):
        fine = rng.standard_normal((no, ni))
        mine = O.coarsen_fluxes(fine, ci, co)
        ref = O.coarsen_fluxes(fine, ci, co, ref=True, n=N3, axis=axis, face=face)
        assert np.array_equal(mine, ref), (ci, co)
        assert np.count_nonzero(mine) == (ni // 2) * (no // 2)


def three_level_mesh():
    """A 4^3 periodic root grid, its central 2^3 refined, the centre of that
    region refined again."""
    def refine(lvl, c):
        if lvl == 0:
            return all(1 <= x < 3 for x in c)
        return lvl == 1 and all(3 <= x < 5 for x in c)
    return M.Mesh((4, 4, 4), refine=refine, max_level=2)


def smr_blocks(n=8, g=4, mesh=None, npassive=0):
    """A moving density contact on a periodic mesh (default: a 2x2x2 root
    grid with one root block refined): oracle blocks (hydro) and their cell
    volumes.  Passive scalar k (conserved form) is the density times a
    mass fraction varying along a different direction."""
    if mesh is None:
        mesh = M.Mesh((2, 2, 2), refine=lambda lvl, c: c == (0, 0, 0))
    root = mesh.root[0]
    blocks, vols = [], []
    for i, (lvl, _) in enumerate(mesh.leaves):
        h = 1.0 / (root * n) / 2 ** lvl
        fine = 1.0 / (root * n) / 2 ** mesh.max_level
        o = [x * fine for x in mesh.origin(i, (n, n, n))]
        ax = [o[a] + (np.arange(n + 2 * g) - g + 0.5) * h for a in range(3)]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        b = O.Block(n, g, (h, h, h), mhd=False, npassive=npassive)
        rho = 1.0 + 0.5 * np.sin(2 * np.pi * (x + 2 * y + 3 * z))
        b.f["rho"][...] = rho
        for k in range(npassive):
            frac = 0.5 + 0.4 * np.cos(2 * np.pi * ((3 - k) * x + (k + 1) * y - z))
            b.f[f"pass{k}"][...] = rho * frac
        b.f["vx"][...] = 0.4
        b.f["vy"][...] = -0.3
        b.f["vz"][...] = 0.2
        b.f["etot"][...] = 0.6 / (2.0 / 3.0) / rho + 0.5 * (0.16 + 0.09 + 0.04)
        blocks.append(b)
        vols.append(h ** 3)
    return mesh, blocks, vols


def totals(blocks, vols, n, g, npassive=0):
    """Mass, x/y/z momentum, total energy and each passive scalar's mass."""
    act = (slice(g, g + n),) * 3
    out = np.zeros(5 + npassive, dtype=np.longdouble)
    for b, v in zip(blocks, vols):
        rho = b.f["rho"][act].astype(np.longdouble)
        out[0] += rho.sum() * v
        for k, key in enumerate(("vx", "vy", "vz")):
            out[1 + k] += (rho * b.f[key][act]).sum() * v
        out[4] += (rho * b.f["etot"][act]).sum() * v
        for k in range(npassive):
            out[5 + k] += b.f[f"pass{k}"][act].astype(np.longdouble).sum() * v
    return out


def smr_slots(b, npassive=0):
    """The refreshed fields of an oracle block by mesh field slot (passive
    scalar k at slot 13 + k)."""
    s = {0: b.f["rho"], 1: b.f["vx"], 2: b.f["vy"], 3: b.f["vz"], 4: b.f["etot"],
         9: b.f["pressure"]}
    for k in range(npassive):
        s[capi.MHD_FIELD_PASSIVE_0 + k] = b.f[f"pass{k}"]
    return s


def fc_fields(b, npassive=0):
    """The corrected fields of an oracle block by flux-correction slot
    (passive scalar k at slot 6 + k)."""
    f = {q: b.f[k] for q, k in enumerate(O.FC_FIELDS[:5])}
    for k in range(npassive):
        f[capi.MHD_Q_PASSIVE_0 + k] = b.f[f"pass{k}"]
    return f


def run(correct, cycles=3, n=8, g=4, mesh=None, npassive=0):
    mesh, blocks, vols = smr_blocks(n, g, mesh, npassive)
    prm = O.params(riemann=O.HLLC, recon=O.PLM, mhd=False, courant=0.4)
    faces = mesh.face_ints()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    slots = [smr_slots(b, npassive) for b in blocks]
    fields = [fc_fields(b, npassive) for b in blocks]
    qs = (0, 1, 2, 3, 4) + tuple(capi.MHD_Q_PASSIVE_0 + k for k in range(npassive))
    O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
    t0 = totals(blocks, vols, n, g, npassive)
    for _ in range(cycles):
        dt = min(O.timestep(prm, b) for b in blocks)
        O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
        fl = [O.step_fc(prm, b, dt, quantities=qs) for b in blocks]
        if correct:
            O.flux_correct(fields, fl, (n,) * 3, (g,) * 3, faces, cons)
    t1 = totals(blocks, vols, n, g, npassive)
    return t0, t1


def test_smr_run_conserves_with_flux_correction():
    t0, t1 = run(correct=True)
    rel = np.abs(t1 - t0) / np.abs(t0)
    # mass, x/y/z momentum, total energy: round-off only (15 digits or more)
    assert float(rel.max()) < 1e-15, rel
    t0u, t1u = run(correct=False)
    relu = np.abs(t1u - t0u) / np.abs(t0u)
    assert float(relu[0]) > 1e3 * float(rel[0]), (relu, rel)


def test_three_level_run_conserves_with_flux_correction():
    # level-1 blocks are corrected from their level-2 neighbours and
    # themselves correct level-0 ones
    t0, t1 = run(correct=True, cycles=2, mesh=three_level_mesh())
    rel = np.abs(t1 - t0) / np.abs(t0)
    assert float(rel.max()) < 1e-15, rel


def test_smr_run_conserves_passive_scalars_with_flux_correction():
    # the passive scalars in the flux-correction group, as Cello corrects
    # every field of its group (src/Cello/problem_MethodFluxCorrect.cpp:55-77):
    # each scalar's mass is conserved to round-off, and not without it
    t0, t1 = run(correct=True, npassive=2)
    rel = np.abs(t1 - t0) / np.abs(t0)
    assert float(rel.max()) < 1e-15, rel
    t0u, t1u = run(correct=False, npassive=2)
    relu = np.abs(t1u - t0u) / np.abs(t0u)
    for k in (5, 6):
        assert float(relu[k]) > 1e3 * max(float(rel[k]), 1e-18), (relu, rel)
