"""Flux correction at coarse-fine faces on the GPU through the C ABI
(mhdvlct_flux_correct), against the oracle (its coarsening pinned to the
reference's own FaceFluxes::coarsen in tests/test_flux_correct_oracle.py):

  - a static-mesh-refinement run -- mesh refresh, step with stored boundary
    fluxes, flux correction, as the reference's SMR VL decks cycle -- equals
    the oracle's run bit for bit in FP64 and conserves mass, momentum and
    total energy to round-off;
  - the FP32 correction alone equals the oracle's FP32 restatement bit for
    bit on random fields and fluxes;
  - with passive scalars in the flux-correction group (Cello corrects every
    field of its group, src/Cello/problem_MethodFluxCorrect.cpp:55-77), the
    per-block and the batched (graph-replayed) runs equal the oracle's bit
    for bit in FP64 and conserve each scalar's mass to round-off.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from mhdvlct import block as B, capi, mesh as M
from test_flux_correct_oracle import fc_fields, smr_blocks, smr_slots, totals

pytestmark = pytest.mark.gpu

NAMES = ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy")
ONAMES = ("rho", "vx", "vy", "vz", "etot")


@pytest.mark.parametrize("levels", [2, 3])
def test_smr_pipeline_bit_exact_and_conservative(levels):
    from test_flux_correct_oracle import three_level_mesh
    n, g, cycles = 8, 4, (3 if levels == 2 else 2)
    mesh, oblocks, vols = smr_blocks(n, g, three_level_mesh() if levels == 3 else None)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=0.4)
    prm = O.params(riemann=O.HLLC, recon=O.PLM, mhd=False, courant=0.4)
    blocks = []
    for ob in oblocks:
        b = B.Block((n,) * 3, g, ob.widths, mhd=False)
        b.load_numpy({k: ob.f[o] for k, o in zip(NAMES, ONAMES)})
        blocks.append(b)
    bufs = [B.FluxBuffers(b, (0, 1, 2, 3, 4)) for b in blocks]
    faces, ofaces = mesh.face_array(), mesh.face_ints()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    slots = [{0: b.f["rho"], 1: b.f["vx"], 2: b.f["vy"], 3: b.f["vz"], 4: b.f["etot"],
              9: b.f["pressure"]} for b in oblocks]
    fields = [{q: b.f[k] for q, k in enumerate(ONAMES)} for b in oblocks]
    meth.refresh_faces(blocks, faces, cons)
    O.refresh_faces(slots, (n,) * 3, (g,) * 3, ofaces, cons)
    t0 = totals(oblocks, vols, n, g)
    for _ in range(cycles):
        dts = [meth.timestep(b) for b in blocks]
        dt = min(O.timestep(prm, b) for b in oblocks)
        assert min(dts) == dt
        meth.refresh_faces(blocks, faces, cons)
        O.refresh_faces(slots, (n,) * 3, (g,) * 3, ofaces, cons)
        for b, buf in zip(blocks, bufs):
            meth.compute_store_fluxes(b, dt, (0, 1, 2, 3, 4), buffers=buf)
        fl = [O.step_fc(prm, b, dt) for b in oblocks]
        meth.flux_correct(blocks, bufs, faces, cons)
        O.flux_correct(fields, fl, (n,) * 3, (g,) * 3, ofaces, cons)
    torch.cuda.synchronize()
    for i, (b, ob) in enumerate(zip(blocks, oblocks)):
        got = b.to_numpy()
        for k, o in zip(NAMES, ONAMES):
            assert np.array_equal(got[k], ob.f[o]), (i, k)
    t1 = totals(oblocks, vols, n, g)
    assert float((np.abs(t1 - t0) / np.abs(t0)).max()) < 1e-15


def test_fp32_correction_bit_exact():
    n, g = 8, 4
    mesh = M.Mesh((2, 2, 2), refine=lambda lvl, c: c == (0, 0, 0))
    rng = np.random.default_rng(31)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               dual_energy=True)
    blocks, bufs, ofields, ofluxes, inputs = [], [], [], [], []
    m = n + 2 * g
    for _ in mesh.leaves:
        st = {"density": 0.5 + rng.random((m, m, m))}
        for k in ("velocity_x", "velocity_y", "velocity_z", "total_energy",
                  "internal_energy"):
            st[k] = rng.standard_normal((m, m, m))
        st = {k: v.astype(np.float32) for k, v in st.items()}
        b = B.Block((n,) * 3, g, (1.0, 1.0, 1.0), mhd=False, dual_energy=True,
                    dtype=torch.float32)
        b.load_numpy(st)
        buf = B.FluxBuffers(b, (0, 1, 2, 3, 4, 5))
        fx = {}
        for key, t in buf.arrays.items():
            a = rng.standard_normal(tuple(t.shape)).astype(np.float32)
            t.copy_(torch.from_numpy(a))
            fx[key] = a
        blocks.append(b)
        bufs.append(buf)
        ofields.append({q: st[k].copy() for q, k in enumerate(NAMES + ("internal_energy",))})
        inputs.append(st["density"].copy())
        ofluxes.append(fx)
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    meth.flux_correct(blocks, bufs, mesh.face_array(), cons)
    torch.cuda.synchronize()
    O.flux_correct(ofields, ofluxes, (n,) * 3, (g,) * 3, mesh.face_ints(), cons)
    changed = 0
    for i, b in enumerate(blocks):
        got = b.to_numpy()
        for q, k in enumerate(NAMES + ("internal_energy",)):
            assert np.array_equal(got[k], ofields[i][q]), (i, k)
        changed += int(np.count_nonzero(got["density"] != inputs[i]))
    # the correction touched the coarse blocks' boundary cells next to the
    # refined region (7 coarse blocks, 3 corrected faces of 8x8 cells each)
    assert changed > 0


def test_batch_graph_with_flux_correction_bit_exact():
    # the batched form: refresh across levels, the two stages (storing the
    # boundary fluxes) and the flux correction replayed as one CUDA graph
    from test_gpu_batch import Batch
    n, g, cycles = 8, 4, 3
    mesh, oblocks, vols = smr_blocks(n, g)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=0.4)
    prm = O.params(riemann=O.HLLC, recon=O.PLM, mhd=False, courant=0.4)
    L = capi.lib()
    bt = Batch(meth, [(n,) * 3] * len(oblocks), [ob.widths for ob in oblocks], ghost=g)
    for i, ob in enumerate(oblocks):
        bt.upload(i, {k: ob.f[o] for k, o in zip(NAMES, ONAMES)})
    farr, nf = mesh.face_array()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    capi.check(L.mhdvlct_batch_set_refresh_faces(bt.h, farr, nf, cons), meth.handle, "faces")
    capi.check(L.mhdvlct_batch_set_flux_correction(bt.h, 0b11111, farr, nf, cons),
               meth.handle, "flux correction")
    capi.check(L.mhdvlct_batch_refresh(bt.h, None), meth.handle, "refresh")
    capi.check(L.mhdvlct_batch_run(bt.h, cycles, 0, None, None), meth.handle, "run")
    # the oracle's run with the correction
    faces = mesh.face_ints()
    slots = [{0: b.f["rho"], 1: b.f["vx"], 2: b.f["vy"], 3: b.f["vz"], 4: b.f["etot"],
              9: b.f["pressure"]} for b in oblocks]
    fields = [{q: b.f[k] for q, k in enumerate(ONAMES)} for b in oblocks]
    O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
    for _ in range(cycles):
        dt = min(O.timestep(prm, b) for b in oblocks)
        O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
        fl = [O.step_fc(prm, b, dt) for b in oblocks]
        O.flux_correct(fields, fl, (n,) * 3, (g,) * 3, faces, cons)
    for i, ob in enumerate(oblocks):
        got = bt.download(i)
        for k, o in zip(NAMES, ONAMES):
            assert np.array_equal(got[k], ob.f[o]), (i, k)
    # and hydro only, as the reference
    mhd = B.EnzoMethodMHDVlct()
    bm = Batch(mhd, [(n,) * 3], [(1.0, 1.0, 1.0)], ghost=g)
    assert L.mhdvlct_batch_set_flux_correction(bm.h, 1, farr, nf, cons) == capi.MHD_ERR_INVALID


def test_batch_fp32_with_flux_correction_close_to_fp64_oracle():
    # the benchmarked form: FP32 batch with the correction in the graph, two
    # cycles against the FP64 oracle (relative L1 over the active cells)
    from test_gpu_batch import Batch
    n, g, cycles = 8, 4, 2
    mesh, oblocks, vols = smr_blocks(n, g)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=0.4)
    prm = O.params(riemann=O.HLLC, recon=O.PLM, mhd=False, courant=0.4)
    L = capi.lib()
    bt = Batch(meth, [(n,) * 3] * len(oblocks), [ob.widths for ob in oblocks],
               dtype=capi.MHD_DTYPE_F32, ghost=g)
    for i, ob in enumerate(oblocks):
        bt.upload(i, {k: ob.f[o] for k, o in zip(NAMES, ONAMES)})
    farr, nf = mesh.face_array()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    capi.check(L.mhdvlct_batch_set_refresh_faces(bt.h, farr, nf, cons), meth.handle, "faces")
    capi.check(L.mhdvlct_batch_set_flux_correction(bt.h, 0b11111, farr, nf, cons),
               meth.handle, "flux correction")
    capi.check(L.mhdvlct_batch_refresh(bt.h, None), meth.handle, "refresh")
    capi.check(L.mhdvlct_batch_run(bt.h, cycles, 0, None, None), meth.handle, "run")
    faces = mesh.face_ints()
    slots = [{0: b.f["rho"], 1: b.f["vx"], 2: b.f["vy"], 3: b.f["vz"], 4: b.f["etot"],
              9: b.f["pressure"]} for b in oblocks]
    fields = [{q: b.f[k] for q, k in enumerate(ONAMES)} for b in oblocks]
    O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
    for _ in range(cycles):
        dt = min(O.timestep(prm, b) for b in oblocks)
        O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
        fl = [O.step_fc(prm, b, dt) for b in oblocks]
        O.flux_correct(fields, fl, (n,) * 3, (g,) * 3, faces, cons)
    act = (slice(g, g + n),) * 3
    for i, ob in enumerate(oblocks):
        got = bt.download(i)
        for k, o in zip(NAMES, ONAMES):
            want = ob.f[o][act]
            err = np.abs(got[k][act].astype(np.float64) - want).sum() / np.abs(want).sum()
            assert err <= 1e-5, (i, k, err)


NPASS = 2
PNAMES = tuple(f"passive_{k}" for k in range(NPASS))
PONAMES = tuple(f"pass{k}" for k in range(NPASS))
PQS = (0, 1, 2, 3, 4) + tuple(capi.MHD_Q_PASSIVE_0 + k for k in range(NPASS))


def _oracle_passive_run(mesh, oblocks, n, g, cycles, cons):
    prm = O.params(riemann=O.HLLC, recon=O.PLM, mhd=False, courant=0.4)
    faces = mesh.face_ints()
    slots = [smr_slots(b, NPASS) for b in oblocks]
    fields = [fc_fields(b, NPASS) for b in oblocks]
    O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
    dts = []
    for _ in range(cycles):
        dt = min(O.timestep(prm, b) for b in oblocks)
        O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
        fl = [O.step_fc(prm, b, dt, quantities=PQS) for b in oblocks]
        O.flux_correct(fields, fl, (n,) * 3, (g,) * 3, faces, cons)
        dts.append(dt)
    return dts


def test_smr_passive_per_block_bit_exact_and_conservative():
    n, g, cycles = 8, 4, 2
    mesh, oblocks, vols = smr_blocks(n, g, npassive=NPASS)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=0.4)
    blocks = []
    for ob in oblocks:
        b = B.Block((n,) * 3, g, ob.widths, mhd=False, npassive=NPASS)
        b.load_numpy({k: ob.f[o] for k, o in zip(NAMES + PNAMES, ONAMES + PONAMES)})
        blocks.append(b)
    bufs = [B.FluxBuffers(b, PQS) for b in blocks]
    faces = mesh.face_array()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    t0 = None
    meth.refresh_faces(blocks, faces, cons)
    for _ in range(cycles):
        dt = min(meth.timestep(b) for b in blocks)
        meth.refresh_faces(blocks, faces, cons)
        for b, buf in zip(blocks, bufs):
            meth.compute_store_fluxes(b, dt, PQS, buffers=buf)
        meth.flux_correct(blocks, bufs, faces, cons)
    torch.cuda.synchronize()
    # the oracle's run from the same initial state
    _, ob0, _ = smr_blocks(n, g, npassive=NPASS)
    O.refresh_faces([smr_slots(b, NPASS) for b in ob0], (n,) * 3, (g,) * 3,
                    mesh.face_ints(), cons)
    t0 = totals(ob0, vols, n, g, NPASS)
    _oracle_passive_run(mesh, oblocks, n, g, cycles, cons)
    for i, (b, ob) in enumerate(zip(blocks, oblocks)):
        got = b.to_numpy()
        for k, o in zip(NAMES + PNAMES, ONAMES + PONAMES):
            assert np.array_equal(got[k], ob.f[o]), (i, k)
    t1 = totals(oblocks, vols, n, g, NPASS)
    assert float((np.abs(t1 - t0) / np.abs(t0)).max()) < 1e-15


def test_batch_graph_passive_flux_correction_bit_exact():
    from test_gpu_batch import Batch
    n, g, cycles = 8, 4, 3
    mesh, oblocks, vols = smr_blocks(n, g, npassive=NPASS)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=0.4)
    L = capi.lib()
    bt = Batch(meth, [(n,) * 3] * len(oblocks), [ob.widths for ob in oblocks], ghost=g,
               npassive=NPASS)
    for i, ob in enumerate(oblocks):
        bt.upload(i, {k: ob.f[o] for k, o in zip(NAMES + PNAMES, ONAMES + PONAMES)})
    farr, nf = mesh.face_array()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    qmask = sum(1 << q for q in PQS)
    capi.check(L.mhdvlct_batch_set_refresh_faces(bt.h, farr, nf, cons), meth.handle, "faces")
    # a scalar the batch lacks is refused
    assert L.mhdvlct_batch_set_flux_correction(
        bt.h, qmask | (1 << (capi.MHD_Q_PASSIVE_0 + NPASS)), farr, nf,
        cons) == capi.MHD_ERR_INVALID
    capi.check(L.mhdvlct_batch_set_flux_correction(bt.h, qmask, farr, nf, cons),
               meth.handle, "flux correction")
    capi.check(L.mhdvlct_batch_refresh(bt.h, None), meth.handle, "refresh")
    capi.check(L.mhdvlct_batch_run(bt.h, cycles, 0, None, None), meth.handle, "run")
    _oracle_passive_run(mesh, oblocks, n, g, cycles, cons)
    for i, ob in enumerate(oblocks):
        got = bt.download(i)
        for k, o in zip(NAMES + PNAMES, ONAMES + PONAMES):
            assert np.array_equal(got[k], ob.f[o]), (i, k)


def test_fp32_passive_correction_bit_exact_with_conservative_scalar():
    # the correction alone on random fields and fluxes, with two passive
    # scalars in the group; scalar 1 is in the "make_field_conservative"
    # mask (field bit MHD_FIELD_PASSIVE_0 + 1), so it is corrected as
    # old density x value, divided by the corrected density
    n, g = 8, 4
    mesh = M.Mesh((2, 2, 2), refine=lambda lvl, c: c == (0, 0, 0))
    rng = np.random.default_rng(37)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc")
    qs = (0, 1, 2, 3, 4) + tuple(capi.MHD_Q_PASSIVE_0 + k for k in range(NPASS))
    keys = NAMES + PNAMES
    blocks, bufs, ofields, ofluxes = [], [], [], []
    m = n + 2 * g
    for _ in mesh.leaves:
        st = {"density": 0.5 + rng.random((m, m, m))}
        for k in keys[1:]:
            st[k] = rng.standard_normal((m, m, m))
        st = {k: v.astype(np.float32) for k, v in st.items()}
        b = B.Block((n,) * 3, g, (1.0, 1.0, 1.0), mhd=False, dtype=torch.float32,
                    npassive=NPASS)
        b.load_numpy(st)
        buf = B.FluxBuffers(b, qs)
        fx = {}
        for key, t in buf.arrays.items():
            a = rng.standard_normal(tuple(t.shape)).astype(np.float32)
            t.copy_(torch.from_numpy(a))
            fx[key] = a
        blocks.append(b)
        bufs.append(buf)
        of = {q: st[k].copy() for q, k in enumerate(NAMES)}
        for k in range(NPASS):
            of[capi.MHD_Q_PASSIVE_0 + k] = st[PNAMES[k]].copy()
        ofields.append(of)
        ofluxes.append(fx)
    cons = capi.MHD_CONSERVATIVE_DEFAULT | (1 << (capi.MHD_FIELD_PASSIVE_0 + 1))
    # the oracle takes the mask in its own slots (MHD_Q_*)
    ocons = capi.MHD_CONSERVATIVE_DEFAULT | (1 << (capi.MHD_Q_PASSIVE_0 + 1))
    meth.flux_correct(blocks, bufs, mesh.face_array(), cons)
    torch.cuda.synchronize()
    O.flux_correct(ofields, ofluxes, (n,) * 3, (g,) * 3, mesh.face_ints(), ocons)
    for i, b in enumerate(blocks):
        got = b.to_numpy()
        for q, k in enumerate(NAMES):
            assert np.array_equal(got[k], ofields[i][q]), (i, k)
        for k in range(NPASS):
            assert np.array_equal(got[PNAMES[k]], ofields[i][capi.MHD_Q_PASSIVE_0 + k]), (i, k)
