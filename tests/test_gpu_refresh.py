"""The mesh ghost refresh on the GPU through the C ABI
(mhdvlct_refresh_faces), against the oracle (itself pinned bit for bit to
the reference's own Box / ProlongLinear / RestrictLinear in
tests/test_refresh_oracle.py):

  - a two-level hydro mesh (copies, restrictions, prolongations; density
    weighting on and off), FP64 and FP32: bit-exact;
  - a one-level MHD mesh including face-centred B: bit-exact;
  - one periodic block refreshed from itself equals mhdvlct_fill_ghosts_periodic;
  - a static-mesh-refinement run -- global dt, refresh, VL+CT step of every
    leaf at its own cell width, as Cello cycles -- equals the oracle's run bit
    for bit in FP64 over several cycles, through the per-block Method calls
    and through the batched form with the face-list refresh replayed inside
    its CUDA graph.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from mhdvlct import block as B, capi, ic, mesh as M
from helpers import HYDRO_SLOTS, MHD_SLOTS, mesh_blocks, oracle_params

pytestmark = pytest.mark.gpu

SLOT_NAME = capi.FIELD_SLOTS


def _gpu_blocks(np_blocks, n, g, dtype, mhd, de, npass):
    out = []
    for nb in np_blocks:
        b = B.Block(n, g, (1.0, 1.0, 1.0), mhd=mhd, dual_energy=de, dtype=dtype,
                    npassive=npass)
        b.load_numpy({SLOT_NAME[s]: a for s, a in nb.items()})
        out.append(b)
    return out


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("cons", [capi.MHD_CONSERVATIVE_DEFAULT, 0])
@pytest.mark.parametrize("n", [(8, 8, 8), (8, 12, 16)])
def test_two_level_refresh_bit_exact(dtype, cons, n):
    mesh = M.Mesh((2, 2, 2), refine=lambda lvl, c: c == (0, 0, 0))
    g = 4
    npdt = np.float64 if dtype == torch.float64 else np.float32
    ref = mesh_blocks(len(mesh.leaves), n, g, HYDRO_SLOTS, npdt, seed=13)
    blocks = _gpu_blocks(ref, n, g, dtype, mhd=False, de=True, npass=1)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc", dual_energy=True)
    meth.refresh_faces(blocks, mesh.face_array(), conservative=cons)
    torch.cuda.synchronize()
    O.refresh_faces(ref, n, (g,) * 3, mesh.face_ints(), cons)
    for i, (b, r) in enumerate(zip(blocks, ref)):
        got = b.to_numpy()
        for s, a in r.items():
            assert np.array_equal(got[SLOT_NAME[s]], a, equal_nan=True), (i, SLOT_NAME[s])


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_one_level_mhd_refresh_bit_exact(dtype):
    mesh = M.Mesh((2, 1, 2))
    n, g = (8, 12, 6), 3
    npdt = np.float64 if dtype == torch.float64 else np.float32
    ref = mesh_blocks(len(mesh.leaves), n, g, MHD_SLOTS, npdt, seed=4)
    blocks = _gpu_blocks(ref, n, g, dtype, mhd=True, de=True, npass=1)
    meth = B.EnzoMethodMHDVlct(dual_energy=True)
    meth.refresh_faces(blocks, mesh.faces())
    torch.cuda.synchronize()
    O.refresh_faces(ref, n, (g,) * 3, mesh.face_ints(), capi.MHD_CONSERVATIVE_DEFAULT)
    for i, (b, r) in enumerate(zip(blocks, ref)):
        got = b.to_numpy()
        for s, a in r.items():
            assert np.isfinite(a).all(), (i, SLOT_NAME[s])
            assert np.array_equal(got[SLOT_NAME[s]], a), (i, SLOT_NAME[s])


def test_single_periodic_block_matches_fill_ghosts():
    state, w = ic.smooth_block((8, 7, 6), 3, seed=21)
    meth = B.EnzoMethodMHDVlct()
    a = B.Block((8, 7, 6), 3, w)
    b = B.Block((8, 7, 6), 3, w)
    a.load_numpy(state)
    b.load_numpy(state)
    meth.fill_ghosts_periodic(a)
    meth.refresh_faces([b], M.Mesh((1, 1, 1)).faces())
    torch.cuda.synchronize()
    x, y = a.to_numpy(), b.to_numpy()
    for k in x:
        if k == "pressure":
            continue  # [w] scratch: the periodic fill leaves it alone
        assert np.array_equal(x[k], y[k]), k


def _smr_case(de):
    """An inclined density contact on a 2x2x2 root grid of 16^3 blocks with
    one root block refined, as the reference's flux-correction SMR decks
    (input/FluxCorrect/inclined_contact*.in, ghost depth 4)."""
    mesh = M.Mesh((2, 2, 2), refine=lambda lvl, c: c == (0, 0, 0))
    n, g = (16, 16, 16), 4
    domain = 1.0
    states, widths = [], []
    for i, (lvl, _) in enumerate(mesh.leaves):
        h = domain / (2 * n[0]) / 2 ** lvl
        o = [x * domain / (2 * n[0] * 2 ** mesh.max_level) for x in mesh.origin(i, n)]
        ax = [o[a] + (np.arange(n[a] + 2 * g) - g + 0.5) * h for a in range(3)]
        z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
        phase = 2 * np.pi * (x + y + z) / domain
        rho = 1.0 + 0.5 * np.sin(phase)
        v = 0.3
        st = {"density": rho, "velocity_x": np.full_like(rho, v),
              "velocity_y": np.full_like(rho, v), "velocity_z": np.full_like(rho, v),
              "pressure": np.full_like(rho, 0.6)}
        eint = 0.6 / (2.0 / 3.0) / rho
        st["total_energy"] = eint + 1.5 * v * v
        if de:
            st["internal_energy"] = eint
        act = tuple(slice(g, g + k) for k in n[::-1])
        for k in st:  # ghosts come from the first refresh
            a = np.full_like(st[k], np.nan)
            a[act] = st[k][act]
            st[k] = a
        states.append(st)
        widths.append((h, h, h))
    return mesh, n, g, states, widths


@pytest.mark.parametrize("de", [False, True])
def test_smr_run_bit_exact(de):
    mesh, n, g, states, widths = _smr_case(de)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", dual_energy=de, courant=0.4)
    prm = oracle_params("hllc", "plm", de=de, courant=0.4)
    blocks, oblocks, slots = [], [], []
    for st, w in zip(states, widths):
        b = B.Block(n, g, w, mhd=False, dual_energy=de)
        b.load_numpy(st)
        blocks.append(b)
        ob = O.Block(n, g, w, mhd=False, dual_energy=de)
        for k, v in st.items():
            ob.f[ic.ORACLE_NAME[k]][...] = v
        oblocks.append(ob)
        names = {0: "rho", 1: "vx", 2: "vy", 3: "vz", 4: "etot", 9: "pressure"}
        if de:
            names[5] = "eint"
        slots.append({s: ob.f[k] for s, k in names.items()})
    faces, ofaces = mesh.face_array(), mesh.face_ints()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    # the first refresh fills every ghost zone
    meth.refresh_faces(blocks, faces, cons)
    O.refresh_faces(slots, n, (g,) * 3, ofaces, cons)
    for cycle in range(3):
        dts = [meth.timestep(b) for b in blocks]
        odts = [O.timestep(prm, ob) for ob in oblocks]
        assert dts == odts, cycle
        dt = min(dts)
        meth.refresh_faces(blocks, faces, cons)
        O.refresh_faces(slots, n, (g,) * 3, ofaces, cons)
        for b, ob in zip(blocks, oblocks):
            meth.compute(b, dt)
            O.step(prm, ob, dt)
    torch.cuda.synchronize()
    for i, (b, ob) in enumerate(zip(blocks, oblocks)):
        got = b.to_numpy()
        for k, a in got.items():
            want = ob.f[ic.ORACLE_NAME[k]]
            assert np.array_equal(a, want, equal_nan=True), (i, k)


def _oracle_smr(mesh, n, g, states, widths, de, prm, cycles):
    oblocks, slots = [], []
    for st, w in zip(states, widths):
        ob = O.Block(n, g, w, mhd=False, dual_energy=de)
        for k, v in st.items():
            ob.f[ic.ORACLE_NAME[k]][...] = v
        oblocks.append(ob)
        names = {0: "rho", 1: "vx", 2: "vy", 3: "vz", 4: "etot", 9: "pressure"}
        if de:
            names[5] = "eint"
        slots.append({s: ob.f[k] for s, k in names.items()})
    ofaces = mesh.face_ints()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    O.refresh_faces(slots, n, (g,) * 3, ofaces, cons)
    for _ in range(cycles):
        dt = min(O.timestep(prm, ob) for ob in oblocks)
        O.refresh_faces(slots, n, (g,) * 3, ofaces, cons)
        for ob in oblocks:
            O.step(prm, ob, dt)
    return oblocks


def test_smr_batch_graph_bit_exact():
    from test_gpu_batch import Batch
    mesh, n, g, states, widths = _smr_case(False)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=0.4)
    prm = oracle_params("hllc", "plm", courant=0.4)
    L = capi.lib()
    bt = Batch(meth, [n] * len(states), widths, ghost=g)
    for i, st in enumerate(states):
        bt.upload(i, st)
    farr, nf = mesh.face_array()
    capi.check(L.mhdvlct_batch_set_refresh_faces(bt.h, farr, nf,
                                                 capi.MHD_CONSERVATIVE_DEFAULT),
               meth.handle, "faces")
    capi.check(L.mhdvlct_batch_refresh(bt.h, None), meth.handle, "refresh")
    capi.check(L.mhdvlct_batch_run(bt.h, 3, 0, None, None), meth.handle, "run")
    oblocks = _oracle_smr(mesh, n, g, states, widths, False, prm, 3)
    for i, ob in enumerate(oblocks):
        got = bt.download(i)
        for k in ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy"):
            assert np.array_equal(got[k], ob.f[ic.ORACLE_NAME[k]], equal_nan=True), (i, k)


def test_smr_batch_fp32_close_to_fp64_oracle():
    # the benchmarked form: FP32 batch, mesh refresh inside the cycle graph,
    # two cycles against the FP64 oracle (relative L1 over the active cells)
    from test_gpu_batch import Batch
    mesh, n, g, states, widths = _smr_case(False)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=0.4)
    prm = oracle_params("hllc", "plm", courant=0.4)
    L = capi.lib()
    bt = Batch(meth, [n] * len(states), widths, dtype=capi.MHD_DTYPE_F32, ghost=g)
    for i, st in enumerate(states):
        bt.upload(i, st)
    farr, nf = mesh.face_array()
    capi.check(L.mhdvlct_batch_set_refresh_faces(bt.h, farr, nf,
                                                 capi.MHD_CONSERVATIVE_DEFAULT),
               meth.handle, "faces")
    capi.check(L.mhdvlct_batch_refresh(bt.h, None), meth.handle, "refresh")
    capi.check(L.mhdvlct_batch_run(bt.h, 2, 0, None, None), meth.handle, "run")
    oblocks = _oracle_smr(mesh, n, g, states, widths, False, prm, 2)
    act = tuple(slice(g, g + k) for k in n[::-1])
    for i, ob in enumerate(oblocks):
        got = bt.download(i)
        for k in ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy"):
            want = ob.f[ic.ORACLE_NAME[k]][act]
            err = np.abs(got[k][act].astype(np.float64) - want).sum() / np.abs(want).sum()
            assert err <= 1e-5, (i, k, err)



@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_three_level_refresh_bit_exact(dtype):
    from test_refresh_oracle import _three_level_mesh
    mesh = _three_level_mesh()
    n, g = (8, 8, 8), 4
    npdt = np.float64 if dtype == torch.float64 else np.float32
    ref = mesh_blocks(len(mesh.leaves), n, g, HYDRO_SLOTS, npdt, seed=17)
    blocks = _gpu_blocks(ref, n, g, dtype, mhd=False, de=True, npass=1)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc", dual_energy=True)
    meth.refresh_faces(blocks, mesh.face_array())
    torch.cuda.synchronize()
    O.refresh_faces(ref, n, (g,) * 3, mesh.face_ints(), capi.MHD_CONSERVATIVE_DEFAULT)
    for i, (b, r) in enumerate(zip(blocks, ref)):
        got = b.to_numpy()
        for s_, a in r.items():
            assert np.isfinite(a).all(), (i, SLOT_NAME[s_])
            assert np.array_equal(got[SLOT_NAME[s_]], a), (i, SLOT_NAME[s_])


def test_smr_batch_graph_gravity_passive_bit_exact():
    """The batched SMR cycle with the acceleration and one passive scalar in
    every leaf: the mesh refresh carries both across levels (slots 10..13)
    and the stages advect the scalar and add the gravity source, bit for bit
    with the oracle in FP64."""
    from test_gpu_batch import Batch
    mesh, n, g, states, widths = _smr_case(False)
    rng = np.random.default_rng(29)
    act = tuple(slice(g, g + k) for k in n[::-1])
    for st in states:
        for ax in "xyz":
            a = np.full_like(st["density"], np.nan)
            a[act] = 0.2 * (rng.random(a[act].shape) - 0.5)
            st[f"acceleration_{ax}"] = a
        p = np.full_like(st["density"], np.nan)
        p[act] = st["density"][act] * (0.2 + 0.6 * rng.random(p[act].shape))
        st["passive_0"] = p
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=0.4)
    prm = oracle_params("hllc", "plm", courant=0.4)
    L = capi.lib()
    bt = Batch(meth, [n] * len(states), widths, ghost=g, npassive=1, gravity=True)
    for i, st in enumerate(states):
        bt.upload(i, st)
    farr, nf = mesh.face_array()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    capi.check(L.mhdvlct_batch_set_refresh_faces(bt.h, farr, nf, cons), meth.handle, "faces")
    capi.check(L.mhdvlct_batch_refresh(bt.h, None), meth.handle, "refresh")
    capi.check(L.mhdvlct_batch_run(bt.h, 3, 0, None, None), meth.handle, "run")
    oname = dict(ic.ORACLE_NAME, acceleration_x="ax", acceleration_y="ay",
                 acceleration_z="az", passive_0="pass0")
    oblocks, slots = [], []
    for st, w in zip(states, widths):
        ob = O.Block(n, g, w, mhd=False, gravity=True, npassive=1)
        for k, v in st.items():
            ob.f[oname[k]][...] = v
        oblocks.append(ob)
        names = {0: "rho", 1: "vx", 2: "vy", 3: "vz", 4: "etot", 9: "pressure",
                 10: "ax", 11: "ay", 12: "az", 13: "pass0"}
        slots.append({s: ob.f[k] for s, k in names.items()})
    ofaces = mesh.face_ints()
    O.refresh_faces(slots, n, (g,) * 3, ofaces, cons)
    for _ in range(3):
        dt = min(O.timestep(prm, ob) for ob in oblocks)
        O.refresh_faces(slots, n, (g,) * 3, ofaces, cons)
        for ob in oblocks:
            O.step(prm, ob, dt)
    for i, ob in enumerate(oblocks):
        got = bt.download(i)
        for k in ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy",
                  "passive_0", "acceleration_x", "acceleration_y", "acceleration_z"):
            assert np.array_equal(got[k], ob.f[oname[k]], equal_nan=True), (i, k)
