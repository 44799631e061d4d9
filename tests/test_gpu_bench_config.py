"""Parity at the benchmarked configuration.

The bench advances the turbulent box (HLLD + PLM, gamma 5/3, CFL 0.4, rms
Mach 2, plasma beta ~ 1) in blocks of 32^3 active cells with 3 ghost layers,
through the batched form at the autotuner's tiles (or the tiles forced with
``bench.py --tile 30x10,28x14``).  Here the same recipe builds a 64^3 box in
a periodic 2x2x2 brick of those blocks and runs the same batched, graph-
replayed cycle (timestep on stale ghosts, global min dt, 27-neighbour
refresh, two stages), against the oracle's cycle
(EnzoMethodMHDVlct.cpp:356-588; the global min of control_stopping.cpp:
96-140):

  - FP64: bit-exact after two cycles, the simulated time included, at the
    autotuned tiles and at a forced tile with z-chunks;
  - FP32: per-field relative L1 error against the FP64 oracle <= 1e-5 per
    cycle (cycle 1 from the initial state; cycle 2 from the oracle's own
    cycle-1 state rounded to float), and normalised div B (|div B| dx /
    max |B|) <= 1e-6, at the autotuned tiles and at the bench's forced
    tiles;
  - the stage kernels compiled for the bench's launch shape (tiles, block
    extent and stale depths as constants) give the FP32 state of the
    run-time kernels bit for bit: the MHD box here, plain and with the
    gravity source and two passive scalars, and hydro (HLLC) leaves of 32^3
    with 4 ghost layers on a two-level mesh, with and without flux storing
    and correction.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from mhdvlct import block as B, capi, ic
from helpers import oracle_block, oracle_params
from test_gpu_batch import KEYS, Batch

pytestmark = pytest.mark.gpu

N, NB, G, COURANT = 64, 2, 3, 0.4
n = N // NB
NBLK = NB ** 3
ACT = (slice(G, G + n),) * 3
FP32_TOL = 1e-5      # relative L1 per field per cycle against the FP64 oracle
DIVB_TOL = 1e-6      # |div B| dx / max |B| in FP32


def _active(k, a):
    """Active cells of a cell field; every interior face of a face field."""
    if not k.startswith("bfieldi"):
        return a[ACT]
    d = "xyz".index(k[-1])
    sl = [slice(G, G + n)] * 3
    sl[2 - d] = slice(G, G + n + 1)
    return a[tuple(sl)]


@pytest.fixture(scope="module")
def box():
    return ic.turbulent_box(N=N, nb=NB, g=G, seed=1, mach=2.0, dtype=np.float64)


@pytest.fixture(scope="module")
def oracle_run(box):
    """Two oracle cycles; the state (every array, ghosts included) after each."""
    blocks, w = box
    prm = oracle_params(courant=COURANT)
    obs = [oracle_block(s, n, G, w) for s in blocks]
    dts, states = [], []
    for _ in range(2):
        dt = min(O.timestep(prm, ob) for ob in obs)
        O.fill_ghosts_brick(obs, NB, NB, NB)
        for ob in obs:
            O.step(prm, ob, dt)
        dts.append(dt)
        states.append([{k: ob.f[ic.ORACLE_NAME[k]].copy() for k in KEYS} for ob in obs])
    return dts, states


def _batch(box, dtype, tiles):
    blocks, w = box
    meth = B.EnzoMethodMHDVlct(riemann_solver="hlld", reconstruct_method="plm",
                               courant=COURANT)
    bt = Batch(meth, [(n, n, n)] * NBLK, [w] * NBLK, dtype=dtype)
    nbr = ic.brick_neighbors(NB)
    L = capi.lib()
    capi.check(L.mhdvlct_batch_set_neighbors(
        bt.h, (ctypes.c_int * nbr.size)(*nbr.ravel().tolist())))
    for i, s in enumerate(blocks):
        bt.upload(i, s)
    if tiles == "tuned":
        buf = ctypes.create_string_buffer(4096)
        capi.check(L.mhdvlct_batch_autotune(bt.h, 1, buf, 4096, None), meth.handle,
                   "autotune")
    else:
        for s_, (tx, ty, zc) in enumerate(tiles):
            capi.check(L.mhdvlct_batch_set_stage_tile(bt.h, s_, tx, ty, zc, 256),
                       meth.handle, "tile")
    return bt, meth


def _run(bt, cycles):
    t = ctypes.c_double()
    capi.check(capi.lib().mhdvlct_batch_run(bt.h, cycles, 0, ctypes.byref(t), None),
               bt.meth.handle, "run")
    return t.value


def _divb(bt, w):
    d = (ctypes.c_double * 8)()
    capi.check(capi.lib().mhdvlct_batch_diagnostics(bt.h, d, None))
    return d[6] * w[0] / d[7]


@pytest.mark.parametrize("tiles", ["tuned", ((16, 8, 0), (12, 12, 8))])
def test_fp64_bit_exact_at_bench_shape(box, oracle_run, tiles):
    dts, states = oracle_run
    bt, _ = _batch(box, capi.MHD_DTYPE_F64, tiles)
    t = _run(bt, 2)
    assert t == dts[0] + dts[1]
    for i in range(NBLK):
        got = bt.download(i)
        for k in KEYS:
            a, r = _active(k, got[k]), _active(k, states[1][i][k])
            assert np.array_equal(a, r), (i, k, np.abs(a - r).max())


def _field_errors(bt, ref):
    """Per-field relative L1 over the active zones of every block."""
    num, den = {}, {}
    for i in range(NBLK):
        got = bt.download(i)
        for k in KEYS:
            a = _active(k, got[k]).astype(np.float64)
            r = _active(k, ref[i][k])
            num[k] = num.get(k, 0.0) + np.abs(a - r).sum()
            den[k] = den.get(k, 0.0) + np.abs(r).sum()
    return {k: num[k] / den[k] for k in KEYS}


@pytest.mark.parametrize("tiles", ["tuned", ((30, 10, 0), (28, 14, 0))])
def test_fp32_error_per_cycle_at_bench_shape(box, oracle_run, tiles):
    dts, states = oracle_run
    blocks, w = box
    bt, _ = _batch(box, capi.MHD_DTYPE_F32, tiles)
    # cycle 1 from the initial state
    t = _run(bt, 1)
    assert abs(t - dts[0]) <= 1e-6 * dts[0]
    err = _field_errors(bt, states[0])
    assert max(err.values()) <= FP32_TOL, err
    assert _divb(bt, w) <= DIVB_TOL
    # cycle 2 from the oracle's cycle-1 state, rounded to float
    for i in range(NBLK):
        bt.upload(i, states[0][i])
    t = _run(bt, 1)
    assert abs(t - dts[1]) <= 1e-6 * dts[1]
    err = _field_errors(bt, states[1])
    assert max(err.values()) <= FP32_TOL, err
    assert _divb(bt, w) <= DIVB_TOL


def _state(bt):
    return [bt.download(i) for i in range(bt.n)]


def test_fp32_fixed_layout_tiles_equal_runtime_layout(box):
    # (30, 10) / (28, 14) split the 36- and 34-wide column regions of a 32^3
    # block into tiles of 18 x 9 and at most 17 x 12, the layouts compiled
    # as constants; (16, 8) / (12, 12) give 12 x 8 and 12 x 12 (run-time)
    a, _ = _batch(box, capi.MHD_DTYPE_F32, ((30, 10, 0), (28, 14, 0)))
    b, _ = _batch(box, capi.MHD_DTYPE_F32, ((16, 8, 0), (12, 12, 0)))
    assert _run(a, 2) == _run(b, 2)
    for i, (ga, gb) in enumerate(zip(_state(a), _state(b))):
        for k in KEYS:
            assert np.array_equal(ga[k], gb[k]), (i, k)


def test_fp32_fixed_layout_extras_equal_runtime_layout(box):
    # the same tiles with the gravity source and two passive scalars (the
    # instantiation that writes the density fluxes for passive_kernel)
    blocks, w = box
    rng = np.random.default_rng(23)
    m = n + 2 * G
    states = []
    for st in blocks:
        st = dict(st)
        for k in ("acceleration_x", "acceleration_y", "acceleration_z"):
            st[k] = np.zeros((m, m, m))
            st[k][ACT] = 0.3 * (rng.random((n, n, n)) - 0.5)
        for k in range(2):
            st[f"passive_{k}"] = st["density"] * (0.2 + 0.6 * rng.random((m, m, m)))
        states.append(st)
    meth = B.EnzoMethodMHDVlct(riemann_solver="hlld", reconstruct_method="plm",
                               courant=COURANT)
    L = capi.lib()
    nbr = ic.brick_neighbors(NB)
    out = []
    for tiles in (((30, 10, 0), (28, 14, 0)), ((16, 8, 0), (12, 12, 0))):
        bt = Batch(meth, [(n, n, n)] * NBLK, [w] * NBLK, dtype=capi.MHD_DTYPE_F32,
                   npassive=2, gravity=True)
        capi.check(L.mhdvlct_batch_set_neighbors(
            bt.h, (ctypes.c_int * nbr.size)(*nbr.ravel().tolist())))
        for i, st in enumerate(states):
            bt.upload(i, st)
        for s_, (tx, ty, zc) in enumerate(tiles):
            capi.check(L.mhdvlct_batch_set_stage_tile(bt.h, s_, tx, ty, zc, 256),
                       meth.handle, "tile")
        out.append((_run(bt, 2), _state(bt)))
    assert out[0][0] == out[1][0]
    for i, (ga, gb) in enumerate(zip(out[0][1], out[1][1])):
        for k in KEYS + ("passive_0", "passive_1"):
            assert np.array_equal(ga[k], gb[k]), (i, k)


@pytest.mark.parametrize("fc", [False, True])
def test_fp32_fixed_layout_hydro_leaves_equal_runtime_layout(fc):
    # the static-mesh-refinement workload's leaves: 32^3 with 4 ghost layers;
    # the default FP32 tiles (34 x 10 / 24 x 16) split the 38- and 36-wide
    # regions into tiles of at most 19 x 10 and 18 x 12 (compiled layouts)
    from test_flux_correct_oracle import smr_blocks
    nn, g = 32, 4
    mesh, oblocks, _ = smr_blocks(nn, g)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=0.4)
    L = capi.lib()
    farr, nf = mesh.face_array()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    names = ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy")
    onames = ("rho", "vx", "vy", "vz", "etot")
    out = []
    for tiles in (((34, 10, 0), (24, 16, 0)), ((16, 8, 0), (12, 12, 0))):
        bt = Batch(meth, [(nn,) * 3] * len(oblocks), [ob.widths for ob in oblocks],
                   dtype=capi.MHD_DTYPE_F32, ghost=g)
        for i, ob in enumerate(oblocks):
            bt.upload(i, {k: ob.f[o] for k, o in zip(names, onames)})
        capi.check(L.mhdvlct_batch_set_refresh_faces(bt.h, farr, nf, cons), meth.handle,
                   "faces")
        if fc:
            capi.check(L.mhdvlct_batch_set_flux_correction(bt.h, 0b11111, farr, nf, cons),
                       meth.handle, "flux correction")
        for s_, (tx, ty, zc) in enumerate(tiles):
            capi.check(L.mhdvlct_batch_set_stage_tile(bt.h, s_, tx, ty, zc, 256),
                       meth.handle, "tile")
        capi.check(L.mhdvlct_batch_refresh(bt.h, None), meth.handle, "refresh")
        t = ctypes.c_double()
        capi.check(L.mhdvlct_batch_run(bt.h, 2, 0, ctypes.byref(t), None), meth.handle, "run")
        out.append((t.value, _state(bt)))
    assert out[0][0] == out[1][0]
    for i, (ga, gb) in enumerate(zip(out[0][1], out[1][1])):
        for k in names:
            assert np.array_equal(ga[k], gb[k]), (i, k)
