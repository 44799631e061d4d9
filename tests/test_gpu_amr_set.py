"""Parity of the mixed-size AMR block set (the batched form with per-block dt).

A scaled-down copy of the benchmarked set: 12 blocks of 16^3, 6 of 32^3 and
2 of 64^3 (3 ghost layers), each a Sedov blast, ghosts refreshed from seeded
same-size neighbours, every block advanced with its own CFL dt
(EnzoMethodMHDVlct::timestep, EnzoMethodMHDVlct.cpp:551-588, with no global
minimum) in one persistent launch per stage at the autotuner's tiles
(mhdvlct_batch_run with dt_mode 1).  The oracle runs the same cycle block by
block: each block's dt on its stale ghosts, the table-driven refresh, the
step.

  - FP64: bit-exact after two cycles;
  - FP32: per-field relative L1 against the FP64 oracle <= 1e-5 after one
    cycle, and each block's dt within 1e-6 of the oracle's.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from mhdvlct import block as B, capi, ic
from helpers import oracle_block, oracle_params
from test_gpu_batch import KEYS, Batch

pytestmark = pytest.mark.gpu

G, COURANT = 3, 0.4
COUNTS = ((16, 12), (32, 6), (64, 2))
FP32_TOL = 1e-5


def _active(k, a, n):
    if not k.startswith("bfieldi"):
        return a[(slice(G, G + n),) * 3]
    d = "xyz".index(k[-1])
    sl = [slice(G, G + n)] * 3
    sl[2 - d] = slice(G, G + n + 1)
    return a[tuple(sl)]


@pytest.fixture(scope="module")
def amr_set():
    return ic.amr_block_set(seed=5, counts=COUNTS, g=G, dtype=np.float64)


@pytest.fixture(scope="module")
def oracle_run(amr_set):
    blocks, dims, widths, nbr = amr_set
    prm = oracle_params(courant=COURANT)
    obs = [oracle_block(s, d[0], G, w) for s, d, w in zip(blocks, dims, widths)]
    dts, states = [], []
    for _ in range(2):
        dt = [O.timestep(prm, ob) for ob in obs]
        O.fill_ghosts_table(obs, nbr)
        for ob, d in zip(obs, dt):
            O.step(prm, ob, d)
        dts.append(dt)
        states.append([{k: ob.f[ic.ORACLE_NAME[k]].copy() for k in KEYS} for ob in obs])
    return dts, states


def _batch(amr_set, dtype):
    blocks, dims, widths, nbr = amr_set
    meth = B.EnzoMethodMHDVlct(riemann_solver="hlld", reconstruct_method="plm",
                               courant=COURANT)
    bt = Batch(meth, dims, widths, dtype=dtype)
    L = capi.lib()
    capi.check(L.mhdvlct_batch_set_neighbors(
        bt.h, (ctypes.c_int * nbr.size)(*nbr.ravel().tolist())))
    for i, s in enumerate(blocks):
        bt.upload(i, {k: v for k, v in s.items() if k != "pressure"})
    buf = ctypes.create_string_buffer(8192)
    capi.check(L.mhdvlct_batch_autotune(bt.h, 1, buf, 8192, None), meth.handle, "autotune")
    return bt


def _run(bt, cycles):
    capi.check(capi.lib().mhdvlct_batch_run(bt.h, cycles, 1, None, None), bt.meth.handle,
               "run")


def _dts(bt):
    """The per-block dt of the batch's current state (a timestep call, which
    does not change the cell fields of a run without dual energy)."""
    out = (ctypes.c_double * bt.n)()
    capi.check(capi.lib().mhdvlct_batch_timestep(bt.h, out, None))
    return list(out)


def test_fp64_per_block_dt_bit_exact(amr_set, oracle_run):
    dts, states = oracle_run
    blocks, dims, widths, nbr = amr_set
    bt = _batch(amr_set, capi.MHD_DTYPE_F64)
    assert _dts(bt) == dts[0]
    _run(bt, 2)
    for i, d in enumerate(dims):
        got = bt.download(i)
        for k in KEYS:
            a, r = _active(k, got[k], d[0]), _active(k, states[1][i][k], d[0])
            assert np.array_equal(a, r), (i, d, k, np.abs(a - r).max())


def test_fp32_per_block_dt_error(amr_set, oracle_run):
    dts, states = oracle_run
    blocks, dims, widths, nbr = amr_set
    bt = _batch(amr_set, capi.MHD_DTYPE_F32)
    got_dt = _dts(bt)
    for a, r in zip(got_dt, dts[0]):
        assert abs(a - r) <= 1e-6 * r
    _run(bt, 1)
    num, den = {}, {}
    for i, d in enumerate(dims):
        got = bt.download(i)
        for k in KEYS:
            a = _active(k, got[k], d[0]).astype(np.float64)
            r = _active(k, states[0][i][k], d[0])
            num[k] = num.get(k, 0.0) + np.abs(a - r).sum()
            den[k] = den.get(k, 0.0) + np.abs(r).sum()
    err = {k: num[k] / den[k] for k in KEYS if den[k] > 0}
    assert max(err.values()) <= FP32_TOL, err
