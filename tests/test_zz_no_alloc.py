"""mhdvlct_block_step_noalloc (static device scratch) against
mhdvlct_block_step (allocated scratch): on identical blocks, two consecutive
calls give bit-identical fields after each call, for both precisions and the
euler / VL forms; a block whose scratch exceeds the static array is rejected
before any work is done.

Named to be collected last, so it runs both alone and after every other test
file has used the library in the same process.
"""
import ctypes

import numpy as np
import pytest
import torch

from mhdvlct import block as B, capi, ic

pytestmark = pytest.mark.gpu

STATIC_SCRATCH_BYTES = 8 << 20


def _noalloc_step(meth, blk, dt):
    v = blk.view()
    rc = capi.lib().mhdvlct_block_step_noalloc(
        meth.handle, ctypes.byref(v), dt, torch.cuda.current_stream().cuda_stream)
    return rc


def _twin(solver, recon, de, scheme, n, dtype, seed):
    mhd = solver != "hllc"
    state, w = ic.smooth_block(n, 3, seed=seed, mhd=mhd, dual_energy=de)
    meth = B.EnzoMethodMHDVlct(
        mhd_choice="constrained_transport" if mhd else "no_bfield",
        riemann_solver=solver, reconstruct_method=recon, time_scheme=scheme,
        dual_energy=de)
    a = B.Block(n, 3, w, mhd=mhd, dual_energy=de, dtype=dtype)
    b = B.Block(n, 3, w, mhd=mhd, dual_energy=de, dtype=dtype)
    a.load_numpy(state)
    b.load_numpy(state)
    return meth, a, b


def _same(a, b):
    fa, fb = a.to_numpy(), b.to_numpy()
    assert fa.keys() == fb.keys()
    for k in fa:
        assert np.array_equal(fa[k], fb[k]), k


@pytest.mark.parametrize("solver,recon,de,scheme,n,dtype", [
    ("hlld", "plm", False, "vl", (8, 6, 7), torch.float64),
    ("hllc", "plm", True, "vl", (8, 8, 8), torch.float64),
    ("hllc", "nn", False, "euler", (6, 7, 8), torch.float64),
    ("hlld", "plm", False, "vl", (12, 12, 12), torch.float32),
])
def test_noalloc_matches_allocating_step_two_calls(solver, recon, de, scheme, n, dtype):
    meth, a, b = _twin(solver, recon, de, scheme, n, dtype, seed=17)
    for _ in range(2):
        dt = meth.timestep(a)
        assert meth.timestep(b) == dt
        meth.fill_ghosts_periodic(a)
        meth.fill_ghosts_periodic(b)
        meth.compute(a, dt)
        assert _noalloc_step(meth, b, dt) == capi.MHD_OK
        torch.cuda.synchronize()
        _same(a, b)


@pytest.mark.parametrize("solver,recon,de,scheme", [
    ("hlld", "plm", False, "vl"), ("hllc", "plm", True, "euler")])
def test_noalloc_passive_scalars_match_allocating_step(solver, recon, de, scheme):
    # three passive scalars: their half step lives in the static array too
    n, npass = (8, 7, 6), 3
    mhd = solver != "hllc"
    state, w = ic.smooth_block(n, 3, seed=23, mhd=mhd, dual_energy=de)
    rng = np.random.default_rng(5)
    for k in range(npass):
        state[f"passive_{k}"] = state["density"] * (0.2 + 0.6 * rng.random(state["density"].shape))
    meth = B.EnzoMethodMHDVlct(
        mhd_choice="constrained_transport" if mhd else "no_bfield",
        riemann_solver=solver, reconstruct_method=recon, time_scheme=scheme,
        dual_energy=de)
    a, b = (B.Block(n, 3, w, mhd=mhd, dual_energy=de, dtype=torch.float64, npassive=npass)
            for _ in range(2))
    a.load_numpy(state)
    b.load_numpy(state)
    for _ in range(2):
        dt = meth.timestep(a)
        assert meth.timestep(b) == dt
        meth.compute(a, dt)
        assert _noalloc_step(meth, b, dt) == capi.MHD_OK
        torch.cuda.synchronize()
        _same(a, b)
    assert "passive_2" in a.to_numpy()


@pytest.mark.parametrize("recon,dtype,npass,gravity", [
    ("plm", torch.float64, 0, True),   # the gravity source on the full-dt stage
    ("nn", torch.float32, 2, False),   # FP32 scalars in the two-CTA NN instantiation
    ("plm", torch.float32, 1, True),
])
def test_noalloc_extras_match_allocating_step(recon, dtype, npass, gravity):
    n = (10, 8, 9)
    state, w = ic.smooth_block(n, 3, seed=29)
    rng = np.random.default_rng(7)
    shp = state["density"].shape
    for k in range(npass):
        state[f"passive_{k}"] = state["density"] * (0.2 + 0.6 * rng.random(shp))
    if gravity:
        for k in ("acceleration_x", "acceleration_y", "acceleration_z"):
            state[k] = 0.3 * (rng.random(shp) - 0.5)
    meth = B.EnzoMethodMHDVlct(riemann_solver="hlld", reconstruct_method=recon)
    a, b = (B.Block(n, 3, w, dtype=dtype, npassive=npass, gravity=gravity) for _ in range(2))
    a.load_numpy(state)
    b.load_numpy(state)
    for _ in range(2):
        dt = meth.timestep(a)
        assert meth.timestep(b) == dt
        meth.fill_ghosts_periodic(a)
        meth.fill_ghosts_periodic(b)
        meth.compute(a, dt)
        assert _noalloc_step(meth, b, dt) == capi.MHD_OK
        torch.cuda.synchronize()
        _same(a, b)
    if npass:
        assert not np.array_equal(a.to_numpy()["passive_0"],
                                  np.asarray(state["passive_0"], dtype=a.to_numpy()["passive_0"].dtype))


def test_noalloc_geometry_change_between_calls():
    # a larger block after a smaller one reuses the same static array
    for n in ((6, 6, 6), (16, 10, 12), (6, 6, 6)):
        meth, a, b = _twin("hlld", "plm", False, "vl", n, torch.float64, seed=3)
        dt = meth.timestep(a)
        assert meth.timestep(b) == dt
        meth.compute(a, dt)
        assert _noalloc_step(meth, b, dt) == capi.MHD_OK
        torch.cuda.synchronize()
        _same(a, b)


def test_noalloc_rejects_oversize_block():
    # 64^3 + 3 ghosts in FP64: 9 cell fields alone are ~19 MB > 8 MiB
    n = (64, 64, 64)
    meth = B.EnzoMethodMHDVlct()
    blk = B.Block(n, 3, (1 / 64,) * 3, dtype=torch.float64)
    before = blk.to_numpy()
    rc = _noalloc_step(meth, blk, 1e-3)
    assert rc == capi.MHD_ERR_INVALID
    msg = capi.lib().mhdvlct_last_error_string(meth.handle).decode()
    assert "bytes of scratch" in msg and str(STATIC_SCRATCH_BYTES) in msg, msg
    torch.cuda.synchronize()
    after = blk.to_numpy()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
