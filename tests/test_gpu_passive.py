"""Passive scalars through the C ABI (the stage kernel writes the density
fluxes, passive_kernel advects the scalars): the CUDA step equals the oracle
(pinned bit for bit to the reference in tests/test_passive_oracle.py) in FP64
and stays within 1e-5 relative L1 in FP32; the periodic ghost refresh covers
the scalar fields; the no-alloc entry point equals the oracle too."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from mhdvlct import block as B, capi, ic
from helpers import oracle_params, rel_l1

pytestmark = pytest.mark.gpu

ONAME = dict(ic.ORACLE_NAME)


def _pair(solver, recon, de, scheme, dtype, n=(8, 9, 7), seed=51, npass=3):
    mhd = solver != "hllc"
    state, w = ic.smooth_block(n, 3, seed=seed, mhd=mhd, dual_energy=de)
    rng = np.random.default_rng(seed + 3)
    for k in range(npass):
        state[f"passive_{k}"] = state["density"] * (0.2 + 0.6 * rng.random(state["density"].shape))
    meth = B.EnzoMethodMHDVlct(
        mhd_choice="constrained_transport" if mhd else "no_bfield",
        riemann_solver=solver, reconstruct_method=recon, time_scheme=scheme,
        dual_energy=de)
    blk = B.Block(n, 3, w, mhd=mhd, dual_energy=de, dtype=dtype, npassive=npass)
    blk.load_numpy(state)
    ob = O.Block(n, 3, w, mhd=mhd, dual_energy=de, npassive=npass)
    for k, v in state.items():
        key = f"pass{k[8:]}" if k.startswith("passive_") else ONAME[k]
        if key in ob.f:
            ob.f[key][...] = v
    prm = oracle_params(solver, recon, de=de, euler=scheme == "euler",
                        courant=meth.courant)
    return meth, blk, ob, prm


def _oname(k):
    return f"pass{k[8:]}" if k.startswith("passive_") else ONAME[k]


CASES = [("hlld", "plm", False, "vl"), ("hllc", "plm", True, "vl"),
         ("hlle", "nn", False, "vl"), ("hllc", "plm_athena", False, "euler")]


@pytest.mark.parametrize("solver,recon,de,scheme", CASES)
def test_fp64_passive_step_bit_exact(solver, recon, de, scheme):
    meth, blk, ob, prm = _pair(solver, recon, de, scheme, torch.float64)
    dt = O.timestep(prm, ob)
    assert meth.timestep(blk) == dt
    O.step(prm, ob, dt)
    meth.compute(blk, dt)
    torch.cuda.synchronize()
    for k, a in blk.to_numpy().items():
        assert np.array_equal(a, ob.f[_oname(k)]), k


def test_fp32_passive_step_close():
    n = (10, 10, 10)
    meth, blk, ob, prm = _pair("hlld", "plm", False, "vl", torch.float32, n=n)
    dt = O.timestep(prm, ob)
    meth.timestep(blk)
    O.step(prm, ob, dt)
    meth.compute(blk, dt)
    torch.cuda.synchronize()
    act = (slice(3, 13),) * 3
    got = blk.to_numpy()
    for k in ("passive_0", "passive_1", "passive_2", "density"):
        assert rel_l1(got[k][act].astype(np.float64), ob.f[_oname(k)][act]) <= 1e-5, k


def test_periodic_refresh_covers_passive():
    meth, blk, ob, prm = _pair("hllc", "plm", False, "vl", torch.float64, npass=2)
    meth.fill_ghosts_periodic(blk)
    torch.cuda.synchronize()
    got = blk.to_numpy()
    g = 3
    for k in ("passive_0", "passive_1"):
        inner = got[k][g:-g, g:-g, g:-g]
        assert np.array_equal(got[k], np.pad(inner, g, mode="wrap")), k


def test_noalloc_passive_step_bit_exact():
    # the no-alloc entry keeps the scalars' half step in its static array
    meth, blk, ob, prm = _pair("hllc", "plm", False, "vl", torch.float64, npass=2)
    dt = O.timestep(prm, ob)
    assert meth.timestep(blk) == dt
    O.step(prm, ob, dt)
    v = blk.view()
    rc = capi.lib().mhdvlct_block_step_noalloc(meth.handle, ctypes.byref(v), dt, None)
    assert rc == capi.MHD_OK
    torch.cuda.synchronize()
    for k, a in blk.to_numpy().items():
        assert np.array_equal(a, ob.f[_oname(k)]), k
