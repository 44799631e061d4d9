"""The gravity source term (EnzoSourceGravity.cpp:17-69) through the C ABI:
with acceleration fields the CUDA step equals the oracle (itself pinned bit
for bit to the reference's own code in tests/test_gravity_oracle.py) in FP64
and stays within 1e-5 relative L1 in FP32; the source enters only the
full-dt stage of vl (never euler), as in the reference."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from mhdvlct import block as B, ic
from helpers import oracle_params, rel_l1

pytestmark = pytest.mark.gpu

ONAME = dict(ic.ORACLE_NAME, acceleration_x="ax", acceleration_y="ay",
             acceleration_z="az")


def _pair(solver, recon, de, scheme, dtype, n=(8, 7, 9), seed=41):
    mhd = solver != "hllc"
    state, w = ic.smooth_block(n, 3, seed=seed, mhd=mhd, dual_energy=de)
    rng = np.random.default_rng(seed + 1)
    m = tuple(x + 6 for x in n)
    for k in ("acceleration_x", "acceleration_y", "acceleration_z"):
        state[k] = 0.3 * (rng.random((m[2], m[1], m[0])) - 0.5)
    meth = B.EnzoMethodMHDVlct(
        mhd_choice="constrained_transport" if mhd else "no_bfield",
        riemann_solver=solver, reconstruct_method=recon, time_scheme=scheme,
        dual_energy=de)
    blk = B.Block(n, 3, w, mhd=mhd, dual_energy=de, dtype=dtype, gravity=True)
    blk.load_numpy(state)
    ob = O.Block(n, 3, w, mhd=mhd, dual_energy=de, gravity=True)
    for k, v in state.items():
        if ONAME[k] in ob.f:
            ob.f[ONAME[k]][...] = v
    prm = oracle_params(solver, recon, de=de, euler=scheme == "euler",
                        courant=meth.courant)
    return meth, blk, ob, prm


CASES = [("hlld", "plm", False, "vl"), ("hllc", "plm", True, "vl"),
         ("hlle", "nn", False, "vl"), ("hllc", "nn", False, "euler")]


@pytest.mark.parametrize("solver,recon,de,scheme", CASES)
def test_fp64_gravity_step_bit_exact(solver, recon, de, scheme):
    meth, blk, ob, prm = _pair(solver, recon, de, scheme, torch.float64)
    dt = O.timestep(prm, ob)
    assert meth.timestep(blk) == dt
    O.step(prm, ob, dt)
    meth.compute(blk, dt)
    torch.cuda.synchronize()
    for k, a in blk.to_numpy().items():
        assert np.array_equal(a, ob.f[ONAME[k]]), k


@pytest.mark.parametrize("solver,recon,de,scheme", CASES[:2])
def test_fp32_gravity_step_close(solver, recon, de, scheme):
    meth, blk, ob, prm = _pair(solver, recon, de, scheme, torch.float32, n=(10, 10, 10))
    dt = O.timestep(prm, ob)
    meth.timestep(blk)
    O.step(prm, ob, dt)
    meth.compute(blk, dt)
    torch.cuda.synchronize()
    g = 3
    act = (slice(g, g + 10),) * 3
    got = blk.to_numpy()
    for k in ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy"):
        assert rel_l1(got[k][act].astype(np.float64), ob.f[ONAME[k]][act]) <= 1e-5, k
