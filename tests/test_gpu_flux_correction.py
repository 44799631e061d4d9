"""Flux correction (store_fluxes_for_corrections, EnzoMethodMHDVlct.cpp:
250-330) through the C ABI: the CUDA step's dt/dx-scaled boundary fluxes
against the oracle's on ragged blocks, FP64 bit for bit and FP32 within 1e-6
of the largest flux, and the reference's restrictions (hydro only,
internal_energy only with dual energy)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from mhdvlct import block as B, capi, ic
from helpers import oracle_block, oracle_params

pytestmark = pytest.mark.gpu

CASES = [("plm", False, "vl"), ("plm", True, "vl"), ("nn", False, "vl"),
         ("plm_athena", True, "vl"), ("nn", False, "euler")]


def _run(recon, de, scheme, dtype, n=(9, 7, 8), seed=31):
    state, w = ic.smooth_block(n, 3, seed=seed, mhd=False, dual_energy=de)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method=recon, time_scheme=scheme,
                               dual_energy=de)
    blk = B.Block(n, 3, w, mhd=False, dual_energy=de, dtype=dtype)
    blk.load_numpy(state)
    ob = oracle_block(state, n, 3, w, mhd=False, de=de)
    prm = oracle_params("hllc", recon, de=de, euler=scheme == "euler",
                        courant=meth.courant)
    qs = (0, 1, 2, 3, 4, 5) if de else (0, 1, 2, 3, 4)
    dt = O.timestep(prm, ob)
    ref = O.step_fc(prm, ob, dt, qs)
    meth.timestep(blk)
    got = meth.compute_store_fluxes(blk, dt, qs)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in got.items()}, ref, blk, ob


@pytest.mark.parametrize("recon,de,scheme", CASES)
def test_fp64_boundary_fluxes_bit_exact(recon, de, scheme):
    got, ref, blk, ob = _run(recon, de, scheme, torch.float64)
    assert got.keys() == ref.keys()
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k
    # the step itself is unchanged by storing the fluxes
    out = blk.to_numpy()
    assert np.array_equal(out["density"], ob.f["rho"])
    assert np.array_equal(out["total_energy"], ob.f["etot"])


@pytest.mark.parametrize("recon,de,scheme", CASES[:3])
def test_fp32_boundary_fluxes_close(recon, de, scheme):
    got, ref, _, _ = _run(recon, de, scheme, torch.float32)
    for k in ref:
        scale = max(np.abs(ref[k]).max(), 1e-30)
        assert np.abs(got[k].astype(np.float64) - ref[k]).max() <= 1e-6 * scale, k


def test_flux_correction_restrictions():
    n = (6, 6, 6)
    mhd_meth = B.EnzoMethodMHDVlct()
    blk = B.Block(n, 3, (0.1, 0.1, 0.1), dtype=torch.float64)
    fc = capi.MhdFluxCorrection()
    rc = capi.lib().mhdvlct_block_step_fc(mhd_meth.handle, ctypes.byref(blk.view()),
                                          1e-3, ctypes.byref(fc), None)
    assert rc == capi.MHD_ERR_INVALID
    assert b"hydro" in capi.lib().mhdvlct_last_error_string(mhd_meth.handle)
    hydro = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc")
    hb = B.Block(n, 3, (0.1, 0.1, 0.1), mhd=False, dtype=torch.float64)
    t = torch.zeros((6, 6), dtype=torch.float64, device="cuda")
    fc.flux[0][0][capi.MHD_Q_INTERNAL_ENERGY] = t.data_ptr()
    rc = capi.lib().mhdvlct_block_step_fc(hydro.handle, ctypes.byref(hb.view()), 1e-3,
                                          ctypes.byref(fc), None)
    assert rc == capi.MHD_ERR_INVALID
