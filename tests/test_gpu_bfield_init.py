"""Initial B from an edge-centred vector potential through the C ABI
(mhdvlct_block_bfield_from_potential): the face and centred B equal the oracle
(EnzoInitialBCenter.cpp:27-127, its centring pinned to the reference in
tests/test_bfield_init_oracle.py) bit for bit in FP64 and FP32, over the
whole ghosted block."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from mhdvlct import block as B, capi

pytestmark = pytest.mark.gpu

FACES = ("bfieldi_x", "bfieldi_y", "bfieldi_z")
CELLS = ("bfield_x", "bfield_y", "bfield_z")


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("n,g", [((7, 9, 6), 3), ((16, 16, 16), 4), ((1, 5, 33), 3)])
def test_bfield_from_potential_bit_exact(dtype, n, g):
    w = (0.1, 0.07, 0.13)
    meth = B.EnzoMethodMHDVlct()
    blk = B.Block(n, g, w, dtype=dtype)
    mx, my, mz = blk.m
    rng = np.random.default_rng(sum(n) + g)
    A = (rng.standard_normal((mz + 1, my + 1, mx)),
         rng.standard_normal((mz + 1, my, mx + 1)),
         rng.standard_normal((mz, my + 1, mx + 1)))
    dA = [torch.from_numpy(a).cuda() for a in A]
    meth.initialize_bfield_from_potential(blk, *dA)
    torch.cuda.synchronize()
    npdt = np.float64 if dtype == torch.float64 else np.float32
    faces, cells = O.bfield_from_potential(*A, w, npdt)
    got = blk.to_numpy()
    for k, ref in zip(FACES + CELLS, faces + cells):
        assert got[k].shape == ref.shape, k
        assert np.array_equal(got[k].astype(npdt), ref), k


def test_bfield_from_potential_rejects_bad_input():
    meth = B.EnzoMethodMHDVlct()
    blk = B.Block((4, 4, 4), 3)
    mx, my, mz = blk.m
    good = [torch.zeros(s, dtype=torch.float64, device="cuda")
            for s in ((mz + 1, my + 1, mx), (mz + 1, my, mx + 1), (mz, my + 1, mx + 1))]
    with pytest.raises(ValueError):
        meth.initialize_bfield_from_potential(blk, good[1], good[0], good[2])
    hydro = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc")
    hblk = B.Block((4, 4, 4), 3, mhd=False)
    with pytest.raises(capi.MhdError):
        hydro.initialize_bfield_from_potential(hblk, *good)
