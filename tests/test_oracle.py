"""CPU tests of the oracle (the restated reference algorithm)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from mhdvlct import ic
from helpers import oracle_block, oracle_params

G53 = 1.6666666666666667
MHD_FIELDS = ["rho", "vx", "vy", "vz", "pressure", "bx", "by", "bz"]


def _linear_wave(wave, N, stop, mhd, solver):
    b = O.Block((2 * N, N, N), 3, (3.0 / (2 * N), 1.5 / N, 1.5 / N), mhd=mhd)
    O.inclined_wave(b, wave)
    b0 = b.copy()
    prm = O.params(riemann=solver, recon=O.PLM, mhd=mhd, theta_limiter=2.0,
                   gamma=G53, courant=0.4)
    O.evolve_periodic(prm, b, stop)
    fields = MHD_FIELDS if mhd else MHD_FIELDS[:5]
    return O.l1_error_norm(b0, b, fields, G53, N)


# Published L1 error norms of the reference's linear-wave regression tests
# (input/vlct/run_MHD_linear_wave_test.py:178-188).  The reference compares
# them at rtol 1e-13 on its own build machine; the value depends on the build
# (FMA contraction alone moves it by ~4e-9 relative), so the bit-level pin is
# the comparison with the reference's own compiled sources below and these
# published numbers are checked to 1e-8.
@pytest.mark.parametrize("wave,N,stop,ref", [
    ("fast", 16, 0.5, 1.6388526155394664e-07),
    ("alfven", 16, 1.0, 1.927245356389947e-07),
    ("mhd_entropy", 16, 1.0, 1.0021263485338544e-07),
])
def test_linear_wave_golden_l1(wave, N, stop, ref):
    l1 = _linear_wave(wave, N, stop, True, O.HLLD)
    assert abs(l1 - ref) / ref < 1e-8, (l1, ref)


def test_divergence_free_after_steps():
    state, w = ic.smooth_block(8, 3, seed=3)
    b = oracle_block(state, 8, 3, w)
    prm = oracle_params()
    for _ in range(3):
        dt = O.timestep(prm, b)
        O.fill_ghosts_periodic(b)
        O.step(prm, b, dt)
    g, n = 3, 8
    fx, fy, fz = b.f["bfx"], b.f["bfy"], b.f["bfz"]
    s = slice(g, g + n)
    div = ((fx[s, s, g + 1:g + n + 1] - fx[s, s, g:g + n]) / w[0] +
           (fy[s, g + 1:g + n + 1, s] - fy[s, g:g + n, s]) / w[1] +
           (fz[g + 1:g + n + 1, s, s] - fz[g:g + n, s, s]) / w[2])
    assert np.abs(div).max() < 1e-13


def test_ghost_fill_periodic_copies_interior():
    state, w = ic.smooth_block(6, 3, seed=1)
    b = oracle_block(state, 6, 3, w)
    O.fill_ghosts_periodic(b)
    r = b.f["rho"]
    assert np.array_equal(r[0:3, 3:9, 3:9], r[6:9, 3:9, 3:9])
    assert np.array_equal(r[9:12, :, :], r[3:6, :, :])
    # face-centred along x: boundary faces 3 and 9 untouched, 0..2 <- 6..8
    fx = b.f["bfx"]
    assert np.array_equal(fx[:, :, 0:3], fx[:, :, 6:9])
    assert np.array_equal(fx[:, :, 10:13], fx[:, :, 4:7])


# The slow wave and the HLLC sound wave at N=16 (input/vlct/
# run_MHD_linear_wave_test.py:184, run_HD_linear_wave_test.py:70); the N=32
# norms run on the CUDA path in tests/test_gpu_known_answers.py.
@pytest.mark.parametrize("wave,stop,ref,mhd,solver", [
    ("slow", 2.0, 2.2373810027584788e-07, True, O.HLLD),
    ("sound", 1.0, 1.3704437791196907e-07, False, O.HLLC),
])
def test_linear_wave_golden_l1_slow_and_sound(wave, stop, ref, mhd, solver):
    l1 = _linear_wave(wave, 16, stop, mhd, solver)
    assert abs(l1 - ref) / ref < 1e-8, (l1, ref)


def test_passive_sound_wave_golden_l1():
    """input/vlct/run_passive_advect_sound_test.py:66, x-aligned: the L1
    norm over the hydro fields, B and the passive scalar after one period."""
    import known_answers as K
    state, n, w = K.passive_sound(0)
    b = O.Block(n, 3, w, mhd=True, npassive=1)
    for k, v in state.items():
        if k == "red":
            b.f["pass0"][...] = v
        elif ic.ORACLE_NAME.get(k) in b.f:
            b.f[ic.ORACLE_NAME[k]][...] = v
    prm = O.params(riemann=O.HLLD, recon=O.PLM, mhd=True, theta_limiter=2.0,
                   gamma=G53, courant=0.4)
    O.evolve_periodic(prm, b, 1.0)
    got = {k: b.f[ic.ORACLE_NAME[k]] for k in state if k in ic.ORACLE_NAME}
    got["red"] = b.f["pass0"]
    names = ["density", "velocity_x", "velocity_y", "velocity_z", "total_energy",
             "bfield_x", "bfield_y", "bfield_z", "red"]
    l1 = K.sim_l1(state, got, names, 3, n)
    ref = 6.918011605252798e-08
    assert abs(l1 - ref) / ref < 1e-8, (l1, ref)
