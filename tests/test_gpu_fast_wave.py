"""The plain-method configuration on the GPU through the C ABI: the linear
fast-magnetosonic wave on one 32^3 periodic block, FP64, run for one period
with Cello's cycle (timestep, clip to the stop time, periodic refresh, step).
The face and centred B are initialised on the device from the edge vector
potential (mhdvlct_block_bfield_from_potential); every field after the period
equals the reference's own CPU run bit for bit (SHA-256 fixtures made by
tests/golden/make_golden_fast_wave.py)."""
import json
import os
import sys

import numpy as np
import pytest
import torch

from mhdvlct import block as B

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from fast_wave_input import G, N, PERIOD, fast_wave_input  # noqa: E402
from golden_input import digest  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(HERE, "golden", "fast_wave.json")))


def test_fast_wave_period_matches_reference_run():
    state, widths, (ax, ay, az) = fast_wave_input(with_potential=True)
    meth = B.EnzoMethodMHDVlct(riemann_solver="hlld", reconstruct_method="plm",
                               courant=0.4, theta_limiter=1.5)
    blk = B.Block(N, G, widths)
    blk.load_numpy({k: v for k, v in state.items() if not k.startswith("bfield")})
    meth.initialize_bfield_from_potential(
        blk, *[torch.from_numpy(a).cuda() for a in (ax, ay, az)])
    torch.cuda.synchronize()
    got = blk.to_numpy()
    for k in ("bfield_x", "bfield_y", "bfield_z", "bfieldi_x", "bfieldi_y", "bfieldi_z"):
        assert digest(got[k]) == GOLDEN["input_sha256"][k], k
    time, cycles = 0.0, 0
    while True:
        dt = min(meth.timestep(blk), PERIOD - time)
        if not time < PERIOD:
            break
        meth.fill_ghosts_periodic(blk)
        meth.compute(blk, dt)
        time += dt
        cycles += 1
    torch.cuda.synchronize()
    assert cycles == GOLDEN["cycles"]
    out = blk.to_numpy()
    for k, want in GOLDEN["output_sha256"].items():
        assert digest(out[k]) == want, k
    act = (slice(G, G + N),) * 3
    l1 = float(np.mean(np.abs(out["density"][act] - state["density"][act])))
    assert l1 == GOLDEN["density_l1_vs_initial"]
