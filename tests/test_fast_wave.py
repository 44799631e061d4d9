"""The plain-method configuration on the CPU: a linear fast-magnetosonic wave
on one 32^3 periodic block (HLLD + PLM, CFL 0.4, FP64) run for one period.
The input is bit-identical to the one tests/golden/make_golden_fast_wave.py
fed the reference's own code, and the oracle's run reproduces the reference's
every field bit for bit."""
import json
import os
import sys

import numpy as np

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from fast_wave_input import G, N, PERIOD, fast_wave_input  # noqa: E402
from golden_input import digest  # noqa: E402
from make_golden_fast_wave import ORACLE_NAME, params  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "fast_wave.json")))


def test_input_is_the_fixture_input():
    state, _ = fast_wave_input()
    for k, v in state.items():
        assert digest(v) == GOLDEN["input_sha256"][k], k


def test_oracle_period_matches_reference_run():
    state, widths = fast_wave_input()
    b = O.Block(N, G, widths)
    for k, v in state.items():
        b.f[ORACLE_NAME[k]][...] = v
    cycles = O.evolve_periodic(params(), b, PERIOD)
    assert cycles == GOLDEN["cycles"]
    for k, o in ORACLE_NAME.items():
        assert digest(b.f[o]) == GOLDEN["output_sha256"][k], k
    act = (slice(G, G + N),) * 3
    l1 = float(np.mean(np.abs(b.f["rho"][act] - state["density"][act])))
    assert l1 == GOLDEN["density_l1_vs_initial"]
