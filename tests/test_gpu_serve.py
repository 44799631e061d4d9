"""Continuous-batching server: admission against a memory budget, overlap of
independent requests, isolation (a result is bit-identical alone and in a
mix), and failure handling (a poisoned input fails only its own request)."""
import numpy as np
import pytest

from mhdvlct import capi
from mhdvlct.serve import DONE, FAILED, Server, request_state

pytestmark = pytest.mark.gpu


def _req(n, seed, mach, solver):
    s, box = request_state(n, seed, mach, solver != "hllc")
    return s, box


def test_same_result_alone_and_in_mix():
    sA, boxA = _req(16, 1, 1.5, "hlld")
    alone = Server(8 << 30, max_active=8)
    ta = alone.submit(sA, 16, 4, "hlld", "plm", boxA)
    alone.drain([ta])
    ra, _ = alone.result(ta)
    alone.close()

    mix = Server(8 << 30, max_active=8)
    tickets = []
    for i, (n, solver, recon) in enumerate([(24, "hlle", "nn"), (12, "hllc", "plm"),
                                            (20, "hlld", "plm")]):
        s, box = _req(n, 10 + i, 2.0, solver)
        tickets.append(mix.submit(s, n, 5, solver, recon, box))
    tA = mix.submit(sA, 16, 4, "hlld", "plm", boxA)
    mix.drain(tickets + [tA])
    rb, _ = mix.result(tA)
    for k in ra:
        assert np.array_equal(ra[k], rb[k]), k
    for t in tickets:
        out, tsim = mix.result(t)
        assert tsim > 0
        assert all(np.isfinite(v).all() for v in out.values())
    mix.close()


def test_admission_budget_and_rejection():
    s, box = _req(16, 3, 1.0, "hlld")
    # room for about two 16^3 requests at a time
    srv = Server(int(2.5 * (4 * (2 * 8 * 22 ** 3 + 9 * 23 * 22 ** 2 + 22 ** 3)
                              + (1 << 20))), max_active=8)
    ts = [srv.submit(s, 16, 3, "hlld", "plm", box) for _ in range(5)]
    srv.drain(ts)
    assert all(srv.poll(t) == DONE for t in ts)
    # admission never exceeded the budget: at most two ran at any instant
    # (checked at every admission, where the running count can rise)
    spans = [srv.timing(t) for t in ts]
    for _, a_i, _ in spans:
        running = sum(1 for _, a_j, d_j in spans if a_j <= a_i < d_j)
        assert running <= 2
    big, bbox = _req(64, 4, 1.0, "hlld")
    with pytest.raises(capi.MhdError):
        srv.submit(big, 64, 2, "hlld", "plm", bbox)
    srv.close()


def test_poisoned_request_fails_alone():
    good, box = _req(12, 5, 1.0, "hlld")
    bad = {k: v.copy() for k, v in good.items()}
    bad["density"][5, 5, 5] = np.nan
    srv = Server(4 << 30)
    tg = srv.submit(good, 12, 3, "hlld", "plm", box)
    tb = srv.submit(bad, 12, 3, "hlld", "plm", box)
    srv.drain([tg, tb])
    assert srv.poll(tg) == DONE
    assert srv.poll(tb) == FAILED
    with pytest.raises(capi.MhdError):
        srv.result(tb)
    srv.close()


def test_invalid_request_rejected():
    s, box = _req(12, 6, 1.0, "hlld")
    srv = Server(1 << 30)
    with pytest.raises(capi.MhdError):
        srv.submit(s, 12, 2, "hllc_bad", "plm", box)
    with pytest.raises(capi.MhdError):
        srv.submit(s, 12, 2, "hlld", "weno", box)
    srv.close()
