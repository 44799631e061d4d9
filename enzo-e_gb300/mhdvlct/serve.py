"""Serving front-end: submit independent MHD solves to the continuous-batching
scheduler of libmhdvlct_gb300.so and collect their results and latencies."""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import capi
from .block import make_params
from . import ic

QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3
FIELDS_IN = ("density", "velocity_x", "velocity_y", "velocity_z",
             "total_energy", "bfield_x", "bfield_y", "bfield_z", "bfieldi_x",
             "bfieldi_y", "bfieldi_z")
FIELDS_OUT = ("density", "velocity_x", "velocity_y", "velocity_z",
              "total_energy", "bfield_x", "bfield_y", "bfield_z")


class Server:
    def __init__(self, hbm_budget_bytes: int, max_active: int = 64, **params):
        p = make_params(**params)
        h = ctypes.c_void_p()
        capi.check(capi.lib().mhdserve_create(ctypes.byref(p), hbm_budget_bytes,
                                              max_active, ctypes.byref(h)))
        self.h = h
        self._keep = {}
        self.meta = {}

    def close(self):
        if self.h:
            capi.lib().mhdserve_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _err(self) -> str:
        return capi.lib().mhdserve_last_error_string(self.h).decode()

    def submit(self, state: dict, n: int, cycles: int, solver: str, recon: str,
               box: float = 1.0) -> int:
        mhd = solver != "hllc"
        req = capi.MhdServeRequest()
        req.n = n
        req.cycles = cycles
        req.riemann_solver = solver.encode()
        req.reconstruct_method = recon.encode()
        req.mhd = int(mhd)
        req.box_size = box
        keep = []
        for k, name in enumerate(FIELDS_IN):
            if not mhd and k >= 5:
                break
            a = np.ascontiguousarray(state[name], dtype=np.float32)
            keep.append(a)
            req.init[k] = a.ctypes.data
        t = ctypes.c_int()
        rc = capi.lib().mhdserve_submit(self.h, ctypes.byref(req), ctypes.byref(t))
        if rc != capi.MHD_OK:
            raise capi.MhdError(rc, self._err())
        self.meta[t.value] = (n, mhd, cycles)
        return t.value

    def pump(self, iterations: int = 1) -> None:
        capi.check(capi.lib().mhdserve_pump(self.h, iterations))

    def poll(self, ticket: int) -> int:
        s = ctypes.c_int()
        capi.check(capi.lib().mhdserve_poll(self.h, ticket, ctypes.byref(s)))
        return s.value

    def result(self, ticket: int) -> tuple[dict, float]:
        n, mhd, _ = self.meta[ticket]
        nf = 8 if mhd else 5
        outs = [np.empty((n, n, n), dtype=np.float32) for _ in range(nf)]
        arr = (ctypes.c_void_p * 8)(*([o.ctypes.data for o in outs] + [None] * (8 - nf)))
        t = ctypes.c_double()
        rc = capi.lib().mhdserve_result(self.h, ticket, arr, ctypes.byref(t))
        if rc != capi.MHD_OK:
            raise capi.MhdError(rc, self._err())
        return dict(zip(FIELDS_OUT, outs)), t.value

    def timing(self, ticket: int) -> tuple[float, float, float]:
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        capi.check(capi.lib().mhdserve_timing(self.h, ticket, ctypes.byref(a),
                                              ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def drain(self, tickets, timeout_s: float = 600.0) -> None:
        t0 = time.time()
        while any(self.poll(t) in (QUEUED, RUNNING) for t in tickets):
            self.pump(1)
            if time.time() - t0 > timeout_s:
                raise TimeoutError("serving drain timed out")
            time.sleep(0.0005)


def request_state(n: int, seed: int, mach: float, mhd: bool):
    """The turbulent-box recipe on a single periodic n^3 block."""
    blocks, w = ic.turbulent_box(N=n, nb=1, g=3, seed=seed, mach=mach)
    s = blocks[0]
    if not mhd:
        s = {k: v for k, v in s.items() if not k.startswith("bfield")}
        # hydro energy: drop the magnetic part
        rho = s["density"]
        p = 0.1 * rho
        v2 = s["velocity_x"] ** 2 + s["velocity_y"] ** 2 + s["velocity_z"] ** 2
        s["total_energy"] = p / ((ic.GAMMA - 1.0) * rho) + 0.5 * v2
    return s, w[0] * n
