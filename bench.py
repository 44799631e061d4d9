#!/usr/bin/env python3
"""VL+CT MHD benchmark on one GB300 (the driver's bench contract).

Workload: the 256^3 periodic turbulent box split into 512 blocks of 32^3
active cells (3 ghost layers), HLLD Riemann solver + PLM reconstruction,
gamma = 5/3, p = 0.1 rho, lognormal density (sigma_ln = 0.5), k^-2 Gaussian
velocity at rms Mach 2, B = (0.2, 0, 0) + curl of a k^-3 vector potential
(plasma beta ~ 1); synthetic seeded data of the reference workload's shape.

A "step" is one full cycle of the path over the whole box: the CFL timestep
(global min over blocks), the ghost refresh between blocks and the two VL+CT
stages.  `value` is zone-updates/s of the batched FP32 form with the state
resident in HBM (the cycle replayed as a CUDA graph); `e2e` is the same
through the C ABI with the state copied from pinned host memory before and
back to the host after every step.  Extra keys report the plain per-block
FP64 path (the Method called block by block), the batched FP64 form, a
serving stream, and a two-level static-mesh-refinement run with flux
correction (`smr`: 960 hydro leaves of 32^3, the mesh refresh and the
correction inside the cycle graph, with the drift of the conserved totals).

Usage:  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "enzo-e_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

N_BOX = 256
N_BLOCKS_SIDE = 8
GHOST = 3
COURANT = 0.4
N_STATE = 11  # rho, v x3, etot, B_cell x3, B_face x3
METRIC = "VL+CT MHD zone-updates/s, batched FP32 vs plain FP64 on 1 GB300; p99 solve latency"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_BOX)
    ap.add_argument("--nb", type=int, default=N_BLOCKS_SIDE)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--cpu-sample-blocks", type=int, default=512)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--mode", default="main",
                    choices=["main", "amr", "serve", "precision", "fc", "smr", "extras"],
                    help="main: the contract line; amr / serve / precision: the "
                         "mixed-size block set, the serving stream, the FP32-vs-FP64 "
                         "study (one JSON line each)")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=48)
    ap.add_argument("--smr-root", type=int, default=8,
                    help="smr mode: root blocks per axis (the central half is refined)")
    ap.add_argument("--no-smr", action="store_true",
                    help="main mode: skip the static-mesh-refinement key")
    ap.add_argument("--smr-fc", action="store_true",
                    help="smr mode: store the boundary fluxes and apply the flux "
                         "correction in every cycle (Method list mhd_vlct, flux_correct)")
    ap.add_argument("--precision-n", type=int, default=512)
    ap.add_argument("--precision-cycles", type=int, default=50)
    ap.add_argument("--tile", type=str, default="",
                    help="force the stage tiles, e.g. 24x12 or 30x10,28x14 (stage 1, "
                         "stage 2; skips the autotuner)")
    return ap.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------- CPU baseline
def _cpu_worker(paths, n, w, barrier, steps):
    """One CPU worker of the baseline: loads its share of the sampled blocks
    into oracle blocks once (untimed), then for every step runs one cycle
    (timestep, periodic ghost fill, step) of each of them between two
    barriers, so that the parent times compute only."""
    sys.path.insert(0, ROOT)
    sys.path.insert(0, PKG)
    import numpy as np
    from oracle import oracle as O
    from mhdvlct import ic
    blocks = []
    for path in paths:
        s = np.load(path)
        b = O.Block(n, GHOST, w)
        for k in s.files:
            if k in ic.ORACLE_NAME and ic.ORACLE_NAME[k] in b.f:
                b.f[ic.ORACLE_NAME[k]][...] = s[k]
        blocks.append(b)
    prm = O.params(riemann=O.HLLD, recon=O.PLM, courant=COURANT)
    for _ in range(steps):
        barrier.wait()
        for b in blocks:
            dt = O.timestep(prm, b)
            O.fill_ghosts_periodic(b)
            O.step(prm, b, dt)
        barrier.wait()


def cpu_sample(blocks, widths, nblocks, tmpdir):
    """Write the first `nblocks` blocks of the workload (FP64) to `tmpdir` for
    the CPU workers; returns the work list."""
    import numpy as np
    n = blocks[0]["density"].shape[0] - 2 * GHOST
    work = []
    for i in range(min(nblocks, len(blocks))):
        path = os.path.join(tmpdir, f"block{i}.npz")
        np.savez(path, **{k: np.asarray(v, dtype=np.float64) for k, v in blocks[i].items()
                          if k != "pressure"})
        work.append((path, n, tuple(widths)))
    return work


def cpu_baseline(work, steps=1):
    """Time the CPU oracle (a port of the reference's CPU path) over the
    sampled blocks with every host core: one process per core, each holding an
    equal share of the blocks, loaded before the timing starts.  Each
    step is one cycle of every sampled block, timed between two barriers that
    every worker and this process pass.  Returns (zone-updates/s per step,
    cores, wall seconds of the last step)."""
    from oracle import oracle as O
    O.build()
    cores = min(os.cpu_count() or 1, len(work))
    ctx = mp.get_context("spawn")
    n, w = work[0][1], work[0][2]
    shares = [[p for p, _, _ in work[i::cores]] for i in range(cores)]
    barrier = ctx.Barrier(cores + 1)
    procs = [ctx.Process(target=_cpu_worker, args=(sh, n, w, barrier, steps + 1))
             for sh in shares]
    for p_ in procs:
        p_.start()
    zones = len(work) * n ** 3
    vals, el = [], 0.0
    try:
        for k in range(steps + 1):  # the first step warms the workers
            # a worker that died breaks the barrier at the timeout
            barrier.wait(timeout=600)
            t0 = time.perf_counter()
            barrier.wait(timeout=600)
            el = time.perf_counter() - t0
            if k > 0:
                vals.append(zones / el)
    finally:
        for p_ in procs:
            p_.join(timeout=60)
            if p_.is_alive():
                p_.terminate()
    return vals, cores, el


def run_reference(a, rank, world):
    """The reference arm: the CPU oracle (the reference's VL+CT restated in
    C++, compiled for the host) over the turbulent box's blocks on every host
    core, `warmup` untimed then `steps` timed samples of one cycle each."""
    if rank != 0:
        return
    import numpy as np
    from mhdvlct import ic
    n = a.n // a.nb
    blocks, widths = ic.turbulent_box(N=a.n, nb=a.nb, g=GHOST, seed=1, mach=2.0,
                                      dtype=np.float64)
    sample = max(1, min(a.cpu_sample_blocks, len(blocks)))
    with tempfile.TemporaryDirectory() as td:
        work = cpu_sample(blocks, widths, sample, td)
        del blocks
        vals, cores, el = cpu_baseline(work, steps=a.warmup + a.steps)
    vals = vals[a.warmup:]
    value = statistics.median(vals)
    desc = (f"{sample} of the {a.nb ** 3} blocks of {n}^3 (+{GHOST} ghosts), one cycle "
            f"(timestep, ghost fill, VL+CT step) per sample step, CPU oracle restating "
            f"the reference's C++ (g++ -O3, no FMA contraction), blocks loaded before "
            f"timing, one process per core, {el:.1f} s wall per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "zone-updates/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup,
        # one cycle of the sampled blocks at the median rate
        "ms_per_step": sample * n ** 3 / value * 1e3,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"turbulent box {a.n}^3 in {a.nb ** 3} blocks of {n}^3 "
                               f"(+{GHOST} ghosts), HLLD+PLM, gamma 5/3, CFL {COURANT}, "
                               f"global dt, one cycle per step",
                   "sample": desc},
        "cpu_baseline": {"value": value, "unit": "zone-updates/s", "cores": cores,
                         "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "zone-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------- clocks
class Clocks:
    def __init__(self, device_index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        self.idx = device_index

    def start(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ helpers
def _cudart():
    from mhdvlct import capi
    capi.lib()
    path = None
    with open("/proc/self/maps") as f:
        for line in f:
            if "libcudart" in line:
                path = line.split()[-1]
                break
    rt = ctypes.CDLL(path or "libcudart.so")
    rt.cudaMemcpyAsync.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                              ctypes.c_int]
    return rt


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _compute_roofline(zone_rate, stage_ms, zones):
    """The compute side of the roofline (the kernels are issue-bound, not
    HBM-bound): the instruction issue of the dominant stage kernel against the
    GPU's issue rate, and the FP32 operations of the cycle against the FP32
    peak, from the per-zone figures of the committed ncu summary
    (profiles/ncu_instructions.json) and of the op-counting oracle
    (profiles/flops_per_zone.json).  Peaks are nominal: 152 SMs x 4 schedulers
    x 1 warp-instruction per cycle, and 152 SMs x 128 FP32 lanes x 2 (FMA),
    at the maximum SM clock."""
    try:
        ins = json.load(open(os.path.join(ROOT, "profiles", "ncu_instructions.json")))["per_zone"]
        alg = json.load(open(os.path.join(ROOT, "profiles", "flops_per_zone.json")))
        alg_flops = alg["configs"]["hlld_plm"]["flops_per_zone_update"]
    except (OSError, KeyError, ValueError):
        return None
    nsm, clk = 152, 2.07e9
    issue_peak = nsm * 4 * clk
    fp32_peak = nsm * 128 * 2 * clk / 1e12
    s2 = ins["stage2_full_dt"]
    issue = s2["warp_inst"] * zones / (stage_ms["stage2_full_dt"] / 1e3)
    flops_exec = ins["stage1_half_dt"]["fp32_flops"] + s2["fp32_flops"]
    return {
        "bound": "issue", "kernel": "stage2_full_dt", "unit": "warp-inst/s",
        "achieved": issue, "peak": issue_peak, "frac": issue / issue_peak,
        "peak_kind": "nominal (152 SMs x 4 schedulers x 1 warp-inst/cycle x 2070 MHz)",
        "warp_inst_per_zone": s2["warp_inst"],
        "fp32": {"flops_per_zone_algorithmic": alg_flops,
                 "flops_per_zone_executed": flops_exec,
                 "achieved_tflops": flops_exec * zone_rate / 1e12,
                 "peak_tflops": fp32_peak, "frac": flops_exec * zone_rate / 1e12 / fp32_peak,
                 "arithmetic_intensity_flop_per_byte": alg_flops / (5 * N_STATE * 4),
                 "ridge_flop_per_byte": fp32_peak * 1e12 / (_peaks()[0] * 1e9),
                 "peak_kind": "nominal (152 SMs x 128 lanes x 2 x 2070 MHz)"}}


def _traffic(kernel_key, zones):
    """DRAM bytes per launch of the dominant kernel: the ncu-measured bytes
    per active zone of that kernel (profiles/ncu_traffic.json, captured on a
    smaller box of the same 32^3 blocks) times this launch's zones."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            t = json.load(f)
        return t["bytes_per_zone"][kernel_key] * zones
    except (OSError, ValueError, KeyError):
        return None


def aggregate(world: int, zones_per_rank: int, steps: int, ms_local: float):
    """Whole-job throughput: every rank advances its own replica of the box
    (no data-path collective); the job time is the max over ranks."""
    t_max = ms_local
    if world > 1:
        import torch
        import torch.distributed as dist
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([ms_local], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    return world * zones_per_rank * steps / (t_max / 1e3), t_max


def make_batch(meth, blocks, widths, dtype, nb):
    """Batch of nb^3 equal blocks of a periodic brick."""
    from mhdvlct import ic
    n_blk = len(blocks)
    n = blocks[0]["density"].shape[0] - 2 * GHOST
    return make_batch_general(meth, blocks, [(n, n, n)] * n_blk,
                              [tuple(widths)] * n_blk, dtype, ic.brick_neighbors(nb))


FIELD_KEYS = ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy",
              "internal_energy", "bfield_x", "bfield_y", "bfield_z", "bfieldi_x",
              "bfieldi_y", "bfieldi_z")


def view_pointers(v):
    return {"density": v.density, "velocity_x": v.velocity[0],
            "velocity_y": v.velocity[1], "velocity_z": v.velocity[2],
            "total_energy": v.total_energy, "internal_energy": v.internal_energy,
            "bfield_x": v.bfield[0], "bfield_y": v.bfield[1], "bfield_z": v.bfield[2],
            "bfieldi_x": v.bfieldi[0], "bfieldi_y": v.bfieldi[1],
            "bfieldi_z": v.bfieldi[2]}


class _DevArray:
    """A raw device array exposed through __cuda_array_interface__, so that
    torch.as_tensor views it without a copy."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"data": (int(ptr), False), "shape": tuple(shape),
                                         "typestr": typestr, "strides": None, "version": 3}


def error_vs_fp64(h32, h64, dims, widths, ghost=GHOST):
    """Per-field relative L1 error of an FP32 batch's current state against
    an FP64 batch's, over the active zones of every block (every interior
    face for the face-centred B), computed on the device; plus the FP32
    state's normalised max |div B| (|div B| dx / max |B|) from the batch
    diagnostics."""
    import torch
    from mhdvlct import capi
    L = capi.lib()
    num, den = {}, {}
    for i, d in enumerate(dims):
        v32, v64 = capi.MhdBlockView(), capi.MhdBlockView()
        capi.check(L.mhdvlct_batch_block_view(h32, i, ctypes.byref(v32)))
        capi.check(L.mhdvlct_batch_block_view(h64, i, ctypes.byref(v64)))
        p32, p64 = view_pointers(v32), view_pointers(v64)
        m = [x + 2 * ghost for x in d]
        for k in FIELD_KEYS:
            if not p32[k]:
                continue
            shp = [m[2], m[1], m[0]]
            act = [slice(ghost, ghost + d[2 - a]) for a in range(3)]
            if k.startswith("bfieldi"):
                ax = 2 - "xyz".index(k[-1])
                shp[ax] += 1
                act[ax] = slice(ghost, ghost + d[2 - ax] + 1)
            a = torch.as_tensor(_DevArray(p32[k], shp, "<f4"), device="cuda")[tuple(act)]
            r = torch.as_tensor(_DevArray(p64[k], shp, "<f8"), device="cuda")[tuple(act)]
            num[k] = num.get(k, 0.0) + (a.double() - r).abs().sum()
            den[k] = den.get(k, 0.0) + r.abs().sum()
    err = {k: float(num[k] / den[k]) for k in num if float(den[k]) > 0}
    diag = (ctypes.c_double * 8)()
    capi.check(L.mhdvlct_batch_diagnostics(h32, diag, None))
    divb = diag[6] * widths[0][0] / diag[7] if diag[7] > 0 else 0.0
    return {"per_field_rel_l1": err, "max_rel_l1": max(err.values()),
            "max_divb_normalised": divb}


def plain_rate(meth, hb, nblocks, zones, cycles, sp):
    """Zone-updates/s of the per-block Method calls over the blocks of batch
    hb (the blocks' fields are the batch's): per cycle every block's
    mhdvlct_block_timestep_device into a device slot, mhdvlct_dt_min_device,
    the batch's ghost refresh, then mhdvlct_block_step_device_dt per block.
    One untimed cycle first; timed with CUDA events on the stream."""
    import torch
    from mhdvlct import capi
    L = capi.lib()
    views = []
    for i in range(nblocks):
        v = capi.MhdBlockView()
        capi.check(L.mhdvlct_batch_block_view(hb, i, ctypes.byref(v)))
        views.append(v)
    slots = torch.zeros(nblocks, dtype=torch.float64, device="cuda")
    dmin = torch.zeros(1, dtype=torch.float64, device="cuda")

    def cycle():
        for i, v in enumerate(views):
            capi.check(L.mhdvlct_block_timestep_device(meth.handle, ctypes.byref(v),
                                                       slots.data_ptr() + 8 * i, sp),
                       meth.handle)
        capi.check(L.mhdvlct_dt_min_device(meth.handle, slots.data_ptr(), nblocks,
                                           dmin.data_ptr(), sp), meth.handle)
        capi.check(L.mhdvlct_batch_refresh(hb, sp))
        for v in views:
            capi.check(L.mhdvlct_block_step_device_dt(meth.handle, ctypes.byref(v),
                                                      dmin.data_ptr(), sp), meth.handle)
    cycle()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(cycles):
        cycle()
    e1.record(stream)
    torch.cuda.synchronize()
    return zones * cycles / (e0.elapsed_time(e1) / 1e3)


def make_batch_general(meth, blocks, dims, widths, dtype, nbr, ghost=GHOST, npass=0,
                       gravity=False):
    """Batch of arbitrary blocks: dims/widths per block, nbr the 27-neighbour
    table (nblocks x 27); blocks' host arrays are copied into the pool (with
    npass passive scalars passive_k and, with gravity, acceleration_x/y/z)."""
    import numpy as np
    from mhdvlct import capi
    n_blk = len(dims)
    cd = (ctypes.c_int * (3 * n_blk))(*[int(x) for d in dims for x in d])
    ws = (ctypes.c_double * (3 * n_blk))(*[float(x) for w in widths for x in w])
    h = ctypes.c_void_p()
    L = capi.lib()
    capi.check(L.mhdvlct_batch_create_ex(meth.handle, cd, ws, n_blk, ghost, dtype, npass,
                                         int(gravity), ctypes.byref(h)),
               meth.handle, "batch_create")
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    capi.check(L.mhdvlct_batch_set_neighbors(
        h, nbr.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), meth.handle, "nbr")
    rt = _cudart()
    npdt = np.float64 if dtype == capi.MHD_DTYPE_F64 else np.float32
    for i, blk in enumerate(blocks):
        v = capi.MhdBlockView()
        capi.check(L.mhdvlct_batch_block_view(h, i, ctypes.byref(v)))
        ptrs = view_pointers(v)
        for d, ax in enumerate("xyz"):
            ptrs[f"acceleration_{ax}"] = v.acceleration[d]
        for k in range(v.npassive):
            ptrs[f"passive_{k}"] = v.passive[k]
        for k, p in ptrs.items():
            if not p or k not in blk:
                continue
            a = np.ascontiguousarray(blk[k], dtype=npdt)
            assert rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0
    return h


def run_serve(seed=4, nreq=48, rate_hz=30.0, cycles=20, budget_gib=6.0,
              max_active=32):
    """Serving stream (Poisson arrivals of independent solves): grids on
    {32,64,96,128}^3, solver on {hlle, hllc (hydro), hlld}, reconstruction on
    {nn, plm}, FP32, `cycles` cycles each, the turbulent-box recipe at rms Mach
    uniform in [0.5, 4] with a per-request seed.  Initial states are made
    before the clock starts; latency is completion minus arrival."""
    import numpy as np
    from mhdvlct import serve as S
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(nreq):
        n = int(rng.choice([32, 64, 96, 128]))
        solver = str(rng.choice(["hlle", "hllc", "hlld"]))
        recon = str(rng.choice(["nn", "plm"]))
        mach = float(rng.uniform(0.5, 4.0))
        state, box = S.request_state(n, seed * 100003 + i, mach, solver != "hllc")
        # a client holds its fields in the request's precision already
        state = {k: np.ascontiguousarray(v, dtype=np.float32) for k, v in state.items()}
        specs.append((n, solver, recon, state, box))
    # arrival times from a stream of their own, so that a shorter run is a
    # prefix of a longer one (requests and arrivals alike)
    arrivals = np.cumsum(np.random.default_rng(seed + 1).exponential(1.0 / rate_hz, nreq))
    srv = S.Server(int(budget_gib * 2 ** 30), max_active=max_active, courant=COURANT)
    # warm the server, untimed: every (solver, reconstruction) kernel once, and
    # a few requests of every grid size at once, so that its staging buffers
    # exist as they would in a server that has been running
    warm = []
    for solver in ("hlle", "hllc", "hlld"):
        for recon in ("nn", "plm"):
            st, bx = S.request_state(16, 7, 1.0, solver != "hllc")
            warm.append(srv.submit(st, 16, 2, solver, recon, bx))
    for n_w in (32, 64, 96, 128):
        st, bx = S.request_state(n_w, 8, 1.0, True)
        st = {k: np.ascontiguousarray(v, dtype=np.float32) for k, v in st.items()}
        warm += [srv.submit(st, n_w, 1, "hlld", "plm", bx) for _ in range(3)]
    srv.drain(warm)
    tickets = [None] * nreq
    t0 = time.perf_counter()
    nxt = 0
    while True:
        now = time.perf_counter() - t0
        while nxt < nreq and arrivals[nxt] <= now:
            n, solver, recon, state, box = specs[nxt]
            tickets[nxt] = srv.submit(state, n, cycles, solver, recon, box)
            nxt += 1
        srv.pump(1)
        live = [t for t in tickets[:nxt] if srv.poll(t) in (S.QUEUED, S.RUNNING)]
        if nxt == nreq and not live:
            break
        if not live and nxt < nreq:
            time.sleep(max(0.0, min(0.002, arrivals[nxt] - (time.perf_counter() - t0))))
    lat, first, last, failed = [], None, None, 0
    waits, runs = [], []
    for t in tickets:
        if srv.poll(t) != S.DONE:
            failed += 1
            continue
        ts, ta, td = srv.timing(t)
        lat.append(td - ts)
        waits.append(ta - ts)
        runs.append(td - ta)
        first = ts if first is None else min(first, ts)
        last = td if last is None else max(last, td)
    zu = sum(sp[0] ** 3 * cycles for sp in specs)
    srv.close()
    lat_ms = np.array(lat) * 1e3
    return {"requests": nreq, "failed": failed, "cycles_per_request": cycles,
            "arrival_rate_hz": rate_hz, "hbm_budget_gib": budget_gib,
            "p50_ms": float(np.percentile(lat_ms, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat_ms, 99)) if len(lat) else None,
            "p99_admission_wait_ms": float(np.percentile(np.array(waits) * 1e3, 99))
            if waits else None,
            "p99_admitted_to_done_ms": float(np.percentile(np.array(runs) * 1e3, 99))
            if runs else None,
            "zone_updates_per_s": zu / (last - first) if lat else None,
            "grids": [32, 64, 96, 128], "dtype": "f32"}


def amr_blocks(seed=3, counts=((16, 1200), (32, 600), (64, 200)), dtype=None):
    """The mixed-size block set (ic.amr_block_set): Sedov blasts in blocks of
    16^3, 32^3 and 64^3, ghosts from seeded same-size neighbours."""
    import numpy as np
    from mhdvlct import ic
    return ic.amr_block_set(seed=seed, counts=counts, g=GHOST,
                            dtype=np.float32 if dtype is None else dtype)


def run_amr(a):
    """Mixed-size AMR block set, FP32, per-block dt, one persistent launch per
    stage over all blocks, tiles from the autotuner."""
    import numpy as np
    import torch
    from mhdvlct import block as B, capi
    L = capi.lib()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    blocks, dims, widths, nbr = amr_blocks()
    zones = int(sum(d[0] * d[1] * d[2] for d in dims))
    meth = B.EnzoMethodMHDVlct(riemann_solver="hlld", reconstruct_method="plm",
                               courant=COURANT)
    h = make_batch_general(meth, blocks, dims, widths, capi.MHD_DTYPE_F32, nbr)
    tune = None
    if not a.no_tune:
        buf = ctypes.create_string_buffer(8192)
        capi.check(L.mhdvlct_batch_autotune(h, 2, buf, 8192, sp), meth.handle, "autotune")
        tune = json.loads(buf.value.decode() or "{}")
    # one FP32 cycle from the initial state against the FP64 cycle (bit-exact
    # to the oracle) from the same state; the tuned batch then runs on
    err = None
    if not a.no_fp64:
        h64 = make_batch_general(meth, blocks, dims, widths, capi.MHD_DTYPE_F64, nbr)
        capi.check(L.mhdvlct_batch_run(h64, 1, 1, None, sp), meth.handle, "fp64 cycle")
        capi.check(L.mhdvlct_batch_run(h, 1, 1, None, sp), meth.handle, "fp32 cycle")
        torch.cuda.synchronize()
        err = dict(error_vs_fp64(h, h64, dims, widths), cycles=1,
                   reference="batched FP64 (bit-exact to the oracle), same initial state")
        L.mhdvlct_batch_destroy(h64)
    del blocks
    capi.check(L.mhdvlct_batch_run(h, a.warmup, 1, None, sp), meth.handle, "warmup")
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    capi.check(L.mhdvlct_batch_run(h, a.steps, 1, None, sp), meth.handle, "run")
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    prof = (ctypes.c_float * 5)()
    capi.check(L.mhdvlct_batch_profile(h, a.steps, 1, prof, sp), meth.handle, "profile")
    diag = (ctypes.c_double * 8)()
    capi.check(L.mhdvlct_batch_diagnostics(h, diag, sp), meth.handle, "diag")
    L.mhdvlct_batch_destroy(h)
    return {"mode": "amr", "metric": "zone-updates/s (mixed-size AMR block set)",
            "value": zones * a.steps / (ms / 1e3), "unit": "zone-updates/s",
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps,
            "dtype": "f32", "data": "synthetic (seeded Sedov blasts)",
            "config": {"workload": "2000 blocks: 1200 x 16^3, 600 x 32^3, 200 x 64^3 "
                                   "(+3 ghosts), HLLD+PLM, per-block dt",
                       "zones_per_step": zones, "tuning": tune},
            "kernels_ms_per_step": dict(zip(("timestep", "refresh", "stage1_half_dt",
                                             "stage2_full_dt", "cycle"), list(prof))),
            "gpu_launches": 6 * a.steps, "clocks": clk,
            "finite": all(np.isfinite(list(diag))), "error_vs_fp64": err}


SMR_GHOST = 4  # the reference's SMR decks (input/FluxCorrect/inclined_contact.incl)


def smr_state(mesh, i, n, g, domain=1.0):
    """Inclined density contact moving along (1,1,1) on leaf i (hydro): the
    shape of the reference's hd_entropy inclined-wave SMR deck at a large
    amplitude; ghosts left NaN for the first refresh to fill."""
    import numpy as np
    lvl, _ = mesh.leaves[i]
    root_n = mesh.root[0] * n
    h = domain / root_n / 2 ** lvl
    fine = domain / root_n / 2 ** mesh.max_level
    o = [x * fine for x in mesh.origin(i, (n, n, n))]
    ax = [o[a] + (np.arange(n + 2 * g) - g + 0.5) * h for a in range(3)]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    rho = 1.0 + 0.5 * np.sin(2 * np.pi * (x + y + z) / domain)
    v = 0.5
    p = 0.6
    st = {"density": rho, "velocity_x": np.full_like(rho, v),
          "velocity_y": np.full_like(rho, v), "velocity_z": np.full_like(rho, v),
          "pressure": np.full_like(rho, p),
          "total_energy": p / (2.0 / 3.0) / rho + 1.5 * v * v}
    act = tuple(slice(g, g + n) for _ in range(3))
    for k in st:
        a = np.full_like(st[k], np.nan)
        a[act] = st[k][act]
        st[k] = a
    return st, (h, h, h)


def _smr_cpu(n=32, cycles=1):
    """CPU oracle on a two-level sample: a 2^3 root grid of n^3 blocks with
    one root block refined (15 leaves), refresh + dt + step per cycle, one
    core.  Returns zone-updates/s."""
    import numpy as np
    from oracle import oracle as O
    from mhdvlct import capi, mesh as M
    mesh = M.Mesh((2, 2, 2), refine=lambda lvl, c: c == (0, 0, 0))
    g = SMR_GHOST
    prm = O.params(riemann=O.HLLC, recon=O.PLM, mhd=False, courant=COURANT)
    obs, slots = [], []
    for i in range(len(mesh.leaves)):
        st, w = smr_state(mesh, i, n, g)
        ob = O.Block(n, g, w, mhd=False)
        for k, v in st.items():
            ob.f[{"density": "rho", "velocity_x": "vx", "velocity_y": "vy",
                  "velocity_z": "vz", "total_energy": "etot",
                  "pressure": "pressure"}[k]][...] = v
        obs.append(ob)
        slots.append({0: ob.f["rho"], 1: ob.f["vx"], 2: ob.f["vy"], 3: ob.f["vz"],
                      4: ob.f["etot"], 9: ob.f["pressure"]})
    faces = mesh.face_ints()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
    t0 = time.perf_counter()
    for _ in range(cycles):
        dt = min(O.timestep(prm, ob) for ob in obs)
        O.refresh_faces(slots, (n,) * 3, (g,) * 3, faces, cons)
        for ob in obs:
            O.step(prm, ob, dt)
    el = time.perf_counter() - t0
    return len(obs) * n ** 3 * cycles / el, len(obs)


def run_smr(a, root=8, n=32, fc=False):
    """Static mesh refinement, two levels: a periodic root grid of root^3
    blocks of n^3 whose central half along every axis is refined once, hydro
    HLLC + PLM in FP32 with ghost depth 4 (the reference's SMR decks), one
    global dt per cycle; the cycle (dt, mesh refresh with restriction and
    prolongation, two stages and, with fc, the flux correction) replayed as
    one CUDA graph.  The line reports the relative drift of the FP64 mass and
    total-energy totals over the warm-up and timed cycles."""
    import numpy as np
    import torch
    from mhdvlct import block as B, capi, mesh as M
    L = capi.lib()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    lo, hi = root // 4, root - root // 4
    mesh = M.Mesh((root,) * 3, refine=lambda lvl, c: all(lo <= x < hi for x in c))
    g = SMR_GHOST
    nleaf = len(mesh.leaves)
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", courant=COURANT)
    dims = [(n, n, n)] * nleaf
    widths = [(1.0 / (root * n) / 2 ** lvl,) * 3 for lvl, _ in mesh.leaves]
    cd = (ctypes.c_int * (3 * nleaf))(*[n] * (3 * nleaf))
    ws = (ctypes.c_double * (3 * nleaf))(*[x for w in widths for x in w])
    h = ctypes.c_void_p()
    capi.check(L.mhdvlct_batch_create(meth.handle, cd, ws, nleaf, g, capi.MHD_DTYPE_F32,
                                      ctypes.byref(h)), meth.handle, "batch_create")
    rt = _cudart()
    for i in range(nleaf):
        st, _ = smr_state(mesh, i, n, g)
        v = capi.MhdBlockView()
        capi.check(L.mhdvlct_batch_block_view(h, i, ctypes.byref(v)))
        for k, p in view_pointers(v).items():
            if p and k in st:
                arr = np.ascontiguousarray(st[k], dtype=np.float32)
                assert rt.cudaMemcpy(p, arr.ctypes.data, arr.nbytes, 1) == 0
        if v.pressure:
            arr = np.ascontiguousarray(st["pressure"], dtype=np.float32)
            assert rt.cudaMemcpy(v.pressure, arr.ctypes.data, arr.nbytes, 1) == 0
    farr, nf = mesh.face_array()
    cons = capi.MHD_CONSERVATIVE_DEFAULT
    capi.check(L.mhdvlct_batch_set_refresh_faces(h, farr, nf, cons), meth.handle, "faces")
    if fc:
        capi.check(L.mhdvlct_batch_set_flux_correction(h, 0b11111, farr, nf, cons),
                   meth.handle, "flux correction")
    capi.check(L.mhdvlct_batch_refresh(h, sp), meth.handle, "first refresh")
    diag0 = (ctypes.c_double * 8)()
    capi.check(L.mhdvlct_batch_diagnostics(h, diag0, sp), meth.handle, "diag")
    zones = nleaf * n ** 3
    capi.check(L.mhdvlct_batch_run(h, a.warmup, 0, None, sp), meth.handle, "warmup")
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    capi.check(L.mhdvlct_batch_run(h, a.steps, 0, None, sp), meth.handle, "run")
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    prof = (ctypes.c_float * 5)()
    capi.check(L.mhdvlct_batch_profile(h, a.steps, 0, prof, sp), meth.handle, "profile")
    diag = (ctypes.c_double * 8)()
    capi.check(L.mhdvlct_batch_diagnostics(h, diag, sp), meth.handle, "diag")
    L.mhdvlct_batch_destroy(h)
    # compulsory bytes of the refresh: every region's receiver cells written
    # and sender cells read once, over the refreshed fields (rho, v, etot, p)
    fields = 6
    i3 = lambda t: (ctypes.c_int * 3)(*t)  # noqa: E731
    out4 = [(ctypes.c_int * 3)() for _ in range(4)]
    moved = 0
    counts = {-1: 0, 0: 0, 1: 0}
    for s_, r_, t, f, k in mesh.faces():
        counts[t] += 1
        if L.mhdvlct_refresh_face_box(i3((n,) * 3), i3((g,) * 3), i3((0, 0, 0)), t, i3(f),
                                      i3(k), *out4) == 1:
            moved += (int(np.prod(list(out4[1]))) + int(np.prod(list(out4[3]))))
    rbytes = moved * fields * 4
    r_ms = float(prof[1])
    hbm, hbm_kind = _peaks()
    cpu = None
    if not a.no_cpu:
        v_cpu, nb_cpu = _smr_cpu()
        cpu = {"value": v_cpu, "unit": "zone-updates/s", "cores": 1, "kind": "port",
               "sample": f"{nb_cpu} leaves of 32^3 (2^3 root grid, one root block "
                         "refined), FP64 oracle, refresh + dt + step, 1 cycle"}
    drift = {"mass": abs(diag[0] - diag0[0]) / abs(diag0[0]),
             "total_energy": abs(diag[4] - diag0[4]) / abs(diag0[4]),
             "cycles": a.warmup + 2 * a.steps}
    return {"mode": "smr", "metric": "zone-updates/s (static mesh refinement, 2 levels)",
            "flux_correction": fc, "conservation_drift": drift,
            "value": zones * a.steps / (ms / 1e3), "unit": "zone-updates/s",
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps,
            "dtype": "f32", "data": "synthetic (inclined density contact)",
            "config": {"workload": f"{nleaf} leaves of {n}^3 (+{g} ghosts): {root}^3 root "
                                   f"grid, central {hi - lo}^3 refined once; HLLC+PLM "
                                   "hydro, global dt" + ("; flux correction" if fc else ""),
                       "zones_per_step": zones,
                       "faces": {"same": counts[0], "to_finer": counts[1],
                                 "to_coarser": counts[-1]}},
            "kernels_ms_per_step": dict(zip(("timestep", "refresh", "stage1_half_dt",
                                             "stage2_full_dt", "cycle"), list(prof))),
            "refresh": {"algorithmic_bytes": rbytes,
                        "achieved_gbs": rbytes / (r_ms * 1e-3) / 1e9 if r_ms > 0 else None,
                        "peak_gbs": hbm, "peak_kind": hbm_kind,
                        "frac": (rbytes / (r_ms * 1e-3) / 1e9 / hbm) if r_ms > 0 else None},
            "cpu_baseline": cpu, "gpu_launches": 5 * a.steps, "clocks": clk,
            "finite": all(np.isfinite(list(diag)))}


def run_extras(a, npass=2):
    """The gravity source and passive scalars in the batched cycle: the
    turbulent box (HLLD + PLM, FP32) advanced by graph-captured cycles
    (timestep, global min dt, refresh, both stages), without and with
    acceleration fields and npass passive scalars, each variant with default
    tiles and (unless --no-tune) with the autotuner's.  Wall clock around
    a.steps cycles of one mhdvlct_batch_run call, synchronised on both
    sides."""
    import numpy as np
    import torch
    from mhdvlct import block as B, capi, ic
    meth = B.EnzoMethodMHDVlct(riemann_solver="hlld", reconstruct_method="plm",
                               courant=COURANT)
    blocks, w = ic.turbulent_box(N=a.n, nb=a.nb, g=GHOST, seed=1, mach=2.0)
    n = a.n // a.nb
    m = n + 2 * GHOST
    rng = np.random.default_rng(2)
    for st in blocks:
        for ax in "xyz":
            st[f"acceleration_{ax}"] = 0.1 * (rng.random((m, m, m)) - 0.5)
        for k in range(npass):
            st[f"passive_{k}"] = st["density"] * (0.2 + 0.6 * rng.random((m, m, m)))
    nblk = len(blocks)
    L = capi.lib()
    steps = max(1, a.steps)
    out = {"mode": "extras", "workload": f"turbulent box {a.n}^3 in {nblk} blocks of {n}^3 "
                                         f"(+{GHOST} ghosts), HLLD+PLM, FP32",
           "unit": "zone-updates/s", "steps": steps}
    for tag, (np_, grav) in (("plain", (0, False)), ("gravity", (0, True)),
                             ("passive", (npass, False)), ("gravity_passive", (npass, True))):
        h = make_batch_general(meth, blocks, [(n, n, n)] * nblk, [tuple(w)] * nblk,
                               capi.MHD_DTYPE_F32, ic.brick_neighbors(a.nb), npass=np_,
                               gravity=grav)
        t = ctypes.c_double()
        for tuned in ((False, True) if not a.no_tune else (False,)):
            if tuned:
                buf = ctypes.create_string_buffer(4096)
                capi.check(L.mhdvlct_batch_autotune(h, 2, buf, 4096, None), meth.handle,
                           "autotune")
            capi.check(L.mhdvlct_batch_run(h, max(3, a.warmup), 0, ctypes.byref(t), None))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            capi.check(L.mhdvlct_batch_run(h, steps, 0, ctypes.byref(t), None))
            torch.cuda.synchronize()
            el = time.perf_counter() - t0
            out[tag + ("_tuned" if tuned else "")] = a.n ** 3 * steps / el
        L.mhdvlct_batch_destroy(h)
    out["npassive"] = npass
    out["overhead_gravity_passive"] = out["plain"] / out["gravity_passive"] - 1.0
    if not a.no_tune:
        out["overhead_gravity_passive_tuned"] = (
            out["plain_tuned"] / out["gravity_passive_tuned"] - 1.0)
    return out


def run_fc(a, nblocks=64, n=32):
    """Flux correction on the plain per-block path: HLLC + PLM hydro blocks
    (dual energy on), each advanced by timestep + compute, with and without
    storing the dt/dx-scaled boundary fluxes of all six quantities."""
    import numpy as np
    import torch
    from mhdvlct import block as B, serve as S
    meth = B.EnzoMethodMHDVlct(mhd_choice="no_bfield", riemann_solver="hllc",
                               reconstruct_method="plm", dual_energy=True,
                               courant=COURANT)
    out = {"mode": "fc", "workload": f"{nblocks} hydro blocks of {n}^3 (+{GHOST} ghosts), "
                                     f"HLLC+PLM, dual energy, per-block Method calls"}
    for dtype, tag in ((torch.float64, "f64"), (torch.float32, "f32")):
        blocks = []
        for i in range(nblocks):
            st, box = S.request_state(n, 500 + i, 2.0, False)
            st["internal_energy"] = (0.1 * st["density"]) / (
                (5.0 / 3.0 - 1.0) * st["density"])
            blk = B.Block((n, n, n), GHOST, (box / n,) * 3, mhd=False, dual_energy=True,
                          dtype=dtype)
            blk.load_numpy(st)
            blocks.append(blk)
        bufs = [B.FluxBuffers(blk, (0, 1, 2, 3, 4, 5)) for blk in blocks]
        res = {}
        for mode in ("plain", "store_fluxes"):
            def cycle():
                for blk, buf in zip(blocks, bufs):
                    dt = meth.timestep(blk)
                    if mode == "plain":
                        meth.compute(blk, dt)
                    else:
                        meth.compute_store_fluxes(blk, dt, buffers=buf)
            cycle()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(max(1, a.steps)):
                cycle()
            torch.cuda.synchronize()
            el = time.perf_counter() - t0
            res[mode] = nblocks * n ** 3 * max(1, a.steps) / el
        out[tag] = {"plain_zone_updates_per_s": res["plain"],
                    "store_fluxes_zone_updates_per_s": res["store_fluxes"],
                    "overhead": res["plain"] / res["store_fluxes"] - 1.0}
    return out


class _DevArray:
    """A device buffer seen by torch through __cuda_array_interface__."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"data": (int(ptr), False), "shape": tuple(shape),
                                         "typestr": typestr, "version": 3,
                                         "strides": None}


def run_precision(a, cycles=50, N=512, nb=8):
    """FP32 form (float-float internal-energy recovery, FP64 totals and dt)
    against the FP64 form on the same initial state: turbulent box at rms
    Mach 4 with dual energy (eta = 0.001), both advanced with the FP64 form's
    global dt.  Reports per-field relative L1 over the active zones, drift of
    the FP64 conserved totals and max |div B|."""
    import numpy as np
    import torch
    from mhdvlct import block as B, capi, ic
    L = capi.lib()
    sp = torch.cuda.current_stream().cuda_stream
    n = N // nb
    nblk = nb ** 3
    meth = B.EnzoMethodMHDVlct(riemann_solver="hlld", reconstruct_method="plm",
                               courant=COURANT, dual_energy=True, dual_energy_eta=0.001)
    w = (1.0 / N,) * 3
    h64 = make_batch_general(meth, [], [(n, n, n)] * nblk, [w] * nblk,
                             capi.MHD_DTYPE_F64, ic.brick_neighbors(nb))
    h32 = make_batch_general(meth, [], [(n, n, n)] * nblk, [w] * nblk,
                             capi.MHD_DTYPE_F32, ic.brick_neighbors(nb))
    rt = _cudart()

    def upload(i, blk):
        for h, npdt in ((h64, np.float64), (h32, np.float32)):
            v = capi.MhdBlockView()
            capi.check(L.mhdvlct_batch_block_view(h, i, ctypes.byref(v)))
            for k, p in view_pointers(v).items():
                if p and k in blk:
                    a = np.ascontiguousarray(blk[k], dtype=npdt)
                    assert rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0

    # the initial state streams block by block into both forms
    ic.turbulent_box(N=N, nb=nb, g=GHOST, seed=11, mach=4.0, dtype=np.float64,
                     dual_energy=True, sink=upload)
    dts = (ctypes.c_double * nblk)()
    dts32 = (ctypes.c_double * nblk)()
    m = n + 2 * GHOST
    act = (slice(GHOST, GHOST + n),) * 3
    keys = ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy",
            "internal_energy", "bfield_x", "bfield_y", "bfield_z")

    def l1():
        num = {k: 0.0 for k in keys}
        den = {k: 0.0 for k in keys}
        for i in range(nblk):
            v64, v32 = capi.MhdBlockView(), capi.MhdBlockView()
            capi.check(L.mhdvlct_batch_block_view(h64, i, ctypes.byref(v64)))
            capi.check(L.mhdvlct_batch_block_view(h32, i, ctypes.byref(v32)))
            p64, p32 = view_pointers(v64), view_pointers(v32)
            for k in keys:
                x = torch.as_tensor(_DevArray(p64[k], (m, m, m), "<f8"), device="cuda")[act]
                y = torch.as_tensor(_DevArray(p32[k], (m, m, m), "<f4"), device="cuda")[act]
                num[k] += float((y.double() - x).abs().sum())
                den[k] += float(x.abs().sum())
        return {k: num[k] / den[k] if den[k] > 0 else num[k] for k in keys}

    def diag(h):
        d = (ctypes.c_double * 8)()
        capi.check(L.mhdvlct_batch_diagnostics(h, d, sp))
        return list(d)

    d0 = {"fp64": diag(h64), "fp32": diag(h32)}
    report = {"l1": {}, "drift": {}, "max_divb": {}, "max_rel_dt_diff": 0.0}
    t0 = time.perf_counter()
    for c in range(1, cycles + 1):
        capi.check(L.mhdvlct_batch_timestep(h64, dts, sp))
        capi.check(L.mhdvlct_batch_timestep(h32, dts32, sp))
        dtm = min(dts)
        report["max_rel_dt_diff"] = max(report["max_rel_dt_diff"],
                                        abs(min(dts32) - dtm) / dtm)
        glob = (ctypes.c_double * nblk)(*([dtm] * nblk))
        for h in (h64, h32):
            capi.check(L.mhdvlct_batch_refresh(h, sp))
            capi.check(L.mhdvlct_batch_step(h, glob, sp))
        if c in (1, 10, cycles):
            report["l1"][str(c)] = l1()
            dd = {"fp64": diag(h64), "fp32": diag(h32)}
            report.setdefault("max_divb_normalised_by_cycle", {})[str(c)] = {
                k: v[6] * (1.0 / N) / v[7] if v[7] > 0 else None for k, v in dd.items()}
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    for tag, h in (("fp64", h64), ("fp32", h32)):
        d = diag(h)
        ref = d0[tag]
        report["drift"][tag] = {
            "mass": (d[0] - ref[0]) / abs(ref[0]),
            "energy": (d[4] - ref[4]) / abs(ref[4]),
            "momentum": [(d[1 + k] - ref[1 + k]) / max(abs(ref[1 + k]), 1e-300)
                         for k in range(3)],
            "momentum_abs": [d[1 + k] - ref[1 + k] for k in range(3)],
        }
        report["max_divb"][tag] = d[6]
        report["max_divb_normalised"] = report.get("max_divb_normalised", {})
        report["max_divb_normalised"][tag] = d[6] * (1.0 / N) / d[7] if d[7] > 0 else None
    L.mhdvlct_batch_destroy(h64)
    L.mhdvlct_batch_destroy(h32)
    report.update({"mode": "precision", "cycles": cycles, "wall_s": wall,
                   "config": {"workload": f"turbulent box {N}^3 in {nb ** 3} blocks of "
                                          f"{n}^3 (+{GHOST} ghosts), rms Mach 4, HLLD+PLM, "
                                          f"dual energy eta 0.001, FP64 global dt"}})
    return report


def main():
    a = _args()
    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    if a.impl == "reference":
        run_reference(a, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return

    import numpy as np
    import torch
    from mhdvlct import block as B, capi, ic
    torch.cuda.set_device(local)
    if a.mode != "main":
        if rank == 0:
            if a.mode == "amr":
                out = run_amr(a)
            elif a.mode == "serve":
                out = {"mode": "serve", **run_serve(nreq=a.serve_requests)}
            elif a.mode == "fc":
                out = run_fc(a)
            elif a.mode == "smr":
                out = run_smr(a, root=a.smr_root, fc=a.smr_fc)
            elif a.mode == "extras":
                out = run_extras(a)
            else:
                out = run_precision(a, cycles=a.precision_cycles, N=a.precision_n)
            print(json.dumps(out), flush=True)
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return
    L = capi.lib()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    n = a.n // a.nb
    zones = a.n ** 3
    blocks, widths = ic.turbulent_box(N=a.n, nb=a.nb, g=GHOST, seed=1 + rank,
                                      mach=2.0, dtype=np.float64)
    meth = B.EnzoMethodMHDVlct(riemann_solver="hlld", reconstruct_method="plm",
                               courant=COURANT)

    # ---------------------------------------------------- batched FP32 form
    h32 = make_batch(meth, blocks, widths, capi.MHD_DTYPE_F32, a.nb)
    tune = None
    if a.tile:
        # "TXxTY" for both stages, or "TXxTY,TXxTY" for stage 1 and stage 2
        for s_, spec in enumerate((a.tile.split(",") * 2)[:2]):
            tx, ty = (int(v) for v in spec.lower().split("x"))
            capi.check(L.mhdvlct_batch_set_stage_tile(h32, s_, tx, ty, 0, 256),
                       meth.handle, "tile")
        tune = {"forced_tile": a.tile}
    elif not a.no_tune:
        buf = ctypes.create_string_buffer(4096)
        capi.check(L.mhdvlct_batch_autotune(h32, 4, buf, 4096, sp), meth.handle,
                   "autotune")
        tune = json.loads(buf.value.decode() or "{}")
    tsim = ctypes.c_double()
    capi.check(L.mhdvlct_batch_run(h32, a.warmup, 0, ctypes.byref(tsim), sp),
               meth.handle, "warmup")
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    capi.check(L.mhdvlct_batch_run(h32, a.steps, 0, ctypes.byref(tsim), sp),
               meth.handle, "timed run")
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    value, t_max = aggregate(world, zones, a.steps, ms)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()

    # per-kernel breakdown of the same cycle (events between the launches)
    prof = (ctypes.c_float * 5)()
    capi.check(L.mhdvlct_batch_profile(h32, a.steps, 0, prof, sp), meth.handle, "profile")
    k_ts, k_ref, k_s1, k_s2, k_cyc = list(prof)
    bytes_s1 = 2 * N_STATE * 4 * zones  # stage 1 reads U^n, writes U^(n+1/2)
    bytes_s2 = 3 * N_STATE * 4 * zones  # stage 2 reads U^(n+1/2), U^n, writes U^(n+1)
    peak, peak_kind = _peaks()
    if k_s2 >= k_s1:
        dom, dom_ms, dom_bytes = "stage2_full_dt", k_s2, bytes_s2
    else:
        dom, dom_ms, dom_bytes = "stage1_half_dt", k_s1, bytes_s1
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    traffic = _traffic(dom, zones)

    # ------------------------------------------------------ e2e (host data)
    e2e = None
    if not a.no_e2e:
        # the host keeps the state (every block's cells and its current
        # face-B buffer, one or two contiguous segments); each step copies it
        # in, runs one cycle through the C ABI and copies the new state back
        rt = _cudart()
        segp = (ctypes.c_void_p * 2)()
        segb = (ctypes.c_size_t * 2)()
        nseg = ctypes.c_int()

        def segments():
            capi.check(L.mhdvlct_batch_state_segments(h32, segp, segb, 2,
                                                      ctypes.byref(nseg)), meth.handle)
            return [(segp[i], segb[i]) for i in range(nseg.value)]

        total = sum(n for _, n in segments())
        dptr, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
        capi.check(L.mhdvlct_batch_state_region(h32, ctypes.byref(dptr),
                                                ctypes.byref(nbytes)))
        host = torch.empty(nbytes.value, dtype=torch.uint8, pin_memory=True)

        def copy(to_device):
            off = 0
            for p_, n_ in segments():
                if to_device:
                    assert rt.cudaMemcpyAsync(p_, host.data_ptr() + off, n_, 1, sp) == 0
                else:
                    assert rt.cudaMemcpyAsync(host.data_ptr() + off, p_, n_, 2, sp) == 0
                off += n_
            return off

        copy(False)  # the host now holds the current state
        e2e_steps = max(1, min(a.steps, 10))
        groups = 8
        # one warm-up call sets up the copy streams and block groups
        capi.check(L.mhdvlct_batch_run_host(h32, host.data_ptr(), total, 1, groups, None, sp),
                   meth.handle, "e2e warm-up")
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        # every step: the state in from pinned host memory, one cycle, the new
        # state back out, the copies pipelined with the full-dt stage
        capi.check(L.mhdvlct_batch_run_host(h32, host.data_ptr(), total, e2e_steps, groups,
                                            None, sp), meth.handle, "e2e")
        e1.record(stream)
        torch.cuda.synchronize()
        e_ms = e0.elapsed_time(e1)
        e2e = {"value": world * zones * e2e_steps / (e_ms / 1e3),
               "unit": "zone-updates/s", "h2d_bytes_per_step": int(total),
               "d2h_bytes_per_step": int(total), "steps": e2e_steps,
               "path": "mhdvlct_batch_run_host, copies pipelined with the full-dt stage "
                       f"by {groups} block groups"}
    L.mhdvlct_batch_destroy(h32)

    # ------------------------------------------- FP64: batched and plain path
    fp64 = {}
    if not a.no_fp64:
        h64 = make_batch(meth, blocks, widths, capi.MHD_DTYPE_F64, a.nb)
        k64 = max(1, min(a.steps, 3))
        capi.check(L.mhdvlct_batch_run(h64, 1, 0, None, sp))
        torch.cuda.synchronize()
        # the error of one FP32 cycle against the FP64 cycle from the same
        # initial state (the FP64 batched form is bit-exact to the oracle)
        h32e = make_batch(meth, blocks, widths, capi.MHD_DTYPE_F32, a.nb)
        capi.check(L.mhdvlct_batch_run(h32e, 1, 0, None, sp))
        torch.cuda.synchronize()
        fp64["error_vs_fp64"] = dict(
            error_vs_fp64(h32e, h64, [(n, n, n)] * len(blocks), [widths] * len(blocks)),
            cycles=1, reference="batched FP64 (bit-exact to the oracle), same initial state")
        L.mhdvlct_batch_destroy(h32e)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        capi.check(L.mhdvlct_batch_run(h64, k64, 0, None, sp))
        e1.record(stream)
        torch.cuda.synchronize()
        fp64["batched_fp64_zone_updates_per_s"] = zones * k64 / (e0.elapsed_time(e1) / 1e3)
        # plain per-block FP64 and FP32: the Method's timestep and compute
        # called block by block, as Cello drives a Method (the refresh between
        # them batched), with each block's dt kept in a device slot and the
        # min taken on the device, so no call waits for the GPU
        plain64 = plain_rate(meth, h64, len(blocks), zones, max(1, min(a.steps, 2)), sp)
        h32p = make_batch(meth, blocks, widths, capi.MHD_DTYPE_F32, a.nb)
        plain32 = plain_rate(meth, h32p, len(blocks), zones, max(1, min(a.steps, 3)), sp)
        L.mhdvlct_batch_destroy(h32p)
        fp64["plain_fp64_zone_updates_per_s"] = plain64
        fp64["plain_fp32_zone_updates_per_s"] = plain32
        fp64["fp32_batched_over_plain_fp64"] = value / world / plain64
        L.mhdvlct_batch_destroy(h64)

    # -------------------------------------------------------- serving stream
    serving = None
    if rank == 0 and not a.no_serve:
        serving = run_serve(nreq=a.serve_requests)

    # ---------------------- static mesh refinement, with flux correction
    smr = None
    if rank == 0 and not a.no_smr:
        r = run_smr(a, root=a.smr_root, fc=True)
        smr = {k: r[k] for k in ("value", "unit", "ms_per_step", "flux_correction",
                                 "conservation_drift", "kernels_ms_per_step", "refresh",
                                 "cpu_baseline")}
        smr["workload"] = r["config"]["workload"]

    # ----------------------------------------------------------- CPU baseline
    cpu = None
    if rank == 0 and not a.no_cpu:
        sample = max(1, min(a.cpu_sample_blocks, len(blocks)))
        with tempfile.TemporaryDirectory() as td:
            work = cpu_sample(blocks, widths, sample, td)
            vals, cores, el = cpu_baseline(work, steps=2)
        cpu = {"value": vals[-1], "unit": "zone-updates/s", "cores": cores, "kind": "port",
               "sample": f"{sample} of the {a.nb ** 3} blocks of {n}^3 (+{GHOST} ghosts), "
                         f"one cycle each (timestep, ghost fill, step), CPU oracle "
                         f"restating the reference's C++ (g++ -O3, no FMA contraction), "
                         f"blocks loaded before timing, one process per core, "
                         f"{el:.1f} s wall (second of two timed passes)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "zone-updates/s",
            "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": t_max / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded turbulent box of the reference workload's shape)",
            "config": {"workload": f"turbulent box {a.n}^3 in {a.nb ** 3} blocks of {n}^3 "
                                   f"(+{GHOST} ghosts), HLLD+PLM, gamma 5/3, CFL {COURANT}, "
                                   f"global dt, one cycle per step",
                       "l2": "state > L2 (no flush needed)",
                       "zones_per_step": zones, "tuning": tune,
                       "simulated_time": tsim.value},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": traffic,
                         "alg_bytes_per_launch": dom_bytes,
                         "cycle_frac": value / world * 5 * N_STATE * 4 / 1e9 / peak,
                         "compute": _compute_roofline(value / world, {"stage2_full_dt": k_s2},
                                                      zones)},
            "kernels_ms_per_step": {"timestep": k_ts, "refresh": k_ref,
                                    "stage1_half_dt": k_s1, "stage2_full_dt": k_s2,
                                    "cycle": k_cyc},
            "gpu_launches": 6 * a.steps,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "serving": serving,
            "smr": smr,
        }
        line.update(fp64)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
