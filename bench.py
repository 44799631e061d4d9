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
FP64 path (the Method called block by block) and the batched FP64 form.

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
    ap.add_argument("--cpu-sample-blocks", type=int, default=256)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--tile", type=str, default="",
                    help="force the stage tile, e.g. 24x12 (skips the autotuner)")
    return ap.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------- CPU baseline
def _cpu_block_cycle(args):
    """One cycle (timestep, periodic refresh, step) of one block on the CPU
    oracle; returns active zones updated."""
    seed, n = args
    sys.path.insert(0, ROOT)
    sys.path.insert(0, PKG)
    from oracle import oracle as O
    from mhdvlct import ic
    s, w = ic.smooth_block(n, GHOST, seed=seed, amp_v=0.8)
    b = O.Block(n, GHOST, w)
    for k, v in s.items():
        b.f[ic.ORACLE_NAME[k]][...] = v
    prm = O.params(riemann=O.HLLD, recon=O.PLM, courant=COURANT)
    t = time.perf_counter()
    dt = O.timestep(prm, b)
    O.fill_ghosts_periodic(b)
    O.step(prm, b, dt)
    return n ** 3, time.perf_counter() - t


def cpu_baseline(nblocks, n, steps=1):
    """Time the CPU oracle (a port of the reference's CPU path) on `nblocks`
    blocks of n^3 with every host core; returns (zone-updates/s, cores,
    seconds)."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    work = [(1000 + i, n) for i in range(nblocks)]
    with ctx.Pool(cores) as pool:
        pool.map(_cpu_block_cycle, work[:cores])  # warm the workers
        t0 = time.perf_counter()
        zones = 0
        for _ in range(steps):
            res = pool.map(_cpu_block_cycle, work)
            zones += sum(r[0] for r in res)
        el = time.perf_counter() - t0
    return zones / el, cores, el


def run_reference(a, rank, world):
    if rank != 0:
        return
    n = a.n // a.nb
    sample = max(1, a.cpu_sample_blocks)
    vals = []
    # warm-up steps are untimed samples too
    for i in range(a.warmup + a.steps):
        v, cores, el = cpu_baseline(sample, n)
        if i >= a.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "zone-updates/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"turbulent box {a.n}^3 in {a.nb ** 3} blocks of {n}^3, HLLD+PLM",
                   "sample": f"{sample} blocks of {n}^3 (+{GHOST} ghosts), one cycle per step"},
        "cpu_baseline": {"value": value, "unit": "zone-updates/s", "cores": cores,
                         "kind": "port",
                         "sample": f"{sample} blocks of {n}^3, 1 cycle, CPU oracle restating the reference, one block per process"},
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


def _traffic(kernel_key):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/ncu_traffic.json), scaled to this workload."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            t = json.load(f)
        return t.get(kernel_key)
    except (OSError, ValueError):
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
    import numpy as np
    from mhdvlct import capi
    n_blk = len(blocks)
    n = blocks[0]["density"].shape[0] - 2 * GHOST
    dims = (ctypes.c_int * (3 * n_blk))(*([n] * 3 * n_blk))
    ws = (ctypes.c_double * (3 * n_blk))(*(list(widths) * n_blk))
    h = ctypes.c_void_p()
    L = capi.lib()
    capi.check(L.mhdvlct_batch_create(meth.handle, dims, ws, n_blk, GHOST, dtype,
                                      ctypes.byref(h)), meth.handle, "batch_create")
    from mhdvlct import ic
    nbr = ic.brick_neighbors(nb)
    capi.check(L.mhdvlct_batch_set_neighbors(
        h, (ctypes.c_int * nbr.size)(*nbr.ravel().tolist())), meth.handle, "nbr")
    rt = _cudart()
    npdt = np.float64 if dtype == capi.MHD_DTYPE_F64 else np.float32
    for i, blk in enumerate(blocks):
        v = capi.MhdBlockView()
        capi.check(L.mhdvlct_batch_block_view(h, i, ctypes.byref(v)))
        ptrs = {"density": v.density, "velocity_x": v.velocity[0],
                "velocity_y": v.velocity[1], "velocity_z": v.velocity[2],
                "total_energy": v.total_energy, "bfield_x": v.bfield[0],
                "bfield_y": v.bfield[1], "bfield_z": v.bfield[2],
                "bfieldi_x": v.bfieldi[0], "bfieldi_y": v.bfieldi[1],
                "bfieldi_z": v.bfieldi[2]}
        for k, p in ptrs.items():
            a = np.ascontiguousarray(blk[k], dtype=npdt)
            assert rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0
    return h


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
        tx, ty = (int(v) for v in a.tile.lower().split("x"))
        capi.check(L.mhdvlct_batch_set_tile(h32, tx, ty), meth.handle, "tile")
        tune = {"forced_tile": a.tile}
    elif not a.no_tune:
        buf = ctypes.create_string_buffer(4096)
        capi.check(L.mhdvlct_batch_autotune(h32, 2, buf, 4096, sp), meth.handle,
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
    traffic = _traffic(dom)

    # ------------------------------------------------------ e2e (host data)
    e2e = None
    if not a.no_e2e:
        rt = _cudart()
        dptr, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
        capi.check(L.mhdvlct_batch_state_region(h32, ctypes.byref(dptr),
                                                ctypes.byref(nbytes)))
        host = torch.empty(nbytes.value, dtype=torch.uint8, pin_memory=True)
        assert rt.cudaMemcpy(host.data_ptr(), dptr.value, nbytes.value, 2) == 0
        e2e_steps = max(1, min(a.steps, 5))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(e2e_steps):
            assert rt.cudaMemcpyAsync(dptr.value, host.data_ptr(), nbytes.value, 1, sp) == 0
            capi.check(L.mhdvlct_batch_run(h32, 1, 0, None, sp), meth.handle, "e2e")
            assert rt.cudaMemcpyAsync(host.data_ptr(), dptr.value, nbytes.value, 2, sp) == 0
        e1.record(stream)
        torch.cuda.synchronize()
        e_ms = e0.elapsed_time(e1)
        e2e = {"value": world * zones * e2e_steps / (e_ms / 1e3),
               "unit": "zone-updates/s", "h2d_bytes_per_step": int(nbytes.value),
               "d2h_bytes_per_step": int(nbytes.value), "steps": e2e_steps}
    L.mhdvlct_batch_destroy(h32)

    # ------------------------------------------- FP64: batched and plain path
    fp64 = {}
    if not a.no_fp64:
        h64 = make_batch(meth, blocks, widths, capi.MHD_DTYPE_F64, a.nb)
        k64 = max(1, min(a.steps, 3))
        capi.check(L.mhdvlct_batch_run(h64, 1, 0, None, sp))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        capi.check(L.mhdvlct_batch_run(h64, k64, 0, None, sp))
        e1.record(stream)
        torch.cuda.synchronize()
        fp64["batched_fp64_zone_updates_per_s"] = zones * k64 / (e0.elapsed_time(e1) / 1e3)
        # plain per-block FP64: the Method's timestep and compute called block
        # by block (as Cello drives a Method), refresh between blocks batched
        views = []
        for i in range(len(blocks)):
            v = capi.MhdBlockView()
            capi.check(L.mhdvlct_batch_block_view(h64, i, ctypes.byref(v)))
            views.append(v)
        dt = ctypes.c_double()

        def plain_cycle():
            dts = []
            for v in views:
                capi.check(L.mhdvlct_block_timestep(meth.handle, ctypes.byref(v),
                                                    ctypes.byref(dt), sp), meth.handle)
                dts.append(dt.value)
            dtm = min(dts)
            capi.check(L.mhdvlct_batch_refresh(h64, sp))
            for v in views:
                capi.check(L.mhdvlct_block_step(meth.handle, ctypes.byref(v), dtm, sp),
                           meth.handle)
        plain_cycle()
        torch.cuda.synchronize()
        kp = max(1, min(a.steps, 2))
        t0 = time.perf_counter()
        for _ in range(kp):
            plain_cycle()
        torch.cuda.synchronize()
        fp64["plain_fp64_zone_updates_per_s"] = zones * kp / (time.perf_counter() - t0)
        fp64["fp32_batched_over_plain_fp64"] = value / world / fp64["plain_fp64_zone_updates_per_s"]
        L.mhdvlct_batch_destroy(h64)

    # ----------------------------------------------------------- CPU baseline
    cpu = None
    if rank == 0 and not a.no_cpu:
        sample = max(1, a.cpu_sample_blocks)
        cv, cores, el = cpu_baseline(sample, n)
        cpu = {"value": cv, "unit": "zone-updates/s", "cores": cores, "kind": "port",
               "sample": f"{sample} blocks of {n}^3 (+{GHOST} ghosts), one cycle each, "
                         f"CPU oracle restating the reference, one block per process, "
                         f"{el:.1f} s wall"}

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
                         "cycle_frac": value / world * 5 * N_STATE * 4 / 1e9 / peak},
            "kernels_ms_per_step": {"timestep": k_ts, "refresh": k_ref,
                                    "stage1_half_dt": k_s1, "stage2_full_dt": k_s2,
                                    "cycle": k_cyc},
            "gpu_launches": 6 * a.steps,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        line.update(fp64)
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
