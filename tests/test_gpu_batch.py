"""The batched form: many blocks in one persistent launch per stage.

Checks (FP64, bit-exact against the per-block oracle): one batched step on a
set of uneven blocks; the neighbour-table ghost refresh of a periodic brick
against the oracle's multi-block refresh; a graph-captured multi-cycle run
against the oracle's cycle (timestep on stale ghosts, global min dt,
refresh, step)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from mhdvlct import block as B, capi, ic
from helpers import oracle_block, oracle_params

pytestmark = pytest.mark.gpu

KEYS = ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy",
        "bfield_x", "bfield_y", "bfield_z", "bfieldi_x", "bfieldi_y",
        "bfieldi_z")


class Batch:
    def __init__(self, meth, dims, widths, dtype=capi.MHD_DTYPE_F64, ghost=3,
                 npassive=0, gravity=False):
        n = len(dims)
        d = (ctypes.c_int * (3 * n))(*[int(v) for t in dims for v in t])
        w = (ctypes.c_double * (3 * n))(*[float(v) for t in widths for v in t])
        h = ctypes.c_void_p()
        rc = capi.lib().mhdvlct_batch_create_ex(meth.handle, d, w, n, ghost, dtype,
                                                npassive, int(gravity), ctypes.byref(h))
        capi.check(rc, meth.handle, "batch_create")
        self.h, self.meth, self.n = h, meth, n
        self.dims, self.dtype = dims, dtype

    def view(self, i):
        v = capi.MhdBlockView()
        capi.check(capi.lib().mhdvlct_batch_block_view(self.h, i, ctypes.byref(v)))
        return v

    def tensors(self, i):
        """torch views (sharing memory) of block i's current fields"""
        v = self.view(i)
        nx, ny, nz = v.n[0], v.n[1], v.n[2]
        g = v.ghost[0]
        mx, my, mz = nx + 2 * g, ny + 2 * g, nz + 2 * g
        out = {}
        ptrs = {"density": v.density, "velocity_x": v.velocity[0],
                "velocity_y": v.velocity[1], "velocity_z": v.velocity[2],
                "total_energy": v.total_energy, "bfield_x": v.bfield[0],
                "bfield_y": v.bfield[1], "bfield_z": v.bfield[2],
                "bfieldi_x": v.bfieldi[0], "bfieldi_y": v.bfieldi[1],
                "bfieldi_z": v.bfieldi[2], "pressure": v.pressure,
                "acceleration_x": v.acceleration[0], "acceleration_y": v.acceleration[1],
                "acceleration_z": v.acceleration[2]}
        for k in range(v.npassive):
            ptrs[f"passive_{k}"] = v.passive[k]
        shapes = {"bfieldi_x": (mz, my, mx + 1), "bfieldi_y": (mz, my + 1, mx),
                  "bfieldi_z": (mz + 1, my, mx)}
        for k, p in ptrs.items():
            if p:
                out[k] = (p, shapes.get(k, (mz, my, mx)))
        return out

    def upload(self, i, state):
        dt = np.float64 if self.dtype == capi.MHD_DTYPE_F64 else np.float32
        for k, (p, shp) in self.tensors(i).items():
            if k in state:
                a = np.ascontiguousarray(state[k], dtype=dt)
                assert a.shape == shp, (k, a.shape, shp)
                torch.cuda.synchronize()
                ctypes_cuda_memcpy(p, a, to_device=True)

    def download(self, i):
        dt = np.float64 if self.dtype == capi.MHD_DTYPE_F64 else np.float32
        out = {}
        torch.cuda.synchronize()
        for k, (p, shp) in self.tensors(i).items():
            a = np.empty(shp, dtype=dt)
            ctypes_cuda_memcpy(p, a, to_device=False)
            out[k] = a
        return out

    def __del__(self):
        if getattr(self, "h", None):
            capi.lib().mhdvlct_batch_destroy(self.h)
            self.h = None


_cudart = None


def _load_cudart():
    """The CUDA runtime the library itself loaded."""
    capi.lib()
    path = None
    with open("/proc/self/maps") as f:
        for line in f:
            if "libcudart" in line:
                path = line.split()[-1]
                break
    rt = ctypes.CDLL(path or "libcudart.so")
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    rt.cudaMemset.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t]
    return rt


def ctypes_cuda_memcpy(dev_ptr, host_arr, to_device):
    """cudaMemcpy through the CUDA runtime the library itself loaded."""
    global _cudart
    if _cudart is None:
        _cudart = _load_cudart()
    n = host_arr.nbytes
    if to_device:
        rc = _cudart.cudaMemcpy(dev_ptr, host_arr.ctypes.data, n, 1)
    else:
        rc = _cudart.cudaMemcpy(host_arr.ctypes.data, dev_ptr, n, 2)
    assert rc == 0, rc


def test_batched_step_uneven_blocks_bit_exact():
    meth = B.EnzoMethodMHDVlct()
    sizes = [(8, 8, 8), (6, 10, 7), (12, 8, 8), (8, 8, 8)]
    states, widths = [], []
    for i, n in enumerate(sizes):
        s, w = ic.smooth_block(n, 3, seed=100 + i)
        states.append(s)
        widths.append(w)
    bt = Batch(meth, sizes, widths)
    for i, s in enumerate(states):
        bt.upload(i, s)
    capi.check(capi.lib().mhdvlct_batch_refresh(bt.h, None))
    dts = (ctypes.c_double * len(sizes))(*[0.004, 0.003, 0.002, 0.005])
    capi.check(capi.lib().mhdvlct_batch_step(bt.h, dts, None))
    prm = oracle_params(courant=meth.courant)
    for i, (s, n, w) in enumerate(zip(states, sizes, widths)):
        ob = oracle_block(s, n, 3, w)
        O.fill_ghosts_periodic(ob)
        O.step(prm, ob, dts[i])
        got = bt.download(i)
        for k in KEYS:
            g = 3
            ref = ob.f[ic.ORACLE_NAME[k]]
            if k.startswith("bfieldi"):
                # the batch's current face buffer holds the updated interior
                d = "xyz".index(k[-1])
                sl = [slice(g, g + nn) for nn in reversed(n)]
                sl[2 - d] = slice(g, g + n[d] + 1)
                a, r = got[k][tuple(sl)], ref[tuple(sl)]
            else:
                a, r = got[k], ref
            assert np.array_equal(a, r), (i, k, np.abs(a - r).max())


def test_brick_refresh_matches_oracle():
    meth = B.EnzoMethodMHDVlct()
    blocks, w = ic.turbulent_box(N=16, nb=2, g=3, seed=3)
    for blk in blocks:  # scramble ghosts so the refresh has work to do
        for k, a in blk.items():
            a[:3] = -1.0
    nb = 2
    bt = Batch(meth, [(8, 8, 8)] * 8, [w] * 8)
    nbr = ic.brick_neighbors(nb)
    arr = (ctypes.c_int * nbr.size)(*nbr.ravel().tolist())
    capi.check(capi.lib().mhdvlct_batch_set_neighbors(bt.h, arr))
    for i, s in enumerate(blocks):
        bt.upload(i, s)
    capi.check(capi.lib().mhdvlct_batch_refresh(bt.h, None))
    obs = [oracle_block(s, 8, 3, w) for s in blocks]
    O.fill_ghosts_brick(obs, nb, nb, nb)
    for i in range(8):
        got = bt.download(i)
        for k in KEYS:
            assert np.array_equal(got[k], obs[i].f[ic.ORACLE_NAME[k]]), (i, k)


def test_graph_run_matches_oracle_cycles():
    meth = B.EnzoMethodMHDVlct()
    nb, N = 2, 16
    blocks, w = ic.turbulent_box(N=N, nb=nb, g=3, seed=9, mach=1.0)
    bt = Batch(meth, [(8, 8, 8)] * 8, [w] * 8)
    nbr = ic.brick_neighbors(nb)
    capi.check(capi.lib().mhdvlct_batch_set_neighbors(
        bt.h, (ctypes.c_int * nbr.size)(*nbr.ravel().tolist())))
    for i, s in enumerate(blocks):
        bt.upload(i, s)
    ncyc = 3
    t = ctypes.c_double()
    capi.check(capi.lib().mhdvlct_batch_run(bt.h, ncyc, 0, ctypes.byref(t), None))
    prm = oracle_params(courant=meth.courant)
    obs = [oracle_block(s, 8, 3, w) for s in blocks]
    tt = 0.0
    for _ in range(ncyc):
        dt = min(O.timestep(prm, ob) for ob in obs)
        O.fill_ghosts_brick(obs, nb, nb, nb)
        for ob in obs:
            O.step(prm, ob, dt)
        tt += dt
    assert t.value == tt
    for i in range(8):
        got = bt.download(i)
        g = 3
        act = (slice(g, g + 8),) * 3
        for k in KEYS[:8]:
            assert np.array_equal(got[k][act], obs[i].f[ic.ORACLE_NAME[k]][act]), (i, k)


def _diag(bt):
    d = (ctypes.c_double * 8)()
    capi.check(capi.lib().mhdvlct_batch_diagnostics(bt.h, d, None))
    return list(d)


@pytest.mark.parametrize("dtype", [capi.MHD_DTYPE_F64, capi.MHD_DTYPE_F32])
def test_diagnostics_totals_and_conservation(dtype):
    """FP64 totals of the active zones match a numpy FP64 sum of the same
    stored values, repeat bit for bit, and stay conserved over periodic
    cycles (mass and momentum to round-off; energy is conserved too since
    the floors are inactive); div B stays at round-off."""
    meth = B.EnzoMethodMHDVlct()
    nb, N = 2, 24
    blocks, w = ic.turbulent_box(N=N, nb=nb, g=3, seed=21, mach=1.5)
    bt = Batch(meth, [(12, 12, 12)] * 8, [w] * 8, dtype=dtype)
    nbr = ic.brick_neighbors(nb)
    capi.check(capi.lib().mhdvlct_batch_set_neighbors(
        bt.h, (ctypes.c_int * nbr.size)(*nbr.ravel().tolist())))
    for i, s in enumerate(blocks):
        bt.upload(i, s)
    d0 = _diag(bt)
    assert _diag(bt) == d0
    g, n = 3, 12
    act = (slice(g, g + n),) * 3
    dv = w[0] * w[1] * w[2]
    ref = np.zeros(5)
    for i in range(8):
        f = {k: a.astype(np.float64)[act] for k, a in bt.download(i).items()
             if not k.startswith("bfieldi")}
        rho = f["density"]
        ref += [rho.sum() * dv, (rho * f["velocity_x"]).sum() * dv,
                (rho * f["velocity_y"]).sum() * dv, (rho * f["velocity_z"]).sum() * dv,
                (rho * f["total_energy"]).sum() * dv]
    np.testing.assert_allclose(d0[:5], ref, rtol=1e-12, atol=1e-14)
    capi.check(capi.lib().mhdvlct_batch_run(bt.h, 3, 0, None, None))
    d1 = _diag(bt)
    tol = 1e-13 if dtype == capi.MHD_DTYPE_F64 else 2e-6
    assert abs(d1[0] - d0[0]) <= tol * abs(d0[0])
    assert abs(d1[4] - d0[4]) <= tol * abs(d0[4])
    scale = d0[0] * 3.0  # momentum scale: mass x rms speed
    for k in (1, 2, 3):
        assert abs(d1[k] - d0[k]) <= tol * scale
    bmax = d1[7]
    divb_tol = 1e-12 if dtype == capi.MHD_DTYPE_F64 else 1e-5
    assert d1[6] * w[0] / bmax <= divb_tol


def test_state_segments_cover_the_current_state():
    """mhdvlct_batch_state_segments: the current state (every cell field and
    the current face-B buffer of every block), one segment after an even
    number of cycles and two after an odd one; every field a block view
    points at lies inside them."""
    meth = B.EnzoMethodMHDVlct()
    sizes = [(8, 8, 8), (6, 10, 7)]
    states, widths = [], []
    for i, n in enumerate(sizes):
        s, w = ic.smooth_block(n, 3, seed=300 + i)
        states.append(s)
        widths.append(w)
    bt = Batch(meth, sizes, widths)
    for i, s in enumerate(states):
        bt.upload(i, s)
    segp = (ctypes.c_void_p * 2)()
    segb = (ctypes.c_size_t * 2)()
    nseg = ctypes.c_int()
    for cycles, expect in ((0, 1), (1, 2), (1, 1)):
        if cycles:
            capi.check(capi.lib().mhdvlct_batch_run(bt.h, cycles, 0, None, None))
        capi.check(capi.lib().mhdvlct_batch_state_segments(bt.h, segp, segb, 2,
                                                           ctypes.byref(nseg)))
        assert nseg.value == expect
        segs = [(segp[i], segb[i]) for i in range(nseg.value)]
        want, narr = 0, 0
        for i, n in enumerate(sizes):
            for k, (p, shp) in bt.tensors(i).items():
                if k == "pressure":
                    continue
                nbytes = int(np.prod(shp)) * 8
                want += nbytes
                narr += 1
                assert any(a <= p and p + nbytes <= a + b for a, b in segs), (i, k)
        # every array is padded to a 256-byte boundary
        assert want <= sum(b for _, b in segs) < want + narr * 256


def test_zchunked_default_tiles_bit_exact():
    """One large block alone: the default work decomposition cuts its columns
    into z-chunks (too few column tiles to fill the GPU); the FP64 result is
    still the oracle's bit for bit, after two cycles."""
    meth = B.EnzoMethodMHDVlct()
    n = (26, 20, 40)
    s, w = ic.smooth_block(n, 3, seed=404)
    bt = Batch(meth, [n], [w])
    bt.upload(0, s)
    capi.check(capi.lib().mhdvlct_batch_run(bt.h, 2, 0, None, None))
    ob = oracle_block(s, n, 3, w)
    prm = oracle_params(courant=meth.courant)
    for _ in range(2):
        dt = O.timestep(prm, ob)
        O.fill_ghosts_periodic(ob)
        O.step(prm, ob, dt)
    got = bt.download(0)
    g = 3
    act = (slice(g, g + n[2]), slice(g, g + n[1]), slice(g, g + n[0]))
    for k in KEYS[:8]:
        assert np.array_equal(got[k][act], ob.f[ic.ORACLE_NAME[k]][act]), k


@pytest.mark.parametrize("ngroups,extras", [(1, False), (3, False), (8, False),
                                            (3, True)])
def test_run_host_matches_device_run(ngroups, extras):
    """mhdvlct_batch_run_host (state in pinned host memory, copies pipelined
    with the full-dt stage by block groups) gives the same state, bit for
    bit, as the device-resident graph run of the same cycles; with extras,
    the blocks also carry the acceleration fields and two passive scalars,
    so the per-group full-dt launches must add the gravity source and
    advect the scalars exactly as the whole-batch launch does."""
    meth = B.EnzoMethodMHDVlct()
    nb, N, g, n = 2, 24, 3, 12
    blocks, w = ic.turbulent_box(N=N, nb=nb, g=g, seed=5, mach=1.5)
    if extras:
        rng = np.random.default_rng(23)
        m = n + 2 * g
        act = (slice(g, g + n),) * 3
        for s in blocks:
            for k in ("acceleration_x", "acceleration_y", "acceleration_z"):
                s[k] = np.zeros((m, m, m))
                s[k][act] = 0.3 * (rng.random((n, n, n)) - 0.5)
            for k in range(2):
                s[f"passive_{k}"] = s["density"] * (0.2 + 0.6 * rng.random((m, m, m)))
    nbr = ic.brick_neighbors(nb)
    L = capi.lib()
    runs = []
    for _ in range(2):
        bt = Batch(meth, [(n, n, n)] * 8, [w] * 8, dtype=capi.MHD_DTYPE_F32,
                   npassive=2 if extras else 0, gravity=extras)
        capi.check(L.mhdvlct_batch_set_neighbors(
            bt.h, (ctypes.c_int * nbr.size)(*nbr.ravel().tolist())))
        for i, s in enumerate(blocks):
            bt.upload(i, s)
        runs.append(bt)
    dev, hst = runs
    t_dev, t_host = ctypes.c_double(), ctypes.c_double()
    capi.check(L.mhdvlct_batch_run(dev.h, 3, 0, ctypes.byref(t_dev), None), meth.handle, "run")
    # the host buffer: the current state segments back to back
    segp = (ctypes.c_void_p * 2)()
    segb = (ctypes.c_size_t * 2)()
    nseg = ctypes.c_int()
    capi.check(L.mhdvlct_batch_state_segments(hst.h, segp, segb, 2, ctypes.byref(nseg)))
    total = sum(segb[k] for k in range(nseg.value))
    host = torch.empty(total, dtype=torch.uint8, pin_memory=True)
    off = 0
    for k in range(nseg.value):
        ctypes_cuda_memcpy_raw(host.data_ptr() + off, segp[k], segb[k], to_device=False)
        off += segb[k]
    # scramble the device copy: the run must take its input from the host
    for k in range(nseg.value):
        torch.cuda.synchronize()
        _memset(segp[k], segb[k])
    capi.check(L.mhdvlct_batch_run_host(hst.h, host.data_ptr(), total, 3, ngroups,
                                        ctypes.byref(t_host), None), meth.handle, "run_host")
    assert t_host.value == t_dev.value
    torch.cuda.synchronize()
    # the device run's state, in the same layout
    capi.check(L.mhdvlct_batch_state_segments(dev.h, segp, segb, 2, ctypes.byref(nseg)))
    want = torch.empty(total, dtype=torch.uint8, pin_memory=True)
    off = 0
    for k in range(nseg.value):
        ctypes_cuda_memcpy_raw(want.data_ptr() + off, segp[k], segb[k], to_device=False)
        off += segb[k]
    assert torch.equal(host, want)
    if extras:
        # the scalars sit in the state region: the host run advected them
        got = hst.download(0)
        assert not np.array_equal(got["passive_0"], blocks[0]["passive_0"].astype(np.float32))


def ctypes_cuda_memcpy_raw(dst, src, nbytes, to_device):
    global _cudart
    if _cudart is None:
        _cudart = _load_cudart()
    kind = 1 if to_device else 2
    assert _cudart.cudaMemcpy(dst, src, nbytes, kind) == 0


def _memset(ptr, nbytes):
    global _cudart
    if _cudart is None:
        _cudart = _load_cudart()
    assert _cudart.cudaMemset(ptr, 0x7F, nbytes) == 0


@pytest.mark.parametrize("dtype", [capi.MHD_DTYPE_F64, capi.MHD_DTYPE_F32])
def test_graph_run_gravity_passive_matches_oracle_cycles(dtype):
    """Blocks with acceleration fields and two passive scalars: graph-captured
    cycles (timestep, global min dt, refresh of every field, both stages
    with the gravity source on the full-dt one) equal the oracle's cycle
    bit for bit in FP64, the scalars and the refreshed acceleration
    included; FP32 stays within 1e-5 relative L1 of the FP64 oracle."""
    meth = B.EnzoMethodMHDVlct()
    nb, N, g, n = 2, 16, 3, 8
    blocks, w = ic.turbulent_box(N=N, nb=nb, g=g, seed=5, mach=1.0)
    rng = np.random.default_rng(17)
    m = n + 2 * g
    act = (slice(g, g + n),) * 3
    for s in blocks:
        for k in ("acceleration_x", "acceleration_y", "acceleration_z"):
            s[k] = np.zeros((m, m, m))  # ghosts come from the refresh
            s[k][act] = 0.3 * (rng.random((n, n, n)) - 0.5)
        for k in range(2):
            s[f"passive_{k}"] = s["density"] * (0.2 + 0.6 * rng.random((m, m, m)))
    bt = Batch(meth, [(n,) * 3] * 8, [w] * 8, dtype=dtype, npassive=2, gravity=True)
    nbr = ic.brick_neighbors(nb)
    capi.check(capi.lib().mhdvlct_batch_set_neighbors(
        bt.h, (ctypes.c_int * nbr.size)(*nbr.ravel().tolist())))
    for i, s in enumerate(blocks):
        bt.upload(i, s)
    oname = dict(ic.ORACLE_NAME, acceleration_x="ax", acceleration_y="ay",
                 acceleration_z="az", passive_0="pass0", passive_1="pass1")
    obs = []
    for s in blocks:
        ob = O.Block(n, g, w, mhd=True, gravity=True, npassive=2)
        for k, v in s.items():
            if oname[k] in ob.f:
                ob.f[oname[k]][...] = v
        obs.append(ob)
    ncyc = 3
    t = ctypes.c_double()
    capi.check(capi.lib().mhdvlct_batch_run(bt.h, ncyc, 0, ctypes.byref(t), None))
    prm = oracle_params(courant=meth.courant)
    tt = 0.0
    for _ in range(ncyc):
        dt = min(O.timestep(prm, ob) for ob in obs)
        O.fill_ghosts_brick(obs, nb, nb, nb)
        for ob in obs:
            O.step(prm, ob, dt)
        tt += dt
    if dtype == capi.MHD_DTYPE_F32:
        assert abs(t.value - tt) <= 1e-5 * tt
        for i in range(8):
            got = bt.download(i)
            for k in KEYS[:8] + ("passive_0", "passive_1"):
                ref = obs[i].f[oname[k]][act]
                err = np.abs(got[k][act].astype(np.float64) - ref).sum() / np.abs(ref).sum()
                assert err <= 1e-5, (i, k, err)
        return
    assert t.value == tt
    for i in range(8):
        got = bt.download(i)
        assert set(got) >= {"passive_0", "passive_1", "acceleration_z"}
        for k in KEYS[:8] + ("passive_0", "passive_1"):
            assert np.array_equal(got[k][act], obs[i].f[oname[k]][act]), (i, k)
        for k in ("acceleration_x", "acceleration_y", "acceleration_z"):
            assert np.array_equal(got[k], obs[i].f[oname[k]]), (i, k)
        # the source and the scalars took effect
        assert not np.array_equal(got["passive_0"][act], blocks[i]["passive_0"][act])


def test_batch_create_ex_rejects_bad_options():
    meth = B.EnzoMethodMHDVlct()
    d = (ctypes.c_int * 3)(8, 8, 8)
    w = (ctypes.c_double * 3)(0.1, 0.1, 0.1)
    h = ctypes.c_void_p()
    for npass, grav in ((5, 0), (-1, 0), (0, 2)):
        rc = capi.lib().mhdvlct_batch_create_ex(meth.handle, d, w, 1, 3,
                                                capi.MHD_DTYPE_F64, npass, grav,
                                                ctypes.byref(h))
        assert rc == capi.MHD_ERR_INVALID and not h.value
