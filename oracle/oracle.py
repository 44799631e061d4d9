"""TEST INFRASTRUCTURE ONLY: ctypes front-end of the CPU oracle.

The oracle (vlct_oracle.cpp) restates Enzo-E's VL+CT step on the CPU.  Only
tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use this
module, and only as the checker or the timed CPU baseline; the product never
imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_vlct.so")

HLLE, HLLC, HLLD = 0, 1, 2
NN, PLM, PLM_ATHENA = 0, 1, 2

CELL_FIELDS = ("rho", "vx", "vy", "vz", "etot", "eint", "bx", "by", "bz",
               "pressure")
FACE_FIELDS = ("bfx", "bfy", "bfz")


class OracleParams(ctypes.Structure):
    _fields_ = [("riemann", ctypes.c_int), ("recon", ctypes.c_int),
                ("mhd", ctypes.c_int), ("dual_energy", ctypes.c_int),
                ("euler", ctypes.c_int), ("eta", ctypes.c_double),
                ("theta_limiter", ctypes.c_double), ("gamma", ctypes.c_double),
                ("density_floor", ctypes.c_double),
                ("pressure_floor", ctypes.c_double),
                ("courant", ctypes.c_double)]


_P = ctypes.POINTER(ctypes.c_double)


class OracleBlock(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("g", ctypes.c_int), ("dx", ctypes.c_double),
                ("dy", ctypes.c_double), ("dz", ctypes.c_double)] + [
                    (n, _P) for n in ("rho", "vx", "vy", "vz", "etot", "eint",
                                      "bx", "by", "bz", "bfx", "bfy", "bfz",
                                      "pressure", "ax", "ay", "az")] + [
                    ("passive", _P * 4), ("npassive", ctypes.c_int)]


def build(force: bool = False) -> str:
    """Compile the oracle with the flags that keep the reference's FP order."""
    srcs = [os.path.join(HERE, f) for f in ("vlct_oracle.cpp", "refresh_oracle.cpp",
                                            "fluxcorrect_oracle.cpp")]
    if force or not os.path.exists(LIB_PATH) or any(
            os.path.getmtime(LIB_PATH) < os.path.getmtime(s) for s in srcs):
        subprocess.check_call([
            "g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
            "-fno-fast-math", "-o", LIB_PATH] + srcs)
    return LIB_PATH


REF_LIB_PATH = os.path.join(HERE, "_ref", "libvlct_ref.so")

_lib = None
_ref = None


def ref_lib():
    """The reference's own VL+CT sources built by oracle/Makefile (only where
    the Enzo-E tree exists); None when it has not been built."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB_PATH):
        L = ctypes.CDLL(REF_LIB_PATH)
        L.ref_step.argtypes = [ctypes.POINTER(OracleParams),
                               ctypes.POINTER(OracleBlock), ctypes.c_double]
        L.ref_step.restype = ctypes.c_int
        L.ref_timestep.argtypes = [ctypes.POINTER(OracleParams),
                                   ctypes.POINTER(OracleBlock)]
        L.ref_timestep.restype = ctypes.c_double
        L.ref_step_fc.argtypes = [ctypes.POINTER(OracleParams),
                                  ctypes.POINTER(OracleBlock), ctypes.c_double,
                                  ctypes.POINTER(_P), ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_int)]
        L.ref_step_fc.restype = ctypes.c_int
        L.ref_center_bfield.argtypes = [ctypes.c_int] * 3 + [_P] * 6
        L.ref_center_bfield.restype = ctypes.c_int
        _ref = L
    return _ref


REFRESH_REF_PATH = os.path.join(HERE, "_ref", "librefresh_ref.so")
_refresh_ref = None


def refresh_ref_lib():
    """The reference's own Box / ProlongLinear / RestrictLinear built by
    oracle/Makefile (only where the Enzo-E tree exists); None otherwise."""
    global _refresh_ref
    if _refresh_ref is None and os.path.exists(REFRESH_REF_PATH):
        L = ctypes.CDLL(REFRESH_REF_PATH)
        ip = ctypes.POINTER(ctypes.c_int)
        L.ref_refresh_box.argtypes = [ip] * 3 + [ctypes.c_int] + [ip] * 6
        L.ref_refresh_faces.argtypes = [ctypes.c_int] * 2 + [ip] * 2 + [
            ctypes.POINTER(ctypes.c_void_p), ip, ctypes.c_int, ctypes.c_uint]
        L.ref_coarsen_fluxes.argtypes = [ip, ctypes.c_int, ctypes.c_int, ip,
                                         ctypes.c_void_p, ctypes.c_void_p]
        _refresh_ref = L
    return _refresh_ref


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_step.argtypes = [ctypes.POINTER(OracleParams),
                                  ctypes.POINTER(OracleBlock), ctypes.c_double]
        L.oracle_step.restype = ctypes.c_int
        L.oracle_timestep.argtypes = [ctypes.POINTER(OracleParams),
                                      ctypes.POINTER(OracleBlock)]
        L.oracle_timestep.restype = ctypes.c_double
        L.oracle_step_fc.argtypes = [ctypes.POINTER(OracleParams),
                                     ctypes.POINTER(OracleBlock), ctypes.c_double,
                                     ctypes.POINTER(_P), ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_int)]
        L.oracle_step_fc.restype = ctypes.c_int
        L.oracle_fill_ghosts_periodic.argtypes = [ctypes.POINTER(OracleBlock)]
        L.oracle_fill_ghosts_brick.argtypes = [ctypes.POINTER(OracleBlock),
                                               ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int]
        L.oracle_fill_ghosts_table.argtypes = [ctypes.POINTER(OracleBlock),
                                               ctypes.c_int,
                                               ctypes.POINTER(ctypes.c_int)]
        L.oracle_ic_inclined_wave.argtypes = [
            ctypes.POINTER(OracleBlock), ctypes.c_char_p, ctypes.c_double,
            ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
            ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.oracle_evolve_periodic.argtypes = [ctypes.POINTER(OracleParams),
                                             ctypes.POINTER(OracleBlock),
                                             ctypes.c_double, ctypes.c_int]
        L.oracle_evolve_periodic.restype = ctypes.c_int
        ip = ctypes.POINTER(ctypes.c_int)
        L.oracle_refresh_box.argtypes = [ip] * 3 + [ctypes.c_int] + [ip] * 6
        L.oracle_refresh_faces.argtypes = [ctypes.c_int] * 2 + [ip] * 2 + [
            ctypes.POINTER(ctypes.c_void_p), ip, ctypes.c_int, ctypes.c_uint]
        vpp = ctypes.POINTER(ctypes.c_void_p)
        L.oracle_flux_correct.argtypes = [ctypes.c_int] * 2 + [ip] * 2 + [
            vpp, vpp, ip, ctypes.c_int, ctypes.c_uint]
        L.oracle_coarsen_fluxes.argtypes = [ctypes.c_int] * 3 + [
            ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.oracle_coarsen_fluxes.restype = None
        _lib = L
    return _lib


def params(riemann=HLLD, recon=PLM, mhd=True, dual_energy=False, euler=False,
           eta=0.001, theta_limiter=1.5, gamma=5.0 / 3.0, density_floor=1e-200,
           pressure_floor=1e-200, courant=0.3) -> OracleParams:
    return OracleParams(riemann, recon, int(mhd), int(dual_energy), int(euler),
                        eta, theta_limiter, gamma, density_floor,
                        pressure_floor, courant)


class Block:
    """One ghosted block held as float64 numpy arrays in Cello's layout."""

    def __init__(self, n, g=3, widths=(1.0, 1.0, 1.0), mhd=True,
                 dual_energy=False, gravity=False, npassive=0):
        nx, ny, nz = (n, n, n) if np.isscalar(n) else n
        self.n = (nx, ny, nz)
        self.g = g
        self.widths = tuple(float(w) for w in widths)
        mx, my, mz = nx + 2 * g, ny + 2 * g, nz + 2 * g
        self.m = (mx, my, mz)
        self.mhd = mhd
        self.dual_energy = dual_energy
        shp = (mz, my, mx)
        self.f = {}
        for k in ("rho", "vx", "vy", "vz", "etot", "pressure"):
            self.f[k] = np.zeros(shp)
        if dual_energy:
            self.f["eint"] = np.zeros(shp)
        if gravity:
            for k in ("ax", "ay", "az"):
                self.f[k] = np.zeros(shp)
        self.npassive = npassive
        for k in range(npassive):
            self.f[f"pass{k}"] = np.zeros(shp)
        if mhd:
            for k in ("bx", "by", "bz"):
                self.f[k] = np.zeros(shp)
            self.f["bfx"] = np.zeros((mz, my, mx + 1))
            self.f["bfy"] = np.zeros((mz, my + 1, mx))
            self.f["bfz"] = np.zeros((mz + 1, my, mx))

    def copy(self):
        b = Block.__new__(Block)
        b.__dict__.update(self.__dict__)
        b.f = {k: v.copy() for k, v in self.f.items()}
        return b

    def cstruct(self) -> OracleBlock:
        def p(k):
            a = self.f.get(k)
            if a is None:
                return _P()
            assert a.flags.c_contiguous and a.dtype == np.float64
            return a.ctypes.data_as(_P)
        nx, ny, nz = self.n
        dx, dy, dz = self.widths
        ob = OracleBlock(nx, ny, nz, self.g, dx, dy, dz,
                         *[p(k) for k in ("rho", "vx", "vy", "vz", "etot",
                                          "eint", "bx", "by", "bz", "bfx",
                                          "bfy", "bfz", "pressure", "ax",
                                          "ay", "az")])
        npass = getattr(self, "npassive", 0)
        for k in range(npass):
            ob.passive[k] = p(f"pass{k}")
        ob.npassive = npass
        return ob


def step(prm: OracleParams, b: Block, dt: float, ref: bool = False) -> None:
    cs = b.cstruct()
    fn = ref_lib().ref_step if ref else lib().oracle_step
    rc = fn(ctypes.byref(prm), ctypes.byref(cs), dt)
    if rc != 0:
        raise RuntimeError(f"oracle_step failed: {rc}")


FC_QUANTITIES = ("density", "velocity_x", "velocity_y", "velocity_z",
                 "total_energy", "internal_energy",
                 "passive_0", "passive_1", "passive_2", "passive_3")


def step_fc(prm: OracleParams, b: Block, dt: float, quantities=(0, 1, 2, 3, 4),
            ref: bool = False) -> dict:
    """The step with store_fluxes_for_corrections; returns
    {(dim, side, quantity): array} of dt/dx-scaled boundary fluxes
    (EnzoMethodMHDVlct.cpp:250-330)."""
    nx, ny, nz = b.n
    shapes = [(nz, ny), (nz, nx), (ny, nx)]
    nq = len(quantities)
    arrs = {}
    ptrs = (_P * (6 * nq))()
    for dim in range(3):
        for side in range(2):
            for iq, q in enumerate(quantities):
                a = np.zeros(shapes[dim])
                arrs[(dim, side, q)] = a
                ptrs[(dim * 2 + side) * nq + iq] = a.ctypes.data_as(_P)
    qs = (ctypes.c_int * nq)(*quantities)
    cs = b.cstruct()
    fn = ref_lib().ref_step_fc if ref else lib().oracle_step_fc
    rc = fn(ctypes.byref(prm), ctypes.byref(cs), dt, ptrs, nq, qs)
    if rc != 0:
        raise RuntimeError(f"step_fc failed: {rc}")
    return arrs


def timestep(prm: OracleParams, b: Block, ref: bool = False) -> float:
    cs = b.cstruct()
    fn = ref_lib().ref_timestep if ref else lib().oracle_timestep
    return fn(ctypes.byref(prm), ctypes.byref(cs))


def fill_ghosts_periodic(b: Block) -> None:
    cs = b.cstruct()
    lib().oracle_fill_ghosts_periodic(ctypes.byref(cs))


def fill_ghosts_brick(blocks, nbx, nby, nbz) -> None:
    arr = (OracleBlock * len(blocks))(*[b.cstruct() for b in blocks])
    lib().oracle_fill_ghosts_brick(arr, nbx, nby, nbz)


def fill_ghosts_table(blocks, nbr) -> None:
    """Same-level refresh from a 27-neighbour table (nblocks x 27, entry
    (sz+1)*9 + (sy+1)*3 + (sx+1) the source of the ghost region at offset
    (sx, sy, sz)); a block and its neighbours have equal extents."""
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    assert nbr.shape == (len(blocks), 27)
    arr = (OracleBlock * len(blocks))(*[b.cstruct() for b in blocks])
    lib().oracle_fill_ghosts_table(arr, len(blocks),
                                   nbr.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))


def inclined_wave(b: Block, wave: str, alpha=0.7297276562269663,
                  beta=1.1071487177940904, gamma=1.6666666666666667,
                  amplitude=1e-6, lam=1.0, positive_vel=True,
                  lower=(0.0, 0.0, 0.0)) -> None:
    cs = b.cstruct()
    rc = lib().oracle_ic_inclined_wave(ctypes.byref(cs), wave.encode(), alpha,
                                       beta, gamma, amplitude, lam,
                                       int(positive_vel), *lower)
    if rc != 0:
        raise ValueError(f"unknown wave {wave}")


def evolve_periodic(prm: OracleParams, b: Block, stop_time: float,
                    max_cycles: int = 1 << 30, ref: bool = False) -> int:
    """Cello's cycle on one periodic block: timestep on the current ghosts,
    clip to the stop time, refresh the ghosts, step."""
    if not ref:
        cs = b.cstruct()
        return lib().oracle_evolve_periodic(ctypes.byref(prm), ctypes.byref(cs),
                                            stop_time, max_cycles)
    time, cycle = 0.0, 0
    while cycle < max_cycles:
        dt = timestep(prm, b, ref=True)
        dt = min(dt, stop_time - time)
        if not time < stop_time:
            break
        fill_ghosts_periodic(b)
        step(prm, b, dt, ref=True)
        time += dt
        cycle += 1
    return cycle


def pressure_of(b: Block, gamma: float) -> np.ndarray:
    """Derived pressure over the whole block (EnzoComputePressure, no DE)."""
    f = b.f
    ke = 0.5 * (f["vx"] * f["vx"] + f["vy"] * f["vy"] + f["vz"] * f["vz"])
    me = 0.0
    if b.mhd:
        me = 0.5 * (f["bx"] * f["bx"] + f["by"] * f["by"] + f["bz"] * f["bz"])
    return (gamma - 1.0) * (f["rho"] * (f["etot"] - ke) - me)


def l1_error_norm(a: Block, b: Block, fields, gamma: float, res: int) -> float:
    """tools/l1_error_norm.py: sqrt(sum_f (sum |a-b| / res^3)^2) over the
    active zone, with pressure derived from the state."""
    g = a.g
    nx, ny, nz = a.n
    sl = (slice(g, g + nz), slice(g, g + ny), slice(g, g + nx))
    errs = []
    for k in fields:
        if k == "pressure":
            x, y = pressure_of(a, gamma), pressure_of(b, gamma)
        else:
            x, y = a.f[k], b.f[k]
        errs.append(np.sum(np.abs(x[sl] - y[sl])) / float(res ** 3))
    return float(np.sqrt(np.sum(np.square(errs))))


def bfield_from_potential(ax, ay, az, widths, dtype=np.float64):
    """Face-centred and centred B of a ghosted block from an edge-centred
    vector potential (float64 arrays in (z, y, x) order with the shapes
    (mz+1, my+1, mx), (mz+1, my, mx+1), (mz, my+1, mx+1)).

    Restates EnzoInitialBCenter::initialize_bfield_interface and
    bfieldi_helper_ (src/Enzo/initial/EnzoInitialBCenter.cpp:41-127): each
    face component is the curl difference evaluated in double, then cast to
    the field type; the centred B is the mean of the two faces in the field
    type (EnzoBfieldMethodCT::compute_center_bfield,
    EnzoBfieldMethodCT.cpp:702-728)."""
    dx, dy, dz = widths
    mz, my, mx = az.shape[0], ay.shape[1], ax.shape[2]
    # Bx(k, j, i-1/2) = (Az(k, j+1/2) - Az(k, j-1/2))/dy - (Ay(k+1/2, j) - Ay(k-1/2, j))/dz
    bfx = ((az[:, 1:, :] - az[:, :-1, :]) / dy
           - (ay[1:, :, :] - ay[:-1, :, :]) / dz).astype(dtype)
    # By(k, j-1/2, i) = (Ax(k+1/2) - Ax(k-1/2))/dz - (Az(i+1/2) - Az(i-1/2))/dx
    bfy = ((ax[1:, :, :] - ax[:-1, :, :]) / dz
           - (az[:, :, 1:] - az[:, :, :-1]) / dx).astype(dtype)
    # Bz(k-1/2, j, i) = (Ay(i+1/2) - Ay(i-1/2))/dx - (Ax(j+1/2) - Ax(j-1/2))/dy
    bfz = ((ay[:, :, 1:] - ay[:, :, :-1]) / dx
           - (ax[:, 1:, :] - ax[:, :-1, :]) / dy).astype(dtype)
    assert bfx.shape == (mz, my, mx + 1) and bfy.shape == (mz, my + 1, mx)
    assert bfz.shape == (mz + 1, my, mx)
    half = dtype(0.5)
    bx = half * (bfx[:, :, :-1] + bfx[:, :, 1:])
    by = half * (bfy[:, :-1, :] + bfy[:, 1:, :])
    bz = half * (bfz[:-1, :, :] + bfz[1:, :, :])
    return (bfx, bfy, bfz), (bx, by, bz)


# ----------------------------------------------------------- mesh refresh
NFIELD_SLOTS = 20  # the C ABI's MHD_FIELD_* slot order


def _i3(v):
    return (ctypes.c_int * 3)(*[int(x) for x in v])


def refresh_box(n, g, c, level, face, child, ref: bool = False):
    """(send start, send size, receive start, receive size) of one face."""
    L = refresh_ref_lib() if ref else lib()
    out = [(ctypes.c_int * 3)() for _ in range(4)]
    fn = L.ref_refresh_box if ref else L.oracle_refresh_box
    rc = fn(_i3(n), _i3(g), _i3(c), int(level), _i3(face), _i3(child), *out)
    if rc != 0:
        raise RuntimeError("refresh_box failed")
    return tuple(tuple(o) for o in out)


def refresh_faces(blocks, n, g, faces, cons: int, ref: bool = False) -> None:
    """Refresh in place.  blocks: list of dicts slot -> C-contiguous numpy
    array (float64 or float32, all alike); faces: int array of 9 per face."""
    dt = None
    ptrs = (ctypes.c_void_p * (NFIELD_SLOTS * len(blocks)))()
    for i, b in enumerate(blocks):
        for s, a in b.items():
            assert a.flags.c_contiguous
            dt = a.dtype if dt is None else dt
            assert a.dtype == dt
            ptrs[NFIELD_SLOTS * i + s] = a.ctypes.data
    faces = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 9)
    L = refresh_ref_lib() if ref else lib()
    fn = L.ref_refresh_faces if ref else L.oracle_refresh_faces
    rc = fn(0 if dt == np.float64 else 1, len(blocks), _i3(n), _i3(g), ptrs,
            faces.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(faces),
            ctypes.c_uint(cons))
    if rc != 0:
        raise RuntimeError(f"refresh_faces failed: {rc}")


# -------------------------------------------------------- flux correction
FC_FIELDS = ("rho", "vx", "vy", "vz", "etot", "eint")  # MHD_Q_* order


def coarsen_fluxes(fine, ci, co, ref: bool = False, n=None, axis=0, face=0):
    """FaceFluxes::coarsen of one fine face array (outer x inner, inner
    fastest) for a child with transverse child index (ci, co).  The
    reference's version (ref=True, FP64) needs the block extents n, the axis
    and the face, and takes the child index per axis."""
    fine = np.ascontiguousarray(fine)
    out = np.zeros_like(fine)
    if ref:
        c3 = [0, 0, 0]
        a_in = 1 if axis == 0 else 0
        a_out = 1 if axis == 2 else 2
        c3[a_in], c3[a_out] = ci, co
        rc = refresh_ref_lib().ref_coarsen_fluxes(_i3(n), axis, face, _i3(c3),
                                                  fine.ctypes.data, out.ctypes.data)
        if rc != 0:
            raise RuntimeError("ref_coarsen_fluxes failed")
        return out
    no, ni = fine.shape
    lib().oracle_coarsen_fluxes(0 if fine.dtype == np.float64 else 1, ni, no,
                                fine.ctypes.data, ci, co, out.ctypes.data)
    return out


def flux_correct(blocks, fluxes, n, g, faces, cons: int) -> None:
    """Correct in place.  blocks: list of dicts MHD_Q index -> array;
    fluxes: list of dicts (axis, side, q) -> stored flux array (as step_fc
    returns them); faces: int array of 9 per face."""
    nb, nq = len(blocks), len(FC_QUANTITIES)
    fp = (ctypes.c_void_p * (nq * nb))()
    xp = (ctypes.c_void_p * (6 * nq * nb))()
    dt = None
    for i, b in enumerate(blocks):
        for q, a in b.items():
            dt = a.dtype if dt is None else dt
            fp[nq * i + q] = a.ctypes.data
        for (ax, side, q), a in fluxes[i].items():
            assert a.flags.c_contiguous and a.dtype == dt
            xp[6 * nq * i + (ax * 2 + side) * nq + q] = a.ctypes.data
    faces = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 9)
    rc = lib().oracle_flux_correct(0 if dt == np.float64 else 1, nb, _i3(n), _i3(g), fp, xp,
                                   faces.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   len(faces), ctypes.c_uint(cons))
    if rc != 0:
        raise RuntimeError(f"flux_correct failed: {rc}")
