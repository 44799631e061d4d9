"""Set-ups of the reference's own VL+CT regression problems (input/vlct/*),
shared by the oracle (CPU) and CUDA (GPU) known-answer tests.

Each problem is rebuilt from its deck: the initial condition (restated from
the reference's initializer), Cello's boundary conditions (periodic, outflow,
inflow), the cycle (timestep on the current ghosts, dt times the global
Courant factor clipped to the stop time, refresh, step; the last timestep
runs once more after the final step, as Cello's does before its output) and
the published error measure (tools/l1_error_norm.py).  Arrays are numpy
(oracle blocks) or torch (device blocks): every helper below works on both.
"""
from __future__ import annotations

import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GAMMA = 1.6666666666666667
CELL = ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy",
        "internal_energy", "bfield_x", "bfield_y", "bfield_z", "pressure")
FACE = ("bfieldi_x", "bfieldi_y", "bfieldi_z")


# ------------------------------------------------------------ boundaries
def _axis_slices(a, ax, idx):
    """Index tuple selecting index `idx` (int or slice) along spatial axis ax
    (0 = x, the last array axis)."""
    sl = [slice(None)] * 3
    sl[2 - ax] = idx
    return tuple(sl)


def outflow(fields, ax, g, side=None):
    """Cello's outflow boundary along spatial axis ax (EnzoBoundary::
    enforce_outflow_precision_, src/Enzo/enzo-core/EnzoBoundary.cpp:356-462):
    every ghost layer takes the outermost active value (for a field centred
    on faces along ax, the block's boundary face)."""
    for k, a in fields.items():
        face = k in FACE and "xyz".index(k[-1]) == ax
        m = a.shape[2 - ax]
        n = m - 2 * g - (1 if face else 0)
        if side in (None, 0):
            for ig in range(g):
                a[_axis_slices(a, ax, g - ig - 1)] = a[_axis_slices(a, ax, g)]
        if side in (None, 1):
            hi = n + g - 1 + (1 if face else 0)
            for ig in range(g):
                a[_axis_slices(a, ax, hi + ig + 1)] = a[_axis_slices(a, ax, hi)]


def inflow(fields, ax, g, values):
    """Cello's inflow (fixed value) boundary on the lower face of axis ax:
    every ghost layer of the named fields takes the given value."""
    for k, v in values.items():
        if k in fields:
            a = fields[k]
            a[_axis_slices(a, ax, slice(0, g))] = v


# ------------------------------------------------------------ shock tubes
SHOCK_L = {"rj2a": dict(density=1.08, pressure=0.95, v=(1.2, 0.01, 0.5),
                        b=(1.0155412503859613, 0.5641895835477563)),
           "sod": dict(density=1.0, pressure=1.0, v=(0.0, 0.0, 0.0), b=(0.0, 0.0))}
SHOCK_R = {"rj2a": dict(density=1.0, pressure=1.0, v=(0.0, 0.0, 0.0),
                        b=(1.1283791670955126, 0.5641895835477563)),
           "sod": dict(density=0.125, pressure=0.1, v=(0.0, 0.0, 0.0), b=(0.0, 0.0))}
SHOCK_B0 = {"rj2a": 0.5641895835477563, "sod": 0.0}


def shock_tube(setup, axis, n, g, widths, gamma, axis_velocity=0.0, de=False):
    """EnzoInitialShockTube::enforce_block (src/Enzo/initial/
    EnzoInitialShockTube.cpp): left and right states split at 0.5 along the
    aligned axis (first cell whose centre is >= 0.5 is right), the aligned
    face B uniform, the other two components per side along the permuted
    axes (j = axis + 1, k = axis + 2), specific energies from the state, then
    the centred B as the mean of the faces.  Returns numpy arrays."""
    m = [x + 2 * g for x in n]
    shp = (m[2], m[1], m[0])
    i_ax, j_ax, k_ax = axis, (axis + 1) % 3, (axis + 2) % 3
    di = widths[axis]
    shock = int(math.ceil((0.5 - 0.0) / di - 0.5 + g))
    shock = min(max(shock, 0), m[axis])
    out = {k: np.zeros(shp) for k in ("density", "velocity_x", "velocity_y", "velocity_z",
                                      "total_energy", "pressure")}
    if de:
        out["internal_energy"] = np.zeros(shp)
    fshape = {0: (m[2], m[1], m[0] + 1), 1: (m[2], m[1] + 1, m[0]), 2: (m[2] + 1, m[1], m[0])}
    faces = {d: np.zeros(fshape[d]) for d in range(3)}
    vel = ("velocity_x", "velocity_y", "velocity_z")
    b0 = SHOCK_B0[setup]
    for side, st, lo, hi in ((0, SHOCK_L[setup], 0, shock), (1, SHOCK_R[setup], shock, m[axis])):
        if lo >= hi:
            continue
        v0 = st["v"][0] + axis_velocity
        v1, v2 = st["v"][1], st["v"][2]
        sel = _axis_slices(out["density"], axis, slice(lo, hi))
        out["density"][sel] = st["density"]
        out[vel[i_ax]][sel] = v0
        out[vel[j_ax]][sel] = v1
        out[vel[k_ax]][sel] = v2
        faces[j_ax][_axis_slices(faces[j_ax], axis, slice(lo, hi))] = st["b"][0]
        faces[k_ax][_axis_slices(faces[k_ax], axis, slice(lo, hi))] = st["b"][1]
        eint = st["pressure"] / ((gamma - 1.) * st["density"])
        if de:
            out["internal_energy"][sel] = eint
        v2s = (v0 * v0 + v1 * v1 + v2 * v2)
        b2 = (b0 * b0 + st["b"][0] * st["b"][0] + st["b"][1] * st["b"][1])
        out["total_energy"][sel] = (eint + 0.5 * (v2s + b2 / st["density"]))
    faces[i_ax][...] = b0
    out["bfieldi_x"], out["bfieldi_y"], out["bfieldi_z"] = faces[0], faces[1], faces[2]
    out["bfield_x"] = 0.5 * (faces[0][:, :, :-1] + faces[0][:, :, 1:])
    out["bfield_y"] = 0.5 * (faces[1][:, :-1, :] + faces[1][:, 1:, :])
    out["bfield_z"] = 0.5 * (faces[2][:-1, :, :] + faces[2][1:, :, :])
    return out


def load_table(name):
    """A 1D solution table of the reference (tests/golden/<name>.npz)."""
    t = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return {str(c): np.asarray(t[str(c)]) for c in t["columns"]}


def table_l1(fields, table, axis, g, n, widths, gamma, names, offset=0.0,
             bkg_velocity=0.0, pressure=None):
    """compare_to_1D_reference of tools/l1_error_norm.py: the run's cells
    along the aligned axis inside the table's span (shifted by `offset`),
    against the table broadcast over the transverse axes; the table's vector
    components are those of the aligned frame (x -> axis, y -> axis + 1,
    z -> axis + 2), missing components are zero and `bkg_velocity` is added
    along the axis.  Per field sum |run - table| / cells, then the root of
    the sum of squares.  `pressure`: the run's pressure array (derived from
    its state)."""
    pos = table["x"] + offset
    dx = pos[1] - pos[0]
    lo_edge, hi_edge = pos[0] - 0.5 * dx, pos[-1] + 0.5 * dx
    centres = (np.arange(n[axis]) + 0.5) * widths[axis]
    sel = np.flatnonzero((centres > lo_edge) & (centres < hi_edge))
    assert len(sel) == len(pos), (len(sel), len(pos))
    comp = {"velocity": ("velocity_x", "velocity_y", "velocity_z"),
            "bfield": ("bfield_x", "bfield_y", "bfield_z")}
    ref = {}
    for k in names:
        base = k.rsplit("_", 1)[0]
        if base in comp:
            d = "xyz".index(k[-1])
            src = comp[base][(d - axis) % 3]  # the table's component along this axis
            v = table.get(src, np.zeros_like(pos))
            if base == "velocity" and d == axis:
                v = v + bkg_velocity
            ref[k] = v
        else:
            ref[k] = table[k]
    act = [slice(g, g + n[a]) for a in range(3)]
    res = []
    for k in names:
        arr = pressure if k == "pressure" else fields[k]
        arr = np.asarray(arr)[act[2], act[1], act[0]]
        arr = np.take(arr, sel, axis=2 - axis)
        shp = [1, 1, 1]
        shp[2 - axis] = len(pos)
        res.append(np.abs(arr - ref[k].reshape(shp)).sum() / arr.size)
    return float(np.sqrt(np.sum(np.square(res)))), res


def derived_pressure(f, gamma, mhd, de=False):
    """The pressure of a state (EnzoComputePressure: from the total energy,
    or from the internal energy with dual energy)."""
    if de:
        return (gamma - 1.0) * f["density"] * f["internal_energy"]
    ke = 0.5 * (f["velocity_x"] ** 2 + f["velocity_y"] ** 2 + f["velocity_z"] ** 2)
    me = 0.0
    if mhd:
        me = 0.5 * (f["bfield_x"] ** 2 + f["bfield_y"] ** 2 + f["bfield_z"] ** 2)
    return (gamma - 1.0) * (f["density"] * (f["total_energy"] - ke) - me)


# ----------------------------------------------------- passive sound wave
def passive_sound(axis, g=3):
    """input/vlct/passive_advect_sound_wave: a sound wave of amplitude 1e-6
    along one axis of a 16 x 4 x 4 periodic box (length 1 along it, 0.25
    across), B = 0, and a passive scalar `red` of 10% of the density with a
    1e-7 perturbation a quarter wavelength off; every value from the deck's
    expressions at the cell centres (ghosts included)."""
    n = [4, 4, 4]
    n[axis] = 16
    L = [0.25, 0.25, 0.25]
    L[axis] = 1.0
    w = tuple(L[a] / n[a] for a in range(3))
    m = [x + 2 * g for x in n]
    c = (np.arange(m[axis]) - g + 0.5) * w[axis]
    s = np.sin(2.0 * np.pi * c)
    s4 = np.sin(2.0 * np.pi * (c - 0.25))
    shp = [1, 1, 1]
    shp[2 - axis] = m[axis]
    full = (m[2], m[1], m[0])

    def bc(v):
        return np.broadcast_to(np.asarray(v).reshape(shp), full).copy()
    vel = ("velocity_x", "velocity_y", "velocity_z")
    out = {"density": bc(1.0 + 1.e-6 * s),
           "total_energy": bc(1.5 * (0.6 + 1.e-6 * s) / (1.0 + 1.e-6 * s)),
           "red": bc((0.1 + 1.e-7 * s4) * (1.0 + 1.e-6 * s)),
           "pressure": np.zeros(full)}
    for d in range(3):
        out[vel[d]] = bc(-1.e-6 * s) if d == axis else np.zeros(full)
        out["bfield_" + "xyz"[d]] = np.zeros(full)
    out["bfieldi_x"] = np.zeros((m[2], m[1], m[0] + 1))
    out["bfieldi_y"] = np.zeros((m[2], m[1] + 1, m[0]))
    out["bfieldi_z"] = np.zeros((m[2] + 1, m[1], m[0]))
    return out, tuple(n), w


def sim_l1(a, b, names, g, n, norm=None):
    """norm_L1_error of two runs over the active zone: per field
    sum |a - b| / (norm or the cell count), root of the sum of squares."""
    act = (slice(g, g + n[2]), slice(g, g + n[1]), slice(g, g + n[0]))
    res = []
    for k in names:
        x, y = np.asarray(a[k])[act], np.asarray(b[k])[act]
        res.append(np.abs(x - y).sum() / (norm or x.size))
    return float(np.sqrt(np.sum(np.square(res))))


# ------------------------------------------------------------------ cloud
CLOUD = dict(radius=1.0, density=1.610075932356949e+01, wind_density=8.944866290871940e-02,
             wind_velocity=1.341500614584355e+01, wind_etot=1.619661509037183e+02,
             wind_eint=7.198495595720811e+01)


def cloud(n=32, g=3, subsample_n=2, mhd=False):
    """EnzoInitialCloud::enforce_block (src/Enzo/initial/EnzoInitialCloud.cpp)
    for input/vlct/dual_energy_cloud: a uniform cloud of radius 1 at the
    origin of [-2, 2]^3 in a wind along x, cells cut by the sphere sampled on
    a 4^3 sub-grid (volume-weighted density, mass-weighted velocity),
    internal energy from the wind's, no perturbation; B = 0 with MHD."""
    h = 4.0 / n
    m = n + 2 * g
    faces = -2.0 + (np.arange(m + 1) - g) * h
    ns = 2 ** subsample_n
    # prep_subcell_offsets_: the fraction accumulates, then scales the width
    cur = 1.0 / 2 ** (subsample_n + 1)
    offs = [cur * h]
    for _ in range(1, ns):
        cur += 1.0 / 2 ** subsample_n
        offs.append(cur * h)
    r2 = CLOUD["radius"] ** 2

    def inside(x, y, z):
        return (x * x + y * y + z * z) <= r2
    frac = np.zeros((m, m, m))
    for iz in range(m):
        for iy in range(m):
            for ix in range(m):
                lo = (faces[ix], faces[iy], faces[iz])
                hi = (faces[ix + 1], faces[iy + 1], faces[iz + 1])
                near, far = [], []
                for a in range(3):
                    if 0.0 <= lo[a]:
                        near.append(lo[a]); far.append(hi[a])
                    elif 0.0 >= hi[a]:
                        near.append(hi[a]); far.append(lo[a])
                    else:
                        near.append(0.0)
                        far.append(lo[a] if (0.0 - lo[a]) > (hi[a] - 0.0) else hi[a])
                if inside(*far):
                    frac[iz, iy, ix] = 1.0
                elif not inside(*near):
                    frac[iz, iy, ix] = 0.0
                else:
                    cnt = 0
                    for oz in offs:
                        for oy in offs:
                            for ox in offs:
                                cnt += inside(lo[0] + ox, lo[1] + oy, lo[2] + oz)
                    frac[iz, iy, ix] = cnt / float(ns ** 3)
    c = CLOUD
    eint_density = c["wind_eint"] * c["wind_density"]
    rho = frac * c["density"] * 1.0 + (1.0 - frac) * c["wind_density"]
    ratio = c["wind_density"] / rho
    vx = ((1.0 - frac) * ratio) * c["wind_velocity"]
    etot = np.where(frac == 0, c["wind_etot"],
                    (eint_density + 0.0) / rho + 0.5 * vx * vx)
    zeros = np.zeros((m, m, m))
    out = {"density": rho, "velocity_x": vx, "velocity_y": zeros.copy(),
           "velocity_z": zeros.copy(), "total_energy": etot,
           "internal_energy": c["wind_eint"] * ratio, "pressure": zeros.copy()}
    if mhd:
        for d in "xyz":
            out["bfield_" + d] = zeros.copy()
        out["bfieldi_x"] = np.zeros((m, m, m + 1))
        out["bfieldi_y"] = np.zeros((m, m + 1, m))
        out["bfieldi_z"] = np.zeros((m + 1, m, m))
    return out, (n, n, n), (h, h, h)


CLOUD_INFLOW = {"density": CLOUD["wind_density"], "velocity_x": CLOUD["wind_velocity"],
                "velocity_y": 0.0, "velocity_z": 0.0, "total_energy": CLOUD["wind_etot"],
                "internal_energy": CLOUD["wind_eint"], "bfield_x": 0.0, "bfield_y": 0.0,
                "bfield_z": 0.0, "bfieldi_x": 0.0, "bfieldi_y": 0.0, "bfieldi_z": 0.0}


def cloud_boundaries(fields, g):
    """The deck's boundary list in order: downwind (outflow, x upper),
    upwind (inflow of the wind, x lower), then outflow on y and z."""
    outflow(fields, 0, g, side=1)
    inflow(fields, 0, g, CLOUD_INFLOW)
    outflow(fields, 1, g)
    outflow(fields, 2, g)


def mirror_asymmetry(density, g, n):
    """check_cloud_asym of input/vlct/run_dual_energy_cloud_test.py on the
    active density (x, y, z indexed): for the slices z = 16 (flipped in y),
    y = 16 (flipped in z) and x = 16 (flipped in y), the sum of
    |(slice - flipped) / slice|."""
    d = np.asarray(density)[g:g + n, g:g + n, g:g + n].transpose(2, 1, 0)  # [x, y, z]
    out = []
    s = d[:, :, 16]
    out.append(np.sum(np.abs((s - d[:, ::-1, 16]) / s)))
    s = d[:, 16, :]
    out.append(np.sum(np.abs((s - d[:, 16, ::-1]) / s)))
    s = d[16, :, :]
    out.append(np.sum(np.abs((s - d[16, ::-1, :]) / s)))
    return out
