"""Seeded block states for the golden fixtures, built from the generator's
uniform numbers and IEEE add / subtract / multiply / divide only.  No
transcendental function is used, so the states are the same bits on every
platform and numpy build.

B is the discrete curl of a random edge-centred vector potential plus a
uniform background, so its face-centred divergence vanishes to round-off.
"""
import hashlib

import numpy as np

GAMMA = 5.0 / 3.0
WIDTHS = (0.1, 0.125, 0.2)


def golden_input(n, g=3, seed=0, mhd=True, dual_energy=False, gamma=GAMMA,
                 widths=WIDTHS):
    """Cell fields and face B of one ghosted block (Cello layout, z, y, x)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    mx, my, mz = nx + 2 * g, ny + 2 * g, nz + 2 * g
    shp = (mz, my, mx)
    dx, dy, dz = widths
    rho = 1.0 + 0.4 * rng.random(shp)
    vx = 0.5 * (rng.random(shp) - 0.5)
    vy = 0.5 * (rng.random(shp) - 0.5)
    vz = 0.5 * (rng.random(shp) - 0.5)
    p = 0.6 + 0.2 * rng.random(shp)
    out = {"density": rho, "velocity_x": vx, "velocity_y": vy, "velocity_z": vz}
    e_int = p / ((gamma - 1.0) * rho)
    e_tot = e_int + 0.5 * (vx * vx + vy * vy + vz * vz)
    if mhd:
        # A_x on x-edges (mz+1, my+1, mx), A_y on y-edges (mz+1, my, mx+1),
        # A_z on z-edges (mz, my+1, mx+1)
        ax = 0.02 * (rng.random((mz + 1, my + 1, mx)) - 0.5)
        ay = 0.02 * (rng.random((mz + 1, my, mx + 1)) - 0.5)
        az = 0.02 * (rng.random((mz, my + 1, mx + 1)) - 0.5)
        bfx = 0.3 + ((az[:, 1:, :] - az[:, :-1, :]) / dy - (ay[1:, :, :] - ay[:-1, :, :]) / dz)
        bfy = 0.2 + ((ax[1:, :, :] - ax[:-1, :, :]) / dz - (az[:, :, 1:] - az[:, :, :-1]) / dx)
        bfz = 0.1 + ((ay[:, :, 1:] - ay[:, :, :-1]) / dx - (ax[:, 1:, :] - ax[:, :-1, :]) / dy)
        bx = 0.5 * (bfx[:, :, :-1] + bfx[:, :, 1:])
        by = 0.5 * (bfy[:, :-1, :] + bfy[:, 1:, :])
        bz = 0.5 * (bfz[:-1, :, :] + bfz[1:, :, :])
        e_tot = e_tot + 0.5 * (bx * bx + by * by + bz * bz) / rho
        out.update({"bfield_x": bx, "bfield_y": by, "bfield_z": bz,
                    "bfieldi_x": bfx, "bfieldi_y": bfy, "bfieldi_z": bfz})
    out["total_energy"] = e_tot
    if dual_energy:
        out["internal_energy"] = e_int
    out["pressure"] = np.zeros(shp)
    return {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in out.items()}


def digest(a) -> str:
    """SHA-256 of an array's float64 little-endian C-order bytes."""
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


# (name, riemann solver, reconstruction, dual energy, time scheme, theta, seed)
CASES = [
    ("hlld_plm", "hlld", "plm", False, "vl", 1.5, 1),
    ("hlld_nn", "hlld", "nn", False, "vl", 1.5, 2),
    ("hlld_plm_athena", "hlld", "plm_athena", False, "vl", 1.5, 3),
    ("hlle_plm", "hlle", "plm", False, "vl", 1.5, 4),
    ("hllc_plm_hydro", "hllc", "plm", False, "vl", 1.5, 5),
    ("hlld_plm_de", "hlld", "plm", True, "vl", 1.5, 6),
    ("hllc_plm_hydro_de", "hllc", "plm", True, "vl", 1.5, 7),
    ("hllc_nn_euler_hydro", "hllc", "nn", False, "euler", 1.5, 8),
    ("hlld_plm_theta2", "hlld", "plm", False, "vl", 2.0, 9),
]
N = (6, 5, 7)
G = 3
