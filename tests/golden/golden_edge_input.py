"""Seeded block states that drive the VL+CT step through the branches that
smooth states never reach, for the edge-case golden fixtures
(golden_edge.json).  Like golden_input.py, every value comes from the
generator's uniform numbers and IEEE add / subtract / multiply / divide
only, so the states are the same bits on every platform.

  - degenerate HLLD states: in the lower half of the block (in z) the field
    is a strong uniform B = (2, 0, 0) with perturbations of 1e-9 in rho, p
    and v, so at the x-faces rho_L (S_L - u_L)(S_L - S_M) - B_x^2 is at
    round-off and the single-star states take the B_t = 0 branch
    (EnzoRiemannHLLD.hpp:203, :234); there and at every x-face of the upper
    half, where B_x = 0 exactly (B is the curl of an x-directed vector
    potential), 0.5 B_x^2 < 1e-8 p* selects the double-star states equal to
    the single-star ones (:263);
  - active floors: a near-vacuum pocket (rho = 1e-20, p = 1e-32) under the
    reference decks' floors (density 1e-15, pressure 1e-30,
    input/vlct/dual_energy_cloud/initial_cloud_HD.in:152-156) with
    velocities diverging from it, so the PLM reconstruction floors
    (EnzoReconstructorPLM.hpp:219-243), the density floor of the update
    (EnzoIntegrationQuanUpdate.cpp:205-231) and the energy floor
    (EnzoPhysicsFluidProps.cpp:162-290) all act;
  - the dual-energy switch both ways (eta = 1e-3, EnzoPhysicsFluidProps.cpp:
    162-290): a Mach-10 converging jump in x, and a Mach-50 stream in the
    upper half, where c_s^2 < eta v^2 keeps the advected internal energy.
"""
import numpy as np

from golden_input import GAMMA, WIDTHS

N = (6, 5, 7)
G = 3
DECK_DENSITY_FLOOR = 1e-15
DECK_PRESSURE_FLOOR = 1e-30


def _curl_faces(ax, ay, az, widths):
    dx, dy, dz = widths
    bfx = (az[:, 1:, :] - az[:, :-1, :]) / dy - (ay[1:, :, :] - ay[:-1, :, :]) / dz
    bfy = (ax[1:, :, :] - ax[:-1, :, :]) / dz - (az[:, :, 1:] - az[:, :, :-1]) / dx
    bfz = (ay[:, :, 1:] - ay[:, :, :-1]) / dx - (ax[:, 1:, :] - ax[:, :-1, :]) / dy
    return bfx, bfy, bfz


def _finish(out, rho, vx, vy, vz, p, gamma, bf=None, dual_energy=False):
    e_int = p / ((gamma - 1.0) * rho)
    e_tot = e_int + 0.5 * (vx * vx + vy * vy + vz * vz)
    out.update({"density": rho, "velocity_x": vx, "velocity_y": vy, "velocity_z": vz})
    if bf is not None:
        bfx, bfy, bfz = bf
        bx = 0.5 * (bfx[:, :, :-1] + bfx[:, :, 1:])
        by = 0.5 * (bfy[:, :-1, :] + bfy[:, 1:, :])
        bz = 0.5 * (bfz[:-1, :, :] + bfz[1:, :, :])
        e_tot = e_tot + 0.5 * (bx * bx + by * by + bz * bz) / rho
        out.update({"bfield_x": bx, "bfield_y": by, "bfield_z": bz,
                    "bfieldi_x": bfx, "bfieldi_y": bfy, "bfieldi_z": bfz})
    out["total_energy"] = e_tot
    if dual_energy:
        out["internal_energy"] = e_int
    out["pressure"] = np.zeros(rho.shape)
    return {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in out.items()}


def degenerate_mhd(n, g, seed, widths=WIDTHS, gamma=GAMMA):
    """Strong uniform B_x with tiny perturbations below, B_x = 0 above."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    mx, my, mz = nx + 2 * g, ny + 2 * g, nz + 2 * g
    shp = (mz, my, mx)
    zmid = mz // 2
    lower = (np.arange(mz) < zmid)[:, None, None]
    eps = 1e-9
    rho = np.where(lower, 1.0 + eps * rng.random(shp), 1.0 + 0.4 * rng.random(shp))
    p = np.where(lower, 0.3 + eps * rng.random(shp), 0.6 + 0.2 * rng.random(shp))
    vel = [np.where(lower, eps * (rng.random(shp) - 0.5), 0.5 * (rng.random(shp) - 0.5))
           for _ in range(3)]
    # x-directed potential on x-edges, zero on the edges of the lower half
    # (and its top face), so B_y = B_z = 0 exactly there; B_x = 2 below, 0 above
    ax = 0.02 * (rng.random((mz + 1, my + 1, mx)) - 0.5)
    ax[:zmid + 1] = 0.0
    ay = np.zeros((mz + 1, my, mx + 1))
    az = np.zeros((mz, my + 1, mx + 1))
    bfx, bfy, bfz = _curl_faces(ax, ay, az, widths)
    bfx = bfx + np.where((np.arange(mz) < zmid)[:, None, None], 2.0, 0.0)
    return _finish({}, rho, vel[0], vel[1], vel[2], p, gamma, bf=(bfx, bfy, bfz))


def vacuum_hydro(n, g, seed, dual_energy=False, gamma=GAMMA):
    """Near-vacuum pocket with diverging flow around it."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    mx, my, mz = nx + 2 * g, ny + 2 * g, nz + 2 * g
    shp = (mz, my, mx)
    rho = 1.0 + 0.4 * rng.random(shp)
    p = 0.6 + 0.2 * rng.random(shp)
    cz, cy, cx = mz // 2, my // 2, mx // 2
    pocket = (slice(cz - 1, cz + 2), slice(cy - 1, cy + 1), slice(cx - 1, cx + 2))
    rho[pocket] = 1e-20
    p[pocket] = 1e-32
    # outflow from the pocket's centre: sign of the offset times 1.5 (+ noise)
    z, y, x = np.meshgrid(np.arange(mz), np.arange(my), np.arange(mx), indexing="ij")
    vx = 1.5 * np.sign(x - cx + 0.5) + 0.1 * (rng.random(shp) - 0.5)
    vy = 1.5 * np.sign(y - cy + 0.5) + 0.1 * (rng.random(shp) - 0.5)
    vz = 1.5 * np.sign(z - cz + 0.5) + 0.1 * (rng.random(shp) - 0.5)
    return _finish({}, rho, vx, vy, vz, p, gamma, dual_energy=dual_energy)


def mach_jump(n, g, seed, mhd, widths=WIDTHS, gamma=GAMMA):
    """Dual energy: a Mach-10 converging jump in x, a Mach-50 stream in the
    upper half (c_s ~ 1), and a cold pocket whose pressure sits below the
    deck's floor."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    mx, my, mz = nx + 2 * g, ny + 2 * g, nz + 2 * g
    shp = (mz, my, mx)
    rho = 1.0 + 0.4 * rng.random(shp)
    p = 0.6 + 0.2 * rng.random(shp)
    left = (np.arange(mx) < mx // 2)[None, None, :]
    upper = (np.arange(mz) >= mz // 2)[:, None, None]
    vx = np.where(left, 10.0, -10.0) + 0.2 * (rng.random(shp) - 0.5)
    vx = np.where(upper, 50.0 + 0.2 * (rng.random(shp) - 0.5), vx)
    vy = 0.3 * (rng.random(shp) - 0.5)
    vz = 0.3 * (rng.random(shp) - 0.5)
    p[1:3, 1:3, 1:4] = 1e-32
    bf = None
    if mhd:
        ax = 0.02 * (rng.random((mz + 1, my + 1, mx)) - 0.5)
        ay = 0.02 * (rng.random((mz + 1, my, mx + 1)) - 0.5)
        az = 0.02 * (rng.random((mz, my + 1, mx + 1)) - 0.5)
        bfx, bfy, bfz = _curl_faces(ax, ay, az, widths)
        bf = (bfx + 0.3, bfy + 0.2, bfz + 0.1)
    return _finish({}, rho, vx, vy, vz, p, gamma, bf=bf, dual_energy=True)


# name: (solver, recon, dual energy, eta, density floor, pressure floor, input builder)
EDGE_CASES = [
    ("hlld_degenerate", "hlld", "plm", False, 0.001, 1e-200, 1e-200,
     lambda: degenerate_mhd(N, G, 101)),
    ("hlld_degenerate_nn", "hlld", "nn", False, 0.001, 1e-200, 1e-200,
     lambda: degenerate_mhd(N, G, 102)),
    ("hlle_degenerate", "hlle", "plm", False, 0.001, 1e-200, 1e-200,
     lambda: degenerate_mhd(N, G, 103)),
    ("hllc_vacuum_floors", "hllc", "plm", False, 0.001, DECK_DENSITY_FLOOR,
     DECK_PRESSURE_FLOOR, lambda: vacuum_hydro(N, G, 104)),
    ("hllc_vacuum_floors_de", "hllc", "plm", True, 0.001, DECK_DENSITY_FLOOR,
     DECK_PRESSURE_FLOOR, lambda: vacuum_hydro(N, G, 105, dual_energy=True)),
    ("hllc_mach_jump_de", "hllc", "plm", True, 0.001, DECK_DENSITY_FLOOR,
     DECK_PRESSURE_FLOOR, lambda: mach_jump(N, G, 106, mhd=False)),
    ("hlld_mach_jump_de", "hlld", "plm", True, 0.001, DECK_DENSITY_FLOOR,
     DECK_PRESSURE_FLOOR, lambda: mach_jump(N, G, 107, mhd=True)),
]
