"""Seeded synthetic initial conditions in Cello's block layout (numpy, FP64).

Magnetic fields are always built as the discrete curl of an edge-centred
vector potential, exactly as EnzoInitialBCenter does
(src/Enzo/initial/EnzoInitialBCenter.cpp:43-127), so div B = 0 to round-off;
the cell-centred B is the face average.

  smooth_block   -- a random smooth periodic state on one block (parity tests)
  turbulent_box  -- lognormal density, k^-2 Gaussian velocity at a given rms
                    Mach number, uniform B plus the curl of a k^-3 potential
                    (the 256^3 turbulent-box workload), split into blocks
  sedov_block    -- a Gaussian energy deposit in a uniform medium with a
                    uniform B (the mixed-size AMR block-set workload)
"""
from __future__ import annotations

import numpy as np

GAMMA = 5.0 / 3.0


def _faces_from_potential(Ax, Ay, Az, dx, dy, dz):
    """Face B = curl A.  A_x on (mz+1, my+1, mx) edges, A_y on (mz+1, my,
    mx+1), A_z on (mz, my+1, mx+1); arrays indexed (z, y, x)."""
    bfx = (Az[:, 1:, :] - Az[:, :-1, :]) / dy - (Ay[1:, :, :] - Ay[:-1, :, :]) / dz
    bfy = (Ax[1:, :, :] - Ax[:-1, :, :]) / dz - (Az[:, :, 1:] - Az[:, :, :-1]) / dx
    bfz = (Ay[:, :, 1:] - Ay[:, :, :-1]) / dx - (Ax[:, 1:, :] - Ax[:, :-1, :]) / dy
    return bfx, bfy, bfz


def _centres(bfx, bfy, bfz):
    return (0.5 * (bfx[:, :, :-1] + bfx[:, :, 1:]),
            0.5 * (bfy[:, :-1, :] + bfy[:, 1:, :]),
            0.5 * (bfz[:-1, :, :] + bfz[1:, :, :]))


def _energy(rho, vx, vy, vz, p, bx=None, by=None, bz=None, gamma=GAMMA):
    e = p / ((gamma - 1.0) * rho) + 0.5 * (vx * vx + vy * vy + vz * vz)
    if bx is not None:
        e = e + 0.5 * (bx * bx + by * by + bz * bz) / rho
    return e


def smooth_block(n, g=3, seed=0, mhd=True, dual_energy=False, amp_v=0.5,
                 gamma=GAMMA, nmodes=4, width=1.0):
    """A random, smooth, periodic (over the active zone) state."""
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    rng = np.random.default_rng(seed)
    mx, my, mz = nx + 2 * g, ny + 2 * g, nz + 2 * g
    dx, dy, dz = width / nx, width / ny, width / nz
    xc = (np.arange(mx) - g + 0.5) * dx
    yc = (np.arange(my) - g + 0.5) * dy
    zc = (np.arange(mz) - g + 0.5) * dz
    xf = (np.arange(mx + 1) - g) * dx
    yf = (np.arange(my + 1) - g) * dy
    zf = (np.arange(mz + 1) - g) * dz

    modes = [(rng.integers(-2, 3, size=3), rng.uniform(0, 2 * np.pi),
              rng.normal()) for _ in range(nmodes)]

    def field(x, y, z, scale, rot):
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        out = np.zeros(Z.shape)
        for k, ph, a in modes:
            kk = np.roll(k, rot)
            out += a * np.sin(2 * np.pi * (kk[0] * X / width + kk[1] * Y / width +
                                           kk[2] * Z / width) + ph + rot)
        return scale * out / max(1, nmodes)

    rho = 1.0 + 0.3 * np.tanh(field(xc, yc, zc, 1.0, 0))
    p = 0.6 + 0.2 * np.tanh(field(xc, yc, zc, 1.0, 1))
    vx = field(xc, yc, zc, amp_v, 2)
    vy = field(xc, yc, zc, amp_v, 3)
    vz = field(xc, yc, zc, amp_v, 4)
    out = {"density": rho, "velocity_x": vx, "velocity_y": vy, "velocity_z": vz}
    if mhd:
        b0 = rng.normal(size=3) * 0.5
        # uniform part: A = (b0_y z, b0_z x, b0_x y) has curl (b0_x, b0_y, b0_z)
        Ax = field(xc, yf, zf, 0.05, 5) + b0[1] * zf[:, None, None]
        Ay = field(xf, yc, zf, 0.05, 6) + b0[2] * xf[None, None, :]
        Az = field(xf, yf, zc, 0.05, 7) + b0[0] * yf[None, :, None]
        bfx, bfy, bfz = _faces_from_potential(Ax, Ay, Az, dx, dy, dz)
        bx, by, bz = _centres(bfx, bfy, bfz)
        out.update(bfieldi_x=bfx, bfieldi_y=bfy, bfieldi_z=bfz, bfield_x=bx,
                   bfield_y=by, bfield_z=bz)
        out["total_energy"] = _energy(rho, vx, vy, vz, p, bx, by, bz, gamma)
    else:
        out["total_energy"] = _energy(rho, vx, vy, vz, p, gamma=gamma)
    if dual_energy:
        out["internal_energy"] = p / ((gamma - 1.0) * rho)
    out["pressure"] = np.zeros_like(rho)
    return out, (dx, dy, dz)


# --------------------------------------------------------------- turbulence
def _grf(shape, kmin, kmax, slope, rng):
    """Real Gaussian random field on a periodic grid with power P(k) ~ k^slope
    on integer shells kmin..kmax, unit variance."""
    nz, ny, nx = shape
    kz = np.fft.fftfreq(nz) * nz
    ky = np.fft.fftfreq(ny) * ny
    kx = np.fft.rfftfreq(nx) * nx
    K = np.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 +
                kx[None, None, :] ** 2)
    amp = np.zeros_like(K)
    sel = (K >= kmin - 0.5) & (K < kmax + 0.5) & (K > 0)
    # P(k) ~ k^slope in 3D shells: per-mode amplitude^2 ~ k^(slope-2)
    amp[sel] = K[sel] ** ((slope - 2.0) / 2.0)
    ph = rng.normal(size=K.shape) + 1j * rng.normal(size=K.shape)
    f = np.fft.irfftn(amp * ph, s=shape, axes=(0, 1, 2))
    f -= f.mean()
    s = f.std()
    return f / s if s > 0 else f


def turbulent_box(N=256, nb=8, g=3, seed=0, mach=2.0, sigma_ln=0.5, b0=0.2,
                  beta=1.0, p_over_rho=0.1, gamma=GAMMA, dtype=np.float64,
                  dual_energy=False, sink=None):
    """The turbulent periodic box: N^3 cells split into nb^3 blocks of
    (N/nb)^3 active cells with g ghost layers (filled periodically).
    Returns (blocks, widths) with blocks[(kz*nb + ky)*nb + kx] a dict of
    arrays in Cello layout (with internal_energy when dual_energy).  With
    `sink`, each block is passed to sink(index, block) instead of being kept
    (blocks is then empty)."""
    rng = np.random.default_rng(seed)
    shape = (N, N, N)
    G = _grf(shape, 1, 8, -2.0, rng)
    rho = np.exp(sigma_ln * G - 0.5 * sigma_ln ** 2)
    p = p_over_rho * rho
    cs = np.sqrt(gamma * p_over_rho)
    vel = [_grf(shape, 1, 8, -2.0, rng) for _ in range(3)]
    vrms = np.sqrt(np.mean(vel[0] ** 2 + vel[1] ** 2 + vel[2] ** 2))
    vel = [v * (mach * cs / vrms) for v in vel]
    # vector potential on edges; B = (b0,0,0) + curl A with B_rms ~ sqrt(2 p / beta)
    A = [_grf(shape, 2, 6, -3.0, rng) for _ in range(3)]
    dx = 1.0 / N
    # periodic discrete curl on the global grid.  A_x[k,j,i] sits at
    # (x_i, y_{j-1/2}, z_{k-1/2}), A_y at (x_{i-1/2}, y_j, z_{k-1/2}), A_z at
    # (x_{i-1/2}, y_{j-1/2}, z_k); then bfx[k,j,i] is B_x on the low x-face of
    # cell (i,j,k), which is Cello's face index convention.
    Ax, Ay, Az = A
    bfx = (np.roll(Az, -1, 1) - Az) / dx - (np.roll(Ay, -1, 0) - Ay) / dx
    bfy = (np.roll(Ax, -1, 0) - Ax) / dx - (np.roll(Az, -1, 2) - Az) / dx
    bfz = (np.roll(Ay, -1, 2) - Ay) / dx - (np.roll(Ax, -1, 1) - Ax) / dx
    brms = np.sqrt(np.mean(bfx ** 2 + bfy ** 2 + bfz ** 2))
    target = np.sqrt(max(2.0 * p_over_rho / beta - b0 * b0, 0.0))
    s = target / brms if brms > 0 else 0.0
    bfx, bfy, bfz = bfx * s + b0, bfy * s, bfz * s
    n = N // nb
    blocks = []
    for kz in range(nb):
        for ky in range(nb):
            for kx in range(nb):
                zi = (np.arange(n + 2 * g) + kz * n - g) % N
                yi = (np.arange(n + 2 * g) + ky * n - g) % N
                xi = (np.arange(n + 2 * g) + kx * n - g) % N
                xf = (np.arange(n + 2 * g + 1) + kx * n - g) % N
                yf = (np.arange(n + 2 * g + 1) + ky * n - g) % N
                zf = (np.arange(n + 2 * g + 1) + kz * n - g) % N
                cell = np.ix_(zi, yi, xi)
                r = rho[cell]
                vx, vy, vz = (v[cell] for v in vel)
                fx = bfx[np.ix_(zi, yi, xf)]
                fy = bfy[np.ix_(zi, yf, xi)]
                fz = bfz[np.ix_(zf, yi, xi)]
                bx, by, bz = _centres(fx, fy, fz)
                blk = {"density": r, "velocity_x": vx, "velocity_y": vy,
                       "velocity_z": vz, "bfieldi_x": fx, "bfieldi_y": fy,
                       "bfieldi_z": fz, "bfield_x": bx, "bfield_y": by,
                       "bfield_z": bz,
                       "total_energy": _energy(r, vx, vy, vz, p[cell], bx, by,
                                               bz, gamma),
                       "pressure": np.zeros_like(r)}
                if dual_energy:
                    blk["internal_energy"] = p[cell] / ((gamma - 1.0) * r)
                blk = {k: np.ascontiguousarray(v, dtype=dtype) for k, v in blk.items()}
                if sink is not None:
                    sink((kz * nb + ky) * nb + kx, blk)
                else:
                    blocks.append(blk)
    return blocks, (dx, dx, dx)


def brick_neighbors(nb):
    """27-neighbour table of a periodic nb^3 brick of blocks."""
    out = np.zeros((nb ** 3, 27), dtype=np.int32)
    for kz in range(nb):
        for ky in range(nb):
            for kx in range(nb):
                b = (kz * nb + ky) * nb + kx
                for sz in (-1, 0, 1):
                    for sy in (-1, 0, 1):
                        for sx in (-1, 0, 1):
                            nbk = (((kz + sz) % nb) * nb + (ky + sy) % nb) * nb + (kx + sx) % nb
                            out[b, (sz + 1) * 9 + (sy + 1) * 3 + (sx + 1)] = nbk
    return out


def sedov_block(n, g=3, seed=0, e_blast=1.0, sigma_cells=2.0, p0=1e-5,
                b=(0.05, 0.05, 0.05), gamma=GAMMA, width=None, dtype=np.float64):
    """Uniform rho=1, p=p0 medium with e_blast deposited (as thermal energy)
    in a Gaussian of sigma_cells cells at a seeded off-centre position, and a
    uniform magnetic field."""
    rng = np.random.default_rng(seed)
    m = n + 2 * g
    dx = (width or 1.0) / n
    c = (np.arange(m) - g + 0.5)
    ctr = n / 2 + rng.uniform(-0.25, 0.25, size=3) * n
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    r2 = (X - ctr[0]) ** 2 + (Y - ctr[1]) ** 2 + (Z - ctr[2]) ** 2
    w = np.exp(-0.5 * r2 / sigma_cells ** 2)
    act = (slice(g, g + n),) * 3
    w /= w[act].sum() * dx ** 3
    rho = np.ones((m, m, m))
    p = p0 + (gamma - 1.0) * e_blast * w
    zeros = np.zeros_like(rho)
    bfx = np.full((m, m, m + 1), b[0])
    bfy = np.full((m, m + 1, m), b[1])
    bfz = np.full((m + 1, m, m), b[2])
    bx, by, bz = _centres(bfx, bfy, bfz)
    blk = {"density": rho, "velocity_x": zeros, "velocity_y": zeros.copy(),
           "velocity_z": zeros.copy(), "bfieldi_x": bfx, "bfieldi_y": bfy,
           "bfieldi_z": bfz, "bfield_x": bx, "bfield_y": by, "bfield_z": bz,
           "total_energy": _energy(rho, zeros, zeros, zeros, p, bx, by, bz, gamma),
           "pressure": np.zeros_like(rho)}
    return {k: np.ascontiguousarray(v, dtype=dtype) for k, v in blk.items()}, (dx, dx, dx)


def amr_block_set(seed=3, counts=((16, 1200), (32, 600), (64, 200)), g=3,
                  dtype=np.float32):
    """The mixed-size AMR block set: Sedov blasts (E = 1 in a Gaussian of 2
    cells at a seeded off-centre point, rho = 1, p = 1e-5,
    B = (0.05, 0.05, 0.05)) of the given (size, count) pairs, sizes shuffled
    with the seed; each block's ghost zones come from seeded same-size
    neighbours.  Returns (blocks, dims, widths, nbr) with nbr the
    27-neighbour table (entry 13 is the block itself)."""
    rng = np.random.default_rng(seed)
    sizes = np.concatenate([np.full(c, n) for n, c in counts])
    rng.shuffle(sizes)
    blocks, dims, widths = [], [], []
    for i, n in enumerate(sizes):
        blk, w = sedov_block(int(n), g, seed=seed * 7919 + i, width=1.0, dtype=dtype)
        blk.pop("pressure", None)
        blocks.append(blk)
        dims.append((int(n),) * 3)
        widths.append(w)
    by_size = {n: np.flatnonzero(sizes == n) for n, _ in counts}
    nbr = np.empty((len(sizes), 27), dtype=np.int32)
    for i, n in enumerate(sizes):
        nbr[i] = rng.choice(by_size[n], size=27)
        nbr[i, 13] = i
    return blocks, dims, widths, nbr


# oracle field names <-> Cello field names
ORACLE_NAME = {"density": "rho", "velocity_x": "vx", "velocity_y": "vy",
               "velocity_z": "vz", "total_energy": "etot",
               "internal_energy": "eint", "bfield_x": "bx", "bfield_y": "by",
               "bfield_z": "bz", "bfieldi_x": "bfx", "bfieldi_y": "bfy",
               "bfieldi_z": "bfz", "pressure": "pressure"}
