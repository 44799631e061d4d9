"""The linear fast-magnetosonic wave of the plain-method configuration: one
n^3 periodic block (3 ghost zones), gamma = 5/3, background rho = 1,
p = 1/gamma, v = 0, B = (1, sqrt 2, 0.5) in the wave frame, wave vector
along (1, 1, 1)/sqrt 3, right-eigenvector perturbation of amplitude 1e-6, B
the discrete curl of an edge-centred vector potential (div B = 0 to
round-off).

A periodic cube admits a (1, 1, 1) wave only with phase 2 pi (x + y + z) / L,
i.e. wavelength L / sqrt 3 (three wavelengths along the box diagonal); that
is the wave used.  Its fast speed is exactly 2 for this background, so one
period is 1 / (2 sqrt 3).

The phase of every cell centre and edge is a multiple of 2 pi / (2 n); the
sines and cosines come from a table built by half-angle square roots and
angle addition, so the state uses IEEE + - * / and sqrt only and is the same
bits on every platform.
"""
import math

import numpy as np

GAMMA = 5.0 / 3.0
N = 32
G = 3
AMPLITUDE = 1e-6
FAST_SPEED = 2.0
PERIOD = 1.0 / (FAST_SPEED * math.sqrt(3.0))


def _trig(nq):
    """cos and sin of 2 pi m / nq, m = 0..nq-1, for nq = 4 * 2^k."""
    c, s = 0.0, 1.0  # the angle pi / 2
    q = 4
    while q < nq:
        c_new = math.sqrt((1.0 + c) / 2.0)
        s = s / (2.0 * c_new)
        c = c_new
        q *= 2
    cos_t, sin_t = [1.0], [0.0]
    for _ in range(1, nq):
        cp, sp = cos_t[-1], sin_t[-1]
        cos_t.append(cp * c - sp * s)
        sin_t.append(sp * c + cp * s)
    return np.array(cos_t), np.array(sin_t)


def _frame():
    r3, r2, r6 = math.sqrt(3.0), math.sqrt(2.0), math.sqrt(6.0)
    e1 = np.array([1.0, 1.0, 1.0]) / r3
    e2 = np.array([-1.0, 1.0, 0.0]) / r2
    e3 = np.array([-1.0, -1.0, 2.0]) / r6
    return e1, e2, e3


def fast_wave_input(n=N, g=G, amplitude=AMPLITUDE, gamma=GAMMA, with_potential=False):
    """Cell fields and face B of the block (Cello layout, (z, y, x)), and the
    cell widths; with with_potential=True also the edge-centred vector potential
    (A_x, A_y, A_z) the face B is the curl of."""
    assert n & (n - 1) == 0 and n >= 2
    m = n + 2 * g
    h = 1.0 / n
    cos_t, sin_t = _trig(2 * n)
    e1, e2, e3 = _frame()
    b_par, b2, b3 = 1.0, math.sqrt(2.0), 0.5
    b0 = b_par * e1 + b2 * e2 + b3 * e3
    rho0, p0 = 1.0, 1.0 / gamma
    # fast-mode right eigenvector, normalised to d rho = amplitude:
    # d v_par = c_f d rho / rho, d p = a^2 d rho, d B_perp = B_perp c_f^2 d rho /
    # (rho (c_f^2 - b_par^2 / rho)), d v_perp = -b_par d B_perp / (rho c_f)
    cf = FAST_SPEED
    a2 = gamma * p0 / rho0
    dv_par = cf * amplitude / rho0
    dp = a2 * amplitude
    k = cf * cf / (rho0 * (cf * cf - b_par * b_par / rho0))
    db2, db3 = b2 * k * amplitude, b3 * k * amplitude
    dv2, dv3 = -b_par * db2 / (rho0 * cf), -b_par * db3 / (rho0 * cf)
    dv = dv_par * e1 + dv2 * e2 + dv3 * e3

    # twice the position in cells from the first active cell's low face:
    # centres are odd, faces even; with x in cells the phase 2 pi (x+y+z) / n
    # is (2x + 2y + 2z) steps of 2 pi / (2n)
    ic = 2 * (np.arange(m) - g) + 1  # cell centres
    iface = 2 * (np.arange(m + 1) - g)  # faces

    def phase_index(tx, ty, tz):
        return np.mod(tz[:, None, None] + ty[None, :, None] + tx[None, None, :], 2 * n)

    pc = phase_index(ic, ic, ic)
    s_c = sin_t[pc]
    rho = rho0 + amplitude * s_c
    vel = [dv[a] * s_c for a in range(3)]
    p = p0 + dp * s_c

    # vector potential: A0 = B0 x r / 2 (uniform B0) plus the perturbation
    # dA = (-dB3 e2 + dB2 e3) cos(phase) / (2 pi sqrt 3 / L)
    kk = 2.0 * math.pi * math.sqrt(3.0)
    da = (-db3 * e2 + db2 * e3) / kk

    def coords(tx, ty, tz):
        return (tx[None, None, :] * (0.5 * h), ty[None, :, None] * (0.5 * h),
                tz[:, None, None] * (0.5 * h))

    def potential(comp, tx, ty, tz):
        x, y, z = coords(tx, ty, tz)
        r = (x, y, z)
        j, l = (comp + 1) % 3, (comp + 2) % 3
        a0 = 0.5 * (b0[j] * r[l] - b0[l] * r[j])
        return a0 + da[comp] * cos_t[phase_index(tx, ty, tz)]

    ax = potential(0, ic, iface, iface)  # (m+1, m+1, m)
    ay = potential(1, iface, ic, iface)  # (m+1, m, m+1)
    az = potential(2, iface, iface, ic)  # (m, m+1, m+1)
    bfx = (az[:, 1:, :] - az[:, :-1, :]) / h - (ay[1:, :, :] - ay[:-1, :, :]) / h
    bfy = (ax[1:, :, :] - ax[:-1, :, :]) / h - (az[:, :, 1:] - az[:, :, :-1]) / h
    bfz = (ay[:, :, 1:] - ay[:, :, :-1]) / h - (ax[:, 1:, :] - ax[:, :-1, :]) / h
    bx = 0.5 * (bfx[:, :, :-1] + bfx[:, :, 1:])
    by = 0.5 * (bfy[:, :-1, :] + bfy[:, 1:, :])
    bz = 0.5 * (bfz[:-1, :, :] + bfz[1:, :, :])
    e_tot = (p / ((gamma - 1.0) * rho)
             + 0.5 * (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2])
             + 0.5 * (bx * bx + by * by + bz * bz) / rho)
    out = {"density": rho, "velocity_x": vel[0], "velocity_y": vel[1],
           "velocity_z": vel[2], "total_energy": e_tot, "bfield_x": bx,
           "bfield_y": by, "bfield_z": bz, "bfieldi_x": bfx, "bfieldi_y": bfy,
           "bfieldi_z": bfz, "pressure": np.zeros((m, m, m))}
    shapes = {"bfieldi_x": (m, m, m + 1), "bfieldi_y": (m, m + 1, m),
              "bfieldi_z": (m + 1, m, m)}
    for key, v in out.items():
        assert v.shape == shapes.get(key, (m, m, m)), (key, v.shape)
    state = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in out.items()}
    if with_potential:
        return state, (h, h, h), tuple(np.ascontiguousarray(a) for a in (ax, ay, az))
    return state, (h, h, h)
