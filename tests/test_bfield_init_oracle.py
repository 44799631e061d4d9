"""Initial B from an edge-centred vector potential (EnzoInitialBCenter.cpp:
27-127): the oracle's centring equals the reference's own
EnzoBfieldMethodCT::compute_center_bfield bit for bit, the face field it
derives has zero discrete divergence to rounding, and a linear potential gives
the uniform field it encodes."""
import numpy as np
import pytest

from oracle import oracle as O


def _potential(m, seed):
    mx, my, mz = m
    rng = np.random.default_rng(seed)
    ax = rng.standard_normal((mz + 1, my + 1, mx))
    ay = rng.standard_normal((mz + 1, my, mx + 1))
    az = rng.standard_normal((mz, my + 1, mx + 1))
    return ax, ay, az


def test_center_matches_reference():
    L = O.ref_lib()
    if L is None:
        pytest.skip("reference sources not built here")
    m = (9, 7, 8)
    (bfx, bfy, bfz), (bx, by, bz) = O.bfield_from_potential(
        *_potential(m, 3), (0.1, 0.07, 0.13))
    out = [np.zeros((m[2], m[1], m[0])) for _ in range(3)]
    P = O._P
    rc = L.ref_center_bfield(*m, *[a.ctypes.data_as(P) for a in (bfx, bfy, bfz)],
                             *[a.ctypes.data_as(P) for a in out])
    assert rc == 0
    for a, b in zip(out, (bx, by, bz)):
        assert np.array_equal(a, b)


def test_face_field_divergence_free():
    m, w = (10, 8, 6), (0.1, 0.07, 0.13)
    (bfx, bfy, bfz), _ = O.bfield_from_potential(*_potential(m, 5), w)
    div = ((bfx[:, :, 1:] - bfx[:, :, :-1]) / w[0] + (bfy[:, 1:, :] - bfy[:, :-1, :]) / w[1]
           + (bfz[1:, :, :] - bfz[:-1, :, :]) / w[2])
    scale = max(np.abs(b).max() for b in (bfx, bfy, bfz)) / min(w)
    assert np.abs(div).max() < 1e-13 * scale


def test_linear_potential_uniform_field():
    # A = (z By0, x Bz0, y Bx0) has curl (Bx0, By0, Bz0)
    m, w, B0 = (6, 5, 7), (0.25, 0.5, 0.125), (0.3, -1.1, 0.7)
    mx, my, mz = m
    xf = np.arange(mx + 1) * w[0]
    yf = np.arange(my + 1) * w[1]
    zf = np.arange(mz + 1) * w[2]
    ax = np.broadcast_to(B0[1] * zf[:, None, None], (mz + 1, my + 1, mx)).copy()
    ay = np.broadcast_to(B0[2] * xf[None, None, :], (mz + 1, my, mx + 1)).copy()
    az = np.broadcast_to(B0[0] * yf[None, :, None], (mz, my + 1, mx + 1)).copy()
    for dtype, tol in ((np.float64, 1e-14), (np.float32, 1e-6)):
        faces, cells = O.bfield_from_potential(ax, ay, az, w, dtype)
        for d in range(3):
            assert faces[d].dtype == dtype and cells[d].dtype == dtype
            np.testing.assert_allclose(faces[d], B0[d], rtol=tol, atol=tol)
            np.testing.assert_allclose(cells[d], B0[d], rtol=tol, atol=tol)
