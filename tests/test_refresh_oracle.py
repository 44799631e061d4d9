"""The mesh ghost refresh on the CPU (Cello's FieldFace::face_to_face with
the "linear" restriction and prolongation, src/Cello/data_FieldFace.cpp:
440-566):

  - the oracle's regions equal the reference's own Box
    (src/Cello/mesh_Box.cpp) and the C ABI's host planner
    (mhdvlct_refresh_face_box) for every face, child, level step, centering
    and ghost depth;
  - the oracle's refresh of a two-level mesh equals the reference's own
    ProlongLinear / RestrictLinear driven through face_to_face's control flow,
    bit for bit in FP64 and FP32 (density a power of two in the senders, so
    that the reference's in-place multiply-divide of the sender is exact);
  - with a general density the two differ only by that round trip: at most
    one rounding in the reference's sender cells, a few roundings in the
    density-weighted ghosts;
  - every ghost cell of the mesh is written, and a linear field is
    reproduced exactly by prolongation and restriction (the geometry);
  - the C ABI rejects what the reference asserts on, before any device work.
"""
import ctypes
import itertools

import numpy as np
import pytest

from oracle import oracle as O
from mhdvlct import block as B, capi, mesh as M
from helpers import HYDRO_SLOTS, mesh_blocks

FACES = [f for f in itertools.product((-1, 0, 1), repeat=3) if f != (0, 0, 0)]
CHILDREN = list(itertools.product((0, 1), repeat=3))


def _product_box(n, g, c, t, f, k):
    out = [(ctypes.c_int * 3)() for _ in range(4)]
    i3 = lambda v: (ctypes.c_int * 3)(*v)  # noqa: E731
    rc = capi.lib().mhdvlct_refresh_face_box(i3(n), i3(g), i3(c), t, i3(f), i3(k), *out)
    return rc, tuple(tuple(o) for o in out)


@pytest.mark.parametrize("n,g", [((16, 16, 16), (4, 4, 4)), ((8, 16, 12), (4, 4, 4)),
                                 ((16, 16, 16), (3, 3, 3)), ((6, 10, 8), (2, 2, 2))])
def test_regions_match_reference_box(n, g):
    have_ref = O.refresh_ref_lib() is not None
    count = 0
    for t in (-1, 0, 1):
        for c in ((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)):
            for f in FACES:
                for k in (CHILDREN if t else [(0, 0, 0)]):
                    mine = O.refresh_box(n, g, c, t, f, k)
                    if have_ref:
                        assert O.refresh_box(n, g, c, t, f, k, ref=True) == mine, (t, c, f, k)
                    rc, prod = _product_box(n, g, c, t, f, k)
                    assert rc in (0, 1)
                    assert prod == mine, (t, c, f, k)
                    count += 1
    assert count == 4 * 26 * (8 + 1 + 8)


def _two_level_mesh():
    # 2x2x2 root blocks, the first refined once: coarse-fine faces on every
    # axis, edge and corner, with periodic wrap
    return M.Mesh((2, 2, 2), refine=lambda lvl, c: c == (0, 0, 0))


def _three_level_mesh():
    # a 4^3 root grid whose central 2^3 is refined, and the centre of that
    # region refined again: level-1 blocks receive both restrictions and
    # prolongations
    def refine(lvl, c):
        if lvl == 0:
            return all(1 <= x < 3 for x in c)
        return lvl == 1 and all(3 <= x < 5 for x in c)
    return M.Mesh((4, 4, 4), refine=refine, max_level=2)


def _run(blocks, n, g, faces, cons, ref):
    O.refresh_faces(blocks, n, g, faces, cons, ref=ref)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("cons", [capi.MHD_CONSERVATIVE_DEFAULT, 0])
@pytest.mark.parametrize("n", [(8, 8, 8), (8, 12, 16)])
def test_refresh_matches_reference(dtype, cons, n):
    if O.refresh_ref_lib() is None:
        pytest.skip("reference sources not built here")
    mesh = _two_level_mesh()
    g = (4, 4, 4)
    faces = mesh.face_ints()
    a = mesh_blocks(len(mesh.leaves), n, g[0], HYDRO_SLOTS, dtype, seed=5, rho_pow2=True)
    b = [{s: x.copy() for s, x in blk.items()} for blk in a]
    _run(a, n, g, faces, cons, ref=False)
    _run(b, n, g, faces, cons, ref=True)
    for i, (x, y) in enumerate(zip(a, b)):
        for s in x:
            assert np.array_equal(x[s], y[s], equal_nan=True), (i, capi.FIELD_SLOTS[s])


def test_general_density_differs_only_by_the_round_trip():
    if O.refresh_ref_lib() is None:
        pytest.skip("reference sources not built here")
    mesh = _two_level_mesh()
    n, g = (8, 8, 8), (4, 4, 4)
    faces = mesh.face_ints()
    a = mesh_blocks(len(mesh.leaves), n, g[0], HYDRO_SLOTS, np.float64, seed=9)
    b = [{s: x.copy() for s, x in blk.items()} for blk in a]
    _run(a, n, g, faces, capi.MHD_CONSERVATIVE_DEFAULT, ref=False)
    _run(b, n, g, faces, capi.MHD_CONSERVATIVE_DEFAULT, ref=True)
    act = tuple(slice(g[0], g[0] + x) for x in n[::-1])
    worst_active = worst_ghost = 0.0
    for x, y in zip(a, b):
        for s in x:
            ok = np.isfinite(x[s])
            rel = np.abs(x[s][ok] - y[s][ok]) / np.maximum(np.abs(x[s][ok]), 1e-300)
            assert np.array_equal(np.isfinite(x[s]), np.isfinite(y[s]))
            if s == 0 or s not in (1, 2, 3, 4):
                assert np.array_equal(x[s], y[s], equal_nan=True)
                continue
            r_act = np.abs(x[s][act] - y[s][act]) / np.abs(x[s][act])
            worst_active = max(worst_active, float(r_act.max()))
            worst_ghost = max(worst_ghost, float(rel.max()))
    assert worst_active <= 2.3e-16 * 2  # one rounding per sending face
    assert worst_ghost < 1e-14


@pytest.mark.parametrize("cons", [capi.MHD_CONSERVATIVE_DEFAULT, 0])
@pytest.mark.parametrize("n", [(8, 8, 8), (8, 12, 16)])
def test_every_ghost_cell_is_written(cons, n):
    mesh = _two_level_mesh()
    g = (4, 4, 4)
    blocks = mesh_blocks(len(mesh.leaves), n, g[0], HYDRO_SLOTS, np.float64, seed=2)
    _run(blocks, n, g, mesh.face_ints(), cons, ref=False)
    for blk in blocks:
        for s, x in blk.items():
            assert np.isfinite(x).all(), capi.FIELD_SLOTS[s]


def test_linear_field_is_reproduced():
    # f = a + b.x in physical coordinates with unit density: linear
    # prolongation and extrapolation, and the 2x2x2 mean, are exact
    mesh = _two_level_mesh()
    n, g = (8, 8, 8), 4
    blocks = mesh_blocks(len(mesh.leaves), n, g, (0, 1), np.float64, seed=1)
    coef = np.array([0.3, -0.7, 1.1])

    def centres(i):
        lvl, _ = mesh.leaves[i]
        h = 2.0 ** (mesh.max_level - lvl)  # cell width in finest cells
        o = mesh.origin(i, n)
        ax = [o[a] + (np.arange(n[a] + 2 * g) - g + 0.5) * h for a in range(3)]
        return np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")  # z, y, x

    for i, blk in enumerate(blocks):
        z, y, x = centres(i)
        blk[0][...] = 1.0
        blk[1][...] = np.nan
        act = tuple(slice(g, g + k) for k in n[::-1])
        blk[1][act] = (coef[0] * x + coef[1] * y + coef[2] * z)[act]
    _run(blocks, n, (g,) * 3, mesh.face_ints(), 0, ref=False)
    ext = [mesh.extent(mesh.max_level)[a] * n[a] for a in range(3)]
    for i, blk in enumerate(blocks):
        z, y, x = centres(i)
        # periodic images: compare modulo the domain
        want = coef[0] * (x % ext[0]) + coef[1] * (y % ext[1]) + coef[2] * (z % ext[2])
        got = blk[1]
        inside = ((x > 0) & (x < ext[0]) & (y > 0) & (y < ext[1]) & (z > 0) & (z < ext[2]))
        assert np.allclose(got[inside], want[inside], rtol=0, atol=1e-12), i


def test_abi_rejects_what_the_reference_asserts_on():
    L = capi.lib()
    h = ctypes.c_void_p()
    p = B.make_params(mhd_choice="no_bfield", riemann_solver="hllc")
    capi.check(L.mhdvlct_create(ctypes.byref(p), ctypes.byref(h)))
    try:
        fake = 0x1000  # never dereferenced: every case fails validation first

        def view(gd, mhd=False):
            v = capi.MhdBlockView()
            v.dtype = capi.MHD_DTYPE_F64
            for a in range(3):
                v.n[a] = 8
                v.ghost[a] = gd
                v.cell_width[a] = 1.0
            v.density = fake
            for a in range(3):
                v.velocity[a] = fake
                if mhd:
                    v.bfield[a] = fake
                    v.bfieldi[a] = fake
            v.total_energy = fake
            return v

        def run(views, face, cons=0):
            arr = (capi.MhdBlockView * len(views))(*views)
            f = capi.MhdRefreshFace()
            f.sender, f.receiver, f.type = face[0], face[1], face[2]
            for a in range(3):
                f.face[a] = face[3][a]
                f.child[a] = face[4][a]
            return L.mhdvlct_refresh_faces(h, arr, len(views), ctypes.byref(f), 1,
                                           ctypes.c_uint(cons), None)

        # odd ghost depth: the fine extent is not twice the coarse one
        assert run([view(3), view(3)], (0, 1, 1, (1, 0, 0), (0, 0, 0))) == capi.MHD_ERR_INVALID
        # face-centred B across levels
        assert run([view(4, True), view(4, True)],
                   (0, 1, -1, (1, 0, 0), (1, 0, 0))) == capi.MHD_ERR_INVALID
        # index out of range, zero face, density weighting of density
        assert run([view(4)], (0, 1, 0, (1, 0, 0), (0, 0, 0))) == capi.MHD_ERR_INVALID
        assert run([view(4)], (0, 0, 0, (0, 0, 0), (0, 0, 0))) == capi.MHD_ERR_INVALID
        assert run([view(4), view(4)], (0, 1, 1, (1, 0, 0), (0, 0, 0)),
                   cons=1) == capi.MHD_ERR_INVALID
        # mixed sizes
        v2 = view(4)
        v2.n[0] = 16
        assert run([view(4), v2], (0, 1, 0, (1, 0, 0), (0, 0, 0))) == capi.MHD_ERR_INVALID
        # an empty face list is a no-op (no device work), for the refresh and
        # for the flux correction
        arr = (capi.MhdBlockView * 2)(view(4), view(4))
        assert L.mhdvlct_refresh_faces(h, arr, 2, None, 0, ctypes.c_uint(0), None) == capi.MHD_OK
        fcs = (capi.MhdFluxCorrection * 2)()
        assert L.mhdvlct_flux_correct(h, arr, 2, fcs, None, 0, ctypes.c_uint(0),
                                      None) == capi.MHD_OK
    finally:
        L.mhdvlct_destroy(h)


def test_mesh_faces_pair_up():
    # every coarse-to-fine face has a fine-to-coarse partner and vice versa
    mesh = M.Mesh((3, 2, 2), refine=lambda lvl, c: c in ((0, 0, 0), (1, 0, 0)))
    fs = mesh.faces()
    fine = {(s, r) for s, r, t, _, _ in fs if t == capi.MHD_REFRESH_FINE}
    coarse = {(r, s) for s, r, t, _, _ in fs if t == capi.MHD_REFRESH_COARSE}
    assert fine == coarse and len(fine) > 0
    with pytest.raises(ValueError):  # a 3-level jump breaks the 2:1 balance
        M.Mesh((2, 1, 1), refine=lambda lvl, c: c[0] == 0 and c[1] == 0 and c[2] == 0,
               max_level=2).faces()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_three_levels_match_reference(dtype):
    if O.refresh_ref_lib() is None:
        pytest.skip("reference sources not built here")
    mesh = _three_level_mesh()
    n, g = (8, 8, 8), (4, 4, 4)
    faces = mesh.face_ints()
    a = mesh_blocks(len(mesh.leaves), n, g[0], HYDRO_SLOTS, dtype, seed=8, rho_pow2=True)
    b = [{s: x.copy() for s, x in blk.items()} for blk in a]
    _run(a, n, g, faces, capi.MHD_CONSERVATIVE_DEFAULT, ref=False)
    _run(b, n, g, faces, capi.MHD_CONSERVATIVE_DEFAULT, ref=True)
    # the power-of-two densities span a factor 64, so the one-sided
    # prolongation weights can extrapolate a density to zero and the
    # density-weighted division gives NaN -- in the reference alike
    for i, (x, y) in enumerate(zip(a, b)):
        for s_ in x:
            assert np.array_equal(x[s_], y[s_], equal_nan=True), (i, capi.FIELD_SLOTS[s_])


def test_three_levels_fill_every_ghost_cell():
    mesh = _three_level_mesh()
    n, g = (8, 8, 8), (4, 4, 4)
    blocks = mesh_blocks(len(mesh.leaves), n, g[0], HYDRO_SLOTS, np.float64, seed=3)
    _run(blocks, n, g, mesh.face_ints(), capi.MHD_CONSERVATIVE_DEFAULT, ref=False)
    for i, blk in enumerate(blocks):
        for s_, x in blk.items():
            assert np.isfinite(x).all(), (i, capi.FIELD_SLOTS[s_])
