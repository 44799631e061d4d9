"""Device-resident block state in Cello's field layout, plus the Method-level
host interface mirroring Enzo-E's EnzoMethodMHDVlct.

`EnzoMethodMHDVlct` here keeps the reference's public surface
(src/Enzo/hydro-mhd/EnzoMethodMHDVlct.hpp; src/Cello/problem_Method.hpp:
23-124): construction from the `Method:mhd_vlct` parameter block, name()
returning "mhd_vlct", compute(block) and timestep(block).  All numerics run in
libmhdvlct_gb300.so; torch only provides device memory and streams.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi

CELL_KEYS = ("density", "velocity_x", "velocity_y", "velocity_z",
             "total_energy", "internal_energy", "bfield_x", "bfield_y",
             "bfield_z", "pressure")
FACE_KEYS = ("bfieldi_x", "bfieldi_y", "bfieldi_z")


class Block:
    """One ghosted block: a dict of device tensors keyed by Cello field name.

    Shapes are (mz, my, mx) with m = n + 2g; bfieldi_d has one more entry
    along axis d (src/Cello/data_FieldData.cpp:585-619)."""

    def __init__(self, n, ghost=3, cell_width=(1.0, 1.0, 1.0), mhd=True,
                 dual_energy=False, dtype=torch.float64, device="cuda",
                 gravity=False, npassive=0):
        nx, ny, nz = (n, n, n) if np.isscalar(n) else tuple(n)
        self.n = (int(nx), int(ny), int(nz))
        self.ghost = int(ghost)
        self.cell_width = tuple(float(w) for w in cell_width)
        self.mhd = mhd
        self.dual_energy = dual_energy
        self.dtype = dtype
        self.device = device
        g = self.ghost
        mx, my, mz = nx + 2 * g, ny + 2 * g, nz + 2 * g
        self.m = (mx, my, mz)
        shp = (mz, my, mx)
        keys = ["density", "velocity_x", "velocity_y", "velocity_z",
                "total_energy", "pressure"]
        if dual_energy:
            keys.append("internal_energy")
        if gravity:
            keys += ["acceleration_x", "acceleration_y", "acceleration_z"]
        self.npassive = int(npassive)
        keys += [f"passive_{k}" for k in range(self.npassive)]
        if mhd:
            keys += ["bfield_x", "bfield_y", "bfield_z"]
        self.fields = {k: torch.zeros(shp, dtype=dtype, device=device)
                       for k in keys}
        if mhd:
            self.fields["bfieldi_x"] = torch.zeros((mz, my, mx + 1), dtype=dtype, device=device)
            self.fields["bfieldi_y"] = torch.zeros((mz, my + 1, mx), dtype=dtype, device=device)
            self.fields["bfieldi_z"] = torch.zeros((mz + 1, my, mx), dtype=dtype, device=device)

    def view(self) -> capi.MhdBlockView:
        v = capi.MhdBlockView()
        v.dtype = capi.MHD_DTYPE_F64 if self.dtype == torch.float64 else capi.MHD_DTYPE_F32
        for a in range(3):
            v.n[a] = self.n[a]
            v.ghost[a] = self.ghost
            v.cell_width[a] = self.cell_width[a]
        f = self.fields

        def p(k):
            t = f.get(k)
            if t is None:
                return None
            assert t.is_contiguous() and t.dtype == self.dtype
            return t.data_ptr()
        v.density = p("density")
        for a, k in enumerate(("velocity_x", "velocity_y", "velocity_z")):
            v.velocity[a] = p(k)
        v.total_energy = p("total_energy")
        v.internal_energy = p("internal_energy")
        for a, k in enumerate(("bfield_x", "bfield_y", "bfield_z")):
            v.bfield[a] = p(k)
        for a, k in enumerate(FACE_KEYS):
            v.bfieldi[a] = p(k)
        v.pressure = p("pressure")
        for a, k in enumerate(("acceleration_x", "acceleration_y", "acceleration_z")):
            v.acceleration[a] = p(k)
        for k in range(self.npassive):
            v.passive[k] = p(f"passive_{k}")
        v.npassive = self.npassive
        return v

    # host <-> device helpers (tests, IC upload)
    def load_numpy(self, arrays: dict) -> None:
        for k, a in arrays.items():
            if k in self.fields:
                self.fields[k].copy_(torch.as_tensor(np.ascontiguousarray(a)).to(
                    self.device, self.dtype))

    def to_numpy(self) -> dict:
        return {k: v.detach().cpu().numpy() for k, v in self.fields.items()}


def make_params(mhd_choice="constrained_transport", riemann_solver="hlld",
                reconstruct_method="plm", time_scheme="vl", theta_limiter=1.5,
                courant=None, gamma=5.0 / 3.0, density_floor=1e-200,
                pressure_floor=1e-200, dual_energy=False,
                dual_energy_eta=0.001) -> capi.MhdVlctParams:
    p = capi.MhdVlctParams()
    capi.lib().mhdvlct_params_default(ctypes.byref(p))
    p.mhd_choice = mhd_choice.encode()
    p.riemann_solver = riemann_solver.encode()
    p.reconstruct_method = reconstruct_method.encode()
    p.time_scheme = time_scheme.encode()
    p.theta_limiter = theta_limiter
    if courant is not None:
        p.courant = courant
    p.gamma = gamma
    p.density_floor = density_floor
    p.pressure_floor = pressure_floor
    p.dual_energy = int(bool(dual_energy))
    p.dual_energy_eta = dual_energy_eta
    return p


def parse_params(text: str) -> capi.MhdVlctParams:
    p = capi.MhdVlctParams()
    err = ctypes.create_string_buffer(256)
    rc = capi.lib().mhdvlct_params_parse(text.encode(), ctypes.byref(p), err, 256)
    if rc != capi.MHD_OK:
        raise capi.MhdError(rc, err.value.decode())
    return p


def _stream_ptr(stream) -> int | None:
    if stream is None:
        stream = torch.cuda.current_stream()
    return stream.cuda_stream


class FluxBuffers:
    """Device arrays of a block's boundary fluxes for flux correction:
    arrays[(axis, side, quantity)] of the active face (axis 0: (nz, ny),
    axis 1: (nz, nx), axis 2: (ny, nx)), in the block's dtype."""

    def __init__(self, block: Block, quantities=(0, 1, 2, 3, 4)):
        nx, ny, nz = block.n
        shapes = [(nz, ny), (nz, nx), (ny, nx)]
        self.fc = capi.MhdFluxCorrection()
        self.arrays = {}
        for ax in range(3):
            for side in range(2):
                for q in quantities:
                    t = torch.zeros(shapes[ax], dtype=block.dtype, device=block.device)
                    self.arrays[(ax, side, q)] = t
                    self.fc.flux[ax][side][q] = t.data_ptr()


class EnzoMethodMHDVlct:
    """The `mhd_vlct` Method on device-resident blocks."""

    def __init__(self, params: capi.MhdVlctParams | str | None = None, **kw):
        if isinstance(params, str):
            params = parse_params(params)
        elif params is None:
            params = make_params(**kw)
        self.params = params
        h = ctypes.c_void_p()
        rc = capi.lib().mhdvlct_create(ctypes.byref(params), ctypes.byref(h))
        if rc != capi.MHD_OK:
            msg = capi.lib().mhdvlct_last_error_string(h).decode() if h else ""
            if h:
                capi.lib().mhdvlct_destroy(h)
            raise capi.MhdError(rc, msg)
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h:
            capi.lib().mhdvlct_destroy(h)
            self.handle = None

    @staticmethod
    def name() -> str:
        return "mhd_vlct"

    @property
    def courant(self) -> float:
        return capi.lib().mhdvlct_courant(self.handle)

    def required_ghost_depth(self) -> int:
        return capi.lib().mhdvlct_required_ghost_depth(self.handle)

    def compute(self, block: Block, dt: float, stream=None) -> None:
        v = block.view()
        rc = capi.lib().mhdvlct_block_step(self.handle, ctypes.byref(v), dt,
                                           _stream_ptr(stream))
        capi.check(rc, self.handle, "mhdvlct_block_step")

    def compute_store_fluxes(self, block: Block, dt: float, quantities=(0, 1, 2, 3, 4),
                             stream=None, buffers: "FluxBuffers | None" = None) -> dict:
        """compute() with store_fluxes_for_corrections (hydro only,
        EnzoMethodMHDVlct.cpp:250-330): returns {(axis, side, quantity):
        device tensor} of dt/dx-scaled fluxes through the block's active
        boundary faces.  Pass `buffers` (a FluxBuffers of this block's shape)
        to reuse device arrays across calls."""
        if buffers is None:
            buffers = FluxBuffers(block, quantities)
        v = block.view()
        rc = capi.lib().mhdvlct_block_step_fc(self.handle, ctypes.byref(v), dt,
                                              ctypes.byref(buffers.fc),
                                              _stream_ptr(stream))
        capi.check(rc, self.handle, "mhdvlct_block_step_fc")
        return buffers.arrays

    def timestep(self, block: Block, stream=None) -> float:
        v = block.view()
        dt = ctypes.c_double()
        rc = capi.lib().mhdvlct_block_timestep(self.handle, ctypes.byref(v),
                                               ctypes.byref(dt),
                                               _stream_ptr(stream))
        capi.check(rc, self.handle, "mhdvlct_block_timestep")
        return dt.value

    def initialize_bfield_from_potential(self, block: Block, ax: torch.Tensor,
                                         ay: torch.Tensor, az: torch.Tensor,
                                         stream=None) -> None:
        """Set the block's face and centred B from an edge-centred vector
        potential (EnzoInitialBCenter::initialize_bfield_interface then
        ::initialize_bfield_center, EnzoInitialBCenter.cpp:27-127).  ax, ay,
        az are float64 device tensors of shapes (mz+1, my+1, mx),
        (mz+1, my, mx+1) and (mz, my+1, mx+1)."""
        mx, my, mz = (x + 2 * block.ghost for x in block.n)
        for a, shp in ((ax, (mz + 1, my + 1, mx)), (ay, (mz + 1, my, mx + 1)),
                       (az, (mz, my + 1, mx + 1))):
            if (tuple(a.shape) != shp or a.dtype != torch.float64 or not a.is_cuda
                    or not a.is_contiguous()):
                raise ValueError(f"vector potential component must be a contiguous "
                                 f"float64 device tensor of shape {shp}")
        v = block.view()
        rc = capi.lib().mhdvlct_block_bfield_from_potential(
            self.handle, ctypes.byref(v), ax.data_ptr(), ay.data_ptr(), az.data_ptr(),
            _stream_ptr(stream))
        capi.check(rc, self.handle, "mhdvlct_block_bfield_from_potential")

    def refresh_faces(self, blocks, faces, conservative=None, stream=None) -> None:
        """Cello's ghost refresh over a mesh of blocks whose neighbours may be
        one level coarser or finer (restrict / prolong, "linear"), all faces in
        one launch.  `faces`: MhdRefreshFace records, as (array, count) from
        mesh.Mesh.face_array() or a list of (sender, receiver, type, face,
        child) tuples; `conservative`: field-slot mask of the density-weighted
        fields (default: velocities and total energy)."""
        if conservative is None:
            conservative = capi.MHD_CONSERVATIVE_DEFAULT
        if isinstance(faces, tuple) and len(faces) == 2 and not isinstance(faces[0], int):
            arr, nf = faces
        else:
            nf = len(faces)
            arr = (capi.MhdRefreshFace * max(1, nf))()
            for i, (s, r, t, f, k) in enumerate(faces):
                arr[i].sender, arr[i].receiver, arr[i].type = s, r, t
                for a in range(3):
                    arr[i].face[a], arr[i].child[a] = f[a], k[a]
        views = (capi.MhdBlockView * len(blocks))(*[b.view() for b in blocks])
        rc = capi.lib().mhdvlct_refresh_faces(self.handle, views, len(blocks), arr, nf,
                                              ctypes.c_uint(conservative),
                                              _stream_ptr(stream))
        capi.check(rc, self.handle, "mhdvlct_refresh_faces")

    def flux_correct(self, blocks, buffers, faces, conservative=None, stream=None) -> None:
        """Cello's "flux_correct" Method over a mesh after a step that stored
        the boundary fluxes: every coarse block's boundary cells next to finer
        blocks are corrected by the difference between its own fluxes and its
        finer neighbours' coarsened ones.  `buffers`: one FluxBuffers per
        block (as compute_store_fluxes filled them); `faces`: the mesh's
        refresh faces (mesh.Mesh.face_array() or a list of tuples)."""
        if conservative is None:
            conservative = capi.MHD_CONSERVATIVE_DEFAULT
        if isinstance(faces, tuple) and len(faces) == 2 and not isinstance(faces[0], int):
            arr, nf = faces
        else:
            nf = len(faces)
            arr = (capi.MhdRefreshFace * max(1, nf))()
            for i, (s_, r, t, f, k) in enumerate(faces):
                arr[i].sender, arr[i].receiver, arr[i].type = s_, r, t
                for a in range(3):
                    arr[i].face[a], arr[i].child[a] = f[a], k[a]
        views = (capi.MhdBlockView * len(blocks))(*[b.view() for b in blocks])
        fcs = (capi.MhdFluxCorrection * len(blocks))(*[bf.fc for bf in buffers])
        rc = capi.lib().mhdvlct_flux_correct(self.handle, views, len(blocks), fcs, arr, nf,
                                             ctypes.c_uint(conservative), _stream_ptr(stream))
        capi.check(rc, self.handle, "mhdvlct_flux_correct")

    def fill_ghosts_periodic(self, block: Block, stream=None) -> None:
        v = block.view()
        rc = capi.lib().mhdvlct_fill_ghosts_periodic(self.handle, ctypes.byref(v),
                                                     _stream_ptr(stream))
        capi.check(rc, self.handle, "mhdvlct_fill_ghosts_periodic")
