"""ctypes binding of libmhdvlct_gb300.so (the C ABI in include/mhdvlct_gb300.h).

This is the reference-facing boundary as a Python caller sees it: plain
pointers and sizes, no torch types in the signatures.  Loading fails loudly
when the shared library has not been built; there is no fallback.
"""
from __future__ import annotations

import ctypes
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "libmhdvlct_gb300.so")

MHD_OK = 0
MHD_ERR_INVALID = 1
MHD_ERR_CUDA = 2
MHD_ERR_NOMEM = 3
MHD_ERR_GHOST = 4
MHD_ERR_NONFINITE = 5
MHD_ERR_TIMEOUT = 6
MHD_ERR_BUSY = 7
MHD_DTYPE_F64 = 0
MHD_DTYPE_F32 = 1

# Every symbol the header declares (checked by the CPU test suite).
EXPORTED = (
    "mhdvlct_params_default", "mhdvlct_params_parse", "mhdvlct_create",
    "mhdvlct_destroy", "mhdvlct_last_error_string",
    "mhdvlct_courant", "mhdvlct_required_ghost_depth", "mhdvlct_block_step",
    "mhdvlct_block_step_noalloc", "mhdvlct_block_step_fc",
    "mhdvlct_block_bfield_from_potential",
    "mhdvlct_block_timestep", "mhdvlct_fill_ghosts_periodic",
    "mhdvlct_block_timestep_device", "mhdvlct_dt_min_device",
    "mhdvlct_block_step_device_dt",
    "mhdvlct_refresh_faces", "mhdvlct_refresh_face_box", "mhdvlct_flux_correct",
    "mhdvlct_batch_create", "mhdvlct_batch_create_ex", "mhdvlct_batch_destroy",
    "mhdvlct_batch_block_view", "mhdvlct_batch_set_neighbors",
    "mhdvlct_batch_refresh", "mhdvlct_batch_set_refresh_faces",
    "mhdvlct_batch_set_flux_correction", "mhdvlct_batch_step", "mhdvlct_batch_timestep",
    "mhdvlct_batch_run", "mhdvlct_batch_set_tile", "mhdvlct_batch_set_stage_tile",
    "mhdvlct_batch_autotune",
    "mhdvlct_batch_state_region", "mhdvlct_batch_profile",
    "mhdvlct_batch_diagnostics", "mhdvlct_batch_state_segments", "mhdvlct_batch_run_host", "mhdserve_create",
    "mhdserve_destroy", "mhdserve_submit", "mhdserve_pump", "mhdserve_poll",
    "mhdserve_result", "mhdserve_timing", "mhdserve_last_error_string",
)


class MhdVlctParams(ctypes.Structure):
    _fields_ = [("mhd_choice", ctypes.c_char * 32),
                ("riemann_solver", ctypes.c_char * 16),
                ("time_scheme", ctypes.c_char * 16),
                ("reconstruct_method", ctypes.c_char * 16),
                ("theta_limiter", ctypes.c_double),
                ("courant", ctypes.c_double),
                ("gamma", ctypes.c_double),
                ("density_floor", ctypes.c_double),
                ("pressure_floor", ctypes.c_double),
                ("dual_energy", ctypes.c_int),
                ("dual_energy_eta", ctypes.c_double)]


class MhdFluxCorrection(ctypes.Structure):
    """flux[axis][side][quantity]: device arrays of the active boundary faces."""
    _fields_ = [("flux", ctypes.c_void_p * 10 * 2 * 3)]


MHD_Q_DENSITY, MHD_Q_VELOCITY_X, MHD_Q_VELOCITY_Y, MHD_Q_VELOCITY_Z = 0, 1, 2, 3
MHD_Q_TOTAL_ENERGY, MHD_Q_INTERNAL_ENERGY = 4, 5
MHD_Q_PASSIVE_0 = 6  # .. 9: the passive scalars (conserved form)
MHD_FC_NQ = 10

MHD_REFRESH_COARSE, MHD_REFRESH_SAME, MHD_REFRESH_FINE = -1, 0, 1
# field slots of the mesh refresh (MHD_FIELD_* in the header)
FIELD_SLOTS = ("density", "velocity_x", "velocity_y", "velocity_z", "total_energy",
               "internal_energy", "bfield_x", "bfield_y", "bfield_z", "pressure",
               "acceleration_x", "acceleration_y", "acceleration_z", "passive_0",
               "passive_1", "passive_2", "passive_3", "bfieldi_x", "bfieldi_y",
               "bfieldi_z")
MHD_NFIELD_SLOTS = len(FIELD_SLOTS)
MHD_FIELD_PASSIVE_0 = FIELD_SLOTS.index("passive_0")
MHD_CONSERVATIVE_DEFAULT = sum(1 << FIELD_SLOTS.index(k) for k in (
    "velocity_x", "velocity_y", "velocity_z", "total_energy"))


class MhdRefreshFace(ctypes.Structure):
    """One (sender, receiver) pair of a mesh refresh, from the sender's side."""
    _fields_ = [("sender", ctypes.c_int), ("receiver", ctypes.c_int),
                ("type", ctypes.c_int), ("face", ctypes.c_int * 3),
                ("child", ctypes.c_int * 3)]


class MhdBlockView(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int),
                ("n", ctypes.c_int * 3),
                ("ghost", ctypes.c_int * 3),
                ("cell_width", ctypes.c_double * 3),
                ("density", ctypes.c_void_p),
                ("velocity", ctypes.c_void_p * 3),
                ("total_energy", ctypes.c_void_p),
                ("internal_energy", ctypes.c_void_p),
                ("bfield", ctypes.c_void_p * 3),
                ("bfieldi", ctypes.c_void_p * 3),
                ("pressure", ctypes.c_void_p),
                ("acceleration", ctypes.c_void_p * 3),
                ("passive", ctypes.c_void_p * 4),
                ("npassive", ctypes.c_int)]


class MhdServeRequest(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int),
                ("cycles", ctypes.c_int),
                ("riemann_solver", ctypes.c_char * 16),
                ("reconstruct_method", ctypes.c_char * 16),
                ("mhd", ctypes.c_int),
                ("box_size", ctypes.c_double),
                ("init", ctypes.c_void_p * 12)]


_lib = None


def lib() -> ctypes.CDLL:
    """Load the library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    P = ctypes.POINTER
    L.mhdvlct_params_default.argtypes = [P(MhdVlctParams)]
    L.mhdvlct_params_default.restype = None
    L.mhdvlct_params_parse.argtypes = [ctypes.c_char_p, P(MhdVlctParams),
                                       ctypes.c_char_p, ctypes.c_size_t]
    L.mhdvlct_create.argtypes = [P(MhdVlctParams), P(vp)]
    L.mhdvlct_destroy.argtypes = [vp]
    L.mhdvlct_last_error_string.argtypes = [vp]
    L.mhdvlct_last_error_string.restype = ctypes.c_char_p
    L.mhdvlct_required_ghost_depth.argtypes = [vp]
    L.mhdvlct_courant.argtypes = [vp]
    L.mhdvlct_courant.restype = dp
    L.mhdvlct_block_step.argtypes = [vp, P(MhdBlockView), dp, vp]
    L.mhdvlct_block_step_noalloc.argtypes = [vp, P(MhdBlockView), dp, vp]
    L.mhdvlct_block_step_fc.argtypes = [vp, P(MhdBlockView), dp, P(MhdFluxCorrection), vp]
    L.mhdvlct_block_bfield_from_potential.argtypes = [vp, P(MhdBlockView), vp, vp, vp, vp]
    L.mhdvlct_block_timestep.argtypes = [vp, P(MhdBlockView), P(dp), vp]
    L.mhdvlct_fill_ghosts_periodic.argtypes = [vp, P(MhdBlockView), vp]
    L.mhdvlct_block_timestep_device.argtypes = [vp, P(MhdBlockView), vp, vp]
    L.mhdvlct_dt_min_device.argtypes = [vp, vp, ip, vp, vp]
    L.mhdvlct_block_step_device_dt.argtypes = [vp, P(MhdBlockView), vp, vp]
    L.mhdvlct_refresh_faces.argtypes = [vp, P(MhdBlockView), ip, P(MhdRefreshFace), ip,
                                        ctypes.c_uint, vp]
    L.mhdvlct_refresh_face_box.argtypes = [P(ip)] * 3 + [ip] + [P(ip)] * 6
    L.mhdvlct_flux_correct.argtypes = [vp, P(MhdBlockView), ip, P(MhdFluxCorrection),
                                       P(MhdRefreshFace), ip, ctypes.c_uint, vp]
    L.mhdvlct_batch_create.argtypes = [vp, P(ip), P(dp), ip, ip, ip, P(vp)]
    L.mhdvlct_batch_create_ex.argtypes = [vp, P(ip), P(dp), ip, ip, ip, ip, ip, P(vp)]
    L.mhdvlct_batch_destroy.argtypes = [vp]
    L.mhdvlct_batch_block_view.argtypes = [vp, ip, P(MhdBlockView)]
    L.mhdvlct_batch_set_neighbors.argtypes = [vp, P(ip)]
    L.mhdvlct_batch_refresh.argtypes = [vp, vp]
    L.mhdvlct_batch_set_refresh_faces.argtypes = [vp, P(MhdRefreshFace), ip, ctypes.c_uint]
    L.mhdvlct_batch_set_flux_correction.argtypes = [vp, ctypes.c_uint, P(MhdRefreshFace), ip,
                                                    ctypes.c_uint]
    L.mhdvlct_batch_step.argtypes = [vp, P(dp), vp]
    L.mhdvlct_batch_timestep.argtypes = [vp, P(dp), vp]
    L.mhdvlct_batch_run.argtypes = [vp, ip, ip, P(dp), vp]
    L.mhdvlct_batch_set_tile.argtypes = [vp, ip, ip]
    L.mhdvlct_batch_autotune.argtypes = [vp, ip, ctypes.c_char_p, ctypes.c_size_t, vp]
    L.mhdvlct_batch_state_region.argtypes = [vp, P(vp), P(ctypes.c_size_t)]
    L.mhdvlct_batch_profile.argtypes = [vp, ip, ip, P(ctypes.c_float), vp]
    L.mhdvlct_batch_set_stage_tile.argtypes = [vp, ip, ip, ip, ip, ip]
    L.mhdvlct_batch_diagnostics.argtypes = [vp, P(dp), vp]
    L.mhdvlct_batch_state_segments.argtypes = [vp, P(vp), P(ctypes.c_size_t), ip, P(ip)]
    L.mhdvlct_batch_run_host.argtypes = [vp, vp, ctypes.c_size_t, ip, ip, P(dp), vp]
    L.mhdserve_create.argtypes = [P(MhdVlctParams), ctypes.c_size_t, ip, P(vp)]
    L.mhdserve_destroy.argtypes = [vp]
    L.mhdserve_submit.argtypes = [vp, P(MhdServeRequest), P(ip)]
    L.mhdserve_pump.argtypes = [vp, ip]
    L.mhdserve_poll.argtypes = [vp, ip, P(ip)]
    L.mhdserve_result.argtypes = [vp, ip, P(ctypes.c_void_p), P(dp)]
    L.mhdserve_timing.argtypes = [vp, ip, P(dp), P(dp), P(dp)]
    L.mhdserve_last_error_string.argtypes = [vp]
    L.mhdserve_last_error_string.restype = ctypes.c_char_p
    _lib = L
    return L


class MhdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def check(rc: int, handle=None, what: str = "") -> None:
    if rc != MHD_OK:
        msg = ""
        if handle is not None:
            msg = lib().mhdvlct_last_error_string(handle).decode()
        raise MhdError(rc, f"{what}: {msg}")
