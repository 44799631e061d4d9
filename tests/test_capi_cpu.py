"""CPU-side checks of the C ABI library: it loads, exports every symbol the
header declares, and its parameter handling mirrors the reference."""
import ctypes
import os
import re

import pytest

from mhdvlct import capi, block as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_symbols_exported():
    L = capi.lib()
    hdr = open(os.path.join(ROOT, "include", "mhdvlct_gb300.h")).read()
    decl = set(re.findall(r"\b((?:mhdvlct|mhdserve)_[a-z_]+)\s*\(", hdr))
    assert decl == set(capi.EXPORTED)
    for name in decl:
        assert hasattr(L, name), name


def test_params_defaults_and_parse():
    p = B.parse_params('''
      Method { mhd_vlct { mhd_choice = "constrained_transport";
                          riemann_solver = "hlle"; theta_limiter = 2.;
                          courant = 0.4; }; }
      Physics { fluid_props { eos { gamma = 1.4; }
                floors { density = 1e-20; pressure = 1e-21; }
                dual_energy { type = "modern"; eta = 0.01; } } }
    ''')
    assert p.mhd_choice == b"constrained_transport"
    assert p.riemann_solver == b"hlle"
    assert p.reconstruct_method == b"plm"
    assert p.theta_limiter == 2.0 and p.courant == 0.4 and p.gamma == 1.4
    assert p.density_floor == 1e-20 and p.pressure_floor == 1e-21
    assert p.dual_energy == 1 and p.dual_energy_eta == 0.01


def test_removed_parameters_rejected():
    with pytest.raises(capi.MhdError):
        B.parse_params('Method { mhd_vlct { half_dt_reconstruct_method = "nn"; }; }')


@pytest.mark.parametrize("kw,ok", [
    (dict(mhd_choice="constrained_transport", riemann_solver="hlld"), True),
    (dict(mhd_choice="no_bfield", riemann_solver="hllc"), True),
    (dict(mhd_choice="constrained_transport", riemann_solver="hlle"), True),
    (dict(mhd_choice="constrained_transport", riemann_solver="hllc"), False),
    (dict(mhd_choice="no_bfield", riemann_solver="hlld"), False),
    (dict(mhd_choice="no_bfield", riemann_solver="hlle"), False),
    (dict(mhd_choice="constrained_transport", riemann_solver="hll"), False),
    (dict(mhd_choice="", riemann_solver="hlld"), False),
    (dict(theta_limiter=2.5), False),
    (dict(reconstruct_method="weno"), False),
    (dict(density_floor=0.0), False),
    # EnzoBfieldMethod.cpp:23-27: constrained transport needs the vl scheme
    (dict(mhd_choice="constrained_transport", time_scheme="euler"), False),
    (dict(mhd_choice="no_bfield", riemann_solver="hllc", time_scheme="euler"), True),
])
def test_create_validation(kw, ok):
    if ok:
        m = B.EnzoMethodMHDVlct(**kw)
        assert m.name() == "mhd_vlct"
        # vl: NN (1) + PLM (2); euler: one PLM stage (2)
        assert m.required_ghost_depth() == (2 if kw.get("time_scheme") == "euler" else 3)
    else:
        with pytest.raises(capi.MhdError):
            B.EnzoMethodMHDVlct(**kw)


def test_default_courant_follows_time_scheme():
    assert B.EnzoMethodMHDVlct().courant == 0.3
    assert B.EnzoMethodMHDVlct(time_scheme="euler", mhd_choice="no_bfield",
                               riemann_solver="hllc",
                               reconstruct_method="nn").courant == 1.0
