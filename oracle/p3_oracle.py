"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/, by __graft_entry__.smoke() as the checker, and by bench.py's
CPU-baseline leg.  The product library never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict

import numpy as np

from . import build as _build

FIELDS_PROG = ["qc", "nc", "qr", "nr", "qi", "qm", "ni", "bm", "qv", "th"]
FIELDS_DIN = ["nc_nuceat_tend", "nccn", "ni_activated", "inv_qc_relvar", "cld_frac_i", "cld_frac_l",
              "cld_frac_r", "pres", "dz", "dpres", "inv_exner", "qv_prev", "t_prev"]
FIELDS_DOUT = ["qv2qi_depos_tend", "precip_liq_surf", "precip_ice_surf", "diag_eff_radius_qc",
               "diag_eff_radius_qi", "diag_eff_radius_qr", "rho_qi", "precip_liq_flux", "precip_ice_flux",
               "precip_total_tend", "nevapr"]
FIELDS_HIST = ["liq_ice_exchange", "vap_liq_exchange", "vap_ice_exchange"]
ALL = FIELDS_PROG + FIELDS_DIN + FIELDS_DOUT + FIELDS_HIST
RUNTIME = ["max_total_ni", "autoconversion_prefactor", "autoconversion_qc_exponent",
           "autoconversion_nc_exponent", "autoconversion_radius", "accretion_prefactor",
           "accretion_qc_exponent", "accretion_qr_exponent", "rain_selfcollection_prefactor",
           "rain_selfcollection_breakup_diameter", "constant_mu_rain", "spa_ccn_to_nc_factor",
           "cldliq_to_ice_collection_factor", "rain_to_ice_collection_factor", "min_rime_rho",
           "max_rime_rho", "immersion_freezing_exponent", "deposition_nucleation_exponent",
           "ice_sedimentation_factor"]


class Runtime(C.Structure):
    _fields_ = [(n, C.c_double) for n in RUNTIME] + [("do_ice_production", C.c_int32), ("pad_", C.c_int32)]


class Tables(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ["ice", "collect", "vn", "vm", "revap", "mu_r", "dnu"]]


class Fields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ALL]


class Call(C.Structure):
    _fields_ = [("ncol", C.c_int32), ("nlev", C.c_int32), ("ld", C.c_int64), ("ld_int", C.c_int64),
                ("dt", C.c_double), ("it", C.c_int32), ("predictNc", C.c_int32),
                ("prescribedCCN", C.c_int32), ("nthreads", C.c_int32)]


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(_build.build()))
        dp = C.POINTER(C.c_double)
        lib.p3o_runtime_defaults.argtypes = [C.POINTER(Runtime)]
        lib.p3o_main.argtypes = [C.POINTER(Call), C.POINTER(Runtime), C.POINTER(Tables), C.POINTER(Fields), dp]
        lib.p3o_main.restype = C.c_int
        lib.p3o_main_part12.argtypes = [C.POINTER(Call), C.POINTER(Runtime), C.POINTER(Tables), C.POINTER(Fields),
                                        dp, C.POINTER(C.c_int32)]
        lib.p3o_main_part12.restype = C.c_int
        lib.p3o_main_sed_part3.argtypes = [C.POINTER(Call), C.POINTER(Runtime), C.POINTER(Tables),
                                           C.POINTER(Fields), dp, C.POINTER(C.c_int32)]
        lib.p3o_main_sed_part3.restype = C.c_int
        lib.p3o_calc_first_order_upwind_step.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                                         dp, dp, dp, C.c_int, C.POINTER(dp),
                                                         C.POINTER(dp), C.POINTER(dp)]
        lib.p3o_find_top.argtypes = [dp, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]
        lib.p3o_find_top.restype = C.c_int
        lib.p3o_find_bottom.argtypes = [dp, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]
        lib.p3o_find_bottom.restype = C.c_int
        lib.p3o_table3_lookup_apply.argtypes = [C.POINTER(Tables), C.c_int, C.c_int, dp, dp, dp]
        lib.p3o_cloud_water_conservation.argtypes = [C.c_double, C.c_double, dp]
        lib.p3o_rain_water_conservation.argtypes = [C.c_double, C.c_double, dp]
        lib.p3o_ice_water_conservation.argtypes = [C.c_double, C.c_double, dp]
        lib.p3o_qv_sat_dry.argtypes = [C.c_double, C.c_double, C.c_int]
        lib.p3o_qv_sat_dry.restype = C.c_double
        _lib = lib
    return _lib


def default_runtime() -> Runtime:
    rt = Runtime()
    load().p3o_runtime_defaults(C.byref(rt))
    return rt


def make_tables(tab: Dict[str, np.ndarray]):
    """Keeps contiguous float64 copies alive together with the struct."""
    keep = {k: np.ascontiguousarray(tab[k], dtype=np.float64) for k in ["ice", "collect", "vn", "vm",
                                                                         "revap", "mu_r", "dnu"]}
    t = Tables(*[keep[k].ctypes.data for k in ["ice", "collect", "vn", "vm", "revap", "mu_r", "dnu"]])
    return t, keep


def empty_outputs(ncol: int, nlev: int) -> Dict[str, np.ndarray]:
    out = {}
    for n in FIELDS_DOUT + FIELDS_HIST:
        if n in ("precip_liq_surf", "precip_ice_surf"):
            out[n] = np.zeros(ncol)
        elif n in ("precip_liq_flux", "precip_ice_flux"):
            out[n] = np.zeros((ncol, nlev + 1))
        else:
            out[n] = np.zeros((ncol, nlev))
    return out


def p3_main(state: Dict[str, np.ndarray], tables: Dict[str, np.ndarray], dt: float, runtime: Runtime = None,
            predictNc=True, prescribedCCN=True, it=1, nthreads=0):
    """One oracle step in place on ``state`` (a dict of every field, float64,
    (ncol, nlev) / (ncol,) / (ncol, nlev+1)).  Returns (error bits, microseconds)."""
    lib = load()
    ncol, nlev = state["qc"].shape
    for n in ALL:
        a = state[n]
        assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], n
    f = Fields(*[state[n].ctypes.data for n in ALL])
    t, keep = make_tables(tables)
    rt = runtime if runtime is not None else default_runtime()
    call = Call(ncol, nlev, nlev, nlev + 1, dt, it, int(predictNc), int(prescribedCCN),
                int(nthreads or os.cpu_count() or 1))
    us = C.c_double(0)
    err = lib.p3o_main(C.byref(call), C.byref(rt), C.byref(t), C.byref(f), C.byref(us))
    del keep
    return err, us.value


HANDOVER_ROWS = ["T_atm", "rho", "rhofacr", "rhofaci", "acn"]


def _stage_args(state, tables, dt, runtime, predictNc, prescribedCCN, it, nthreads):
    ncol, nlev = state["qc"].shape
    for n in ALL:
        a = state[n]
        assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], n
    f = Fields(*[state[n].ctypes.data for n in ALL])
    t, keep = make_tables(tables)
    rt = runtime if runtime is not None else default_runtime()
    call = Call(ncol, nlev, nlev, nlev + 1, dt, it, int(predictNc), int(prescribedCCN),
                int(nthreads or os.cpu_count() or 1))
    return f, t, keep, rt, call


def p3_main_part12(state, tables, dt, runtime=None, predictNc=True, prescribedCCN=True, it=1, nthreads=0):
    """p3_main_init + part1 + part2 in place on ``state``.  Returns (error bits,
    hand-over (5, ncol, nlev) float64 in HANDOVER_ROWS order, cflag (ncol,)
    int32: 1 where the column goes on to sedimentation and part3)."""
    lib = load()
    ncol, nlev = state["qc"].shape
    f, t, keep, rt, call = _stage_args(state, tables, dt, runtime, predictNc, prescribedCCN, it, nthreads)
    ho = np.zeros((len(HANDOVER_ROWS), ncol, nlev))
    cflag = np.zeros(ncol, dtype=np.int32)
    err = lib.p3o_main_part12(C.byref(call), C.byref(rt), C.byref(t), C.byref(f),
                              ho.ctypes.data_as(C.POINTER(C.c_double)), cflag.ctypes.data_as(C.POINTER(C.c_int32)))
    del keep
    return err, ho, cflag


def p3_main_sed_part3(state, tables, dt, handover, cflag, runtime=None, predictNc=True, prescribedCCN=True, it=1,
                      nthreads=0):
    """Sedimentation + homogeneous freezing + part3 in place on ``state`` for
    the columns with cflag = 1, from ``handover`` ((5, ncol, nlev),
    HANDOVER_ROWS order).  Returns the error bits."""
    lib = load()
    f, t, keep, rt, call = _stage_args(state, tables, dt, runtime, predictNc, prescribedCCN, it, nthreads)
    ho = np.ascontiguousarray(handover, dtype=np.float64)
    cf = np.ascontiguousarray(cflag, dtype=np.int32)
    err = lib.p3o_main_sed_part3(C.byref(call), C.byref(rt), C.byref(t), C.byref(f),
                                 ho.ctypes.data_as(C.POINTER(C.c_double)), cf.ctypes.data_as(C.POINTER(C.c_int32)))
    del keep
    return err
