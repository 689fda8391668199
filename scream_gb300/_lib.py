"""ctypes bindings of libp3x (include/p3x.h).

The library is the product: every compute entry point runs CUDA kernels.
Loading fails loudly when the shared library has not been built.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libp3x.so"

P3X_OK = 0
P3X_EINVAL = -1
P3X_ENOMEM = -2
P3X_ENUMERIC = -3
P3X_ETIMEOUT = -4
P3X_ECUDA = -5
P3X_ETABLE = -6
P3X_ERANGE = -7
P3X_CHECK_OFF = 0
P3X_CHECK_RECORD = 1
P3X_CHECK_FAIL = 2
P3X_FP64 = 0
P3X_FP32_BULK = 1
P3X_STAGE_PART12 = 1
P3X_STAGE_SED = 2
P3X_STAGE_PART3 = 4

STATUS_NAMES = {0: "P3X_OK", -1: "P3X_EINVAL", -2: "P3X_ENOMEM", -3: "P3X_ENUMERIC",
                -4: "P3X_ETIMEOUT", -5: "P3X_ECUDA", -6: "P3X_ETABLE", -7: "P3X_ERANGE"}

# field order of the 23 inputs (P3X_F_*)
INPUT_FIELDS = ["qc", "nc", "qr", "nr", "qi", "qm", "ni", "bm", "qv", "th",
                "nc_nuceat_tend", "nccn", "ni_activated", "inv_qc_relvar", "cld_frac_i",
                "cld_frac_l", "cld_frac_r", "pres", "dz", "dpres", "inv_exner", "qv_prev", "t_prev"]
PROG_FIELDS = INPUT_FIELDS[:10]
DIAG_IN_FIELDS = INPUT_FIELDS[10:]
DIAG_OUT_FIELDS = ["qv2qi_depos_tend", "precip_liq_surf", "precip_ice_surf", "diag_eff_radius_qc",
                   "diag_eff_radius_qi", "diag_eff_radius_qr", "rho_qi", "precip_liq_flux",
                   "precip_ice_flux", "precip_total_tend", "nevapr"]
HIST_FIELDS = ["liq_ice_exchange", "vap_liq_exchange", "vap_ice_exchange"]
SURFACE_FIELDS = ["precip_liq_surf", "precip_ice_surf"]
INTERFACE_FIELDS = ["precip_liq_flux", "precip_ice_flux"]
OUTPUT_FIELDS = DIAG_OUT_FIELDS + HIST_FIELDS
ALL_FIELDS = INPUT_FIELDS + OUTPUT_FIELDS

RUNTIME_FIELDS = [
    "max_total_ni", "autoconversion_prefactor", "autoconversion_qc_exponent",
    "autoconversion_nc_exponent", "autoconversion_radius", "accretion_prefactor",
    "accretion_qc_exponent", "accretion_qr_exponent", "rain_selfcollection_prefactor",
    "rain_selfcollection_breakup_diameter", "constant_mu_rain", "spa_ccn_to_nc_factor",
    "cldliq_to_ice_collection_factor", "rain_to_ice_collection_factor", "min_rime_rho",
    "max_rime_rho", "immersion_freezing_exponent", "deposition_nucleation_exponent",
    "ice_sedimentation_factor"]

_dp = C.POINTER(C.c_double)


class Runtime(C.Structure):
    _fields_ = [(n, C.c_double) for n in RUNTIME_FIELDS] + [("do_ice_production", C.c_int32),
                                                            ("pad_", C.c_int32)]


class PrognosticState(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in PROG_FIELDS]


class DiagnosticInputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in DIAG_IN_FIELDS]


class DiagnosticOutputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in DIAG_OUT_FIELDS]


class Infrastructure(C.Structure):
    _fields_ = [("dt", C.c_double), ("it", C.c_int32), ("its", C.c_int32), ("ite", C.c_int32),
                ("kts", C.c_int32), ("kte", C.c_int32), ("predictNc", C.c_int32),
                ("prescribedCCN", C.c_int32), ("col_location", C.c_void_p)]


class HistoryOnly(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in HIST_FIELDS]


class Layout(C.Structure):
    _fields_ = [("ld", C.c_int64), ("ld_int", C.c_int64)]


HOST_MODEL_FIELDS = ["pmid", "pseudo_density", "pseudo_density_dry", "cld_frac_t", "T_atm", "T_prev",
                    "precip_liq_surf_mass", "precip_ice_surf_mass", "vapor_flux", "water_flux", "ice_flux",
                    "heat_flux"]


class InterfaceFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in HOST_MODEL_FIELDS]


# EAM driver (micro_p3_tend) fields, in the order of p3x_eam_fields
EAM_SPECIES = ["qv", "cldliq", "numliq", "rain", "numrain", "cldice", "numice", "cldrim", "rimvol"]
EAM_STATE = ["pmid", "pmiddry", "pdel", "pdeldry", "zi", "t"]
EAM_PBUF_IN = ["ast", "npccn", "ni_activated", "relvar", "cmeliq"]
EAM_DIAG = ["qme", "rho", "icimrst", "icwmrst", "icinc", "icwnc", "rel", "rei", "dei", "mu", "lambdac", "nfice",
            "efcout", "ncout", "freql", "efiout", "niout", "freqi", "aqrain", "anrain", "freqr", "reff_rain",
            "deff_rain", "flxprc", "flxsnw", "prec_pcw", "snow_pcw", "prec_str", "snow_str", "cdnumc"]
PRECIP_FRAC_MAX_OVERLAP, PRECIP_FRAC_IN_CLOUD = 0, 1


class EamFields(C.Structure):
    _fields_ = ([(n, C.c_void_p) for n in EAM_STATE] + [("q", C.c_void_p * 9)] +
                [(n, C.c_void_p) for n in EAM_PBUF_IN] + [("t_prev", C.c_void_p), ("qv_prev", C.c_void_p),
                                                         ("ptend_s", C.c_void_p), ("ptend_q", C.c_void_p * 9)] +
                [(n, C.c_void_p) for n in EAM_DIAG] + [("subgrid_clouds", C.c_int32),
                                                      ("precip_frac_method", C.c_int32)])


class LaunchConfig(C.Structure):
    _fields_ = [("lanes_per_column", C.c_int32), ("columns_per_block", C.c_int32),
                ("table_staging", C.c_int32), ("blocks_per_sm", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class InstanceDesc(C.Structure):
    _fields_ = [("prog", PrognosticState), ("din", DiagnosticInputs), ("dout", DiagnosticOutputs),
                ("hist", HistoryOnly), ("layout", Layout), ("ncol", C.c_int32), ("nlev", C.c_int32),
                ("dt", C.c_double), ("it", C.c_int32), ("predictNc", C.c_int32),
                ("prescribedCCN", C.c_int32), ("precision", C.c_int32)]


class CheckReport(C.Structure):
    _fields_ = [("t_out_of_range", C.c_int64), ("qv_out_of_range", C.c_int64),
                ("t_first_instance", C.c_int32), ("t_first_column", C.c_int32), ("t_first_level", C.c_int32),
                ("qv_first_instance", C.c_int32), ("qv_first_column", C.c_int32), ("qv_first_level", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


CONS_FIELDS = ["pseudo_density", "T_mid", "qv", "qc", "qi", "qr", "horiz_winds", "ps", "phis", "vapor_flux",
               "water_flux", "ice_flux", "heat_flux"]


class ConservationFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in CONS_FIELDS]


class ConservationReport(C.Structure):
    _fields_ = [("max_mass_err", C.c_double), ("max_energy_err", C.c_double), ("mass_col", C.c_int32),
                ("energy_col", C.c_int32), ("pass_", C.c_int32), ("pad_", C.c_int32)]

    def as_dict(self):
        return {"max_mass_err": self.max_mass_err, "mass_col": self.mass_col,
                "max_energy_err": self.max_energy_err, "energy_col": self.energy_col, "pass": bool(self.pass_)}


SIZE_CLASSES = ["1-9", "10-99", "100-999", "1000-9999", "10000-65536"]


class ServeStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("rejected", C.c_int64), ("p50_ms", C.c_double),
                ("p90_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double),
                ("mean_ms", C.c_double), ("wall_s", C.c_double),
                ("column_levels_per_s", C.c_double), ("offered_rate_hz", C.c_double),
                ("peak_bytes", C.c_int64), ("peak_inflight", C.c_int32), ("pad_", C.c_int32),
                ("class_count", C.c_int64 * 5), ("class_p50_ms", C.c_double * 5),
                ("class_p99_ms", C.c_double * 5), ("slowdown_p50", C.c_double), ("slowdown_p99", C.c_double),
                ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64)]

    def as_dict(self):
        d = {}
        for k, _ in self._fields_:
            if k == "pad_":
                continue
            v = getattr(self, k)
            d[k] = list(v) if k.startswith("class_") else v
        d["by_size_class"] = {c: {"count": d["class_count"][i], "p50_ms": d["class_p50_ms"][i],
                                  "p99_ms": d["class_p99_ms"][i]} for i, c in enumerate(SIZE_CLASSES)}
        for k in ("class_count", "class_p50_ms", "class_p99_ms"):
            del d[k]
        return d


# name -> (restype, argtypes)
_V = C.c_void_p
_I = C.c_int32
PROTOTYPES = {
    "p3x_version": (C.c_char_p, []),
    "p3x_runtime_defaults": (None, [C.POINTER(Runtime)]),
    "p3x_context_create": (C.c_int, [C.c_char_p, C.POINTER(_V), C.POINTER(C.c_int)]),
    "p3x_context_destroy": (C.c_int, [_V]),
    "p3x_context_get_tables": (C.c_int, [_V, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "p3x_write_ice_table": (C.c_int, [C.c_char_p, C.c_char_p]),
    "p3x_tables_generate": (C.c_int, [C.c_char_p, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "p3x_saturation_table": (C.c_int, [_dp, C.POINTER(C.c_int32), _dp, _dp]),
    "p3x_set_kernel_timing": (C.c_int, [_V, _I]),
    "p3x_selftest": (C.c_int, [C.POINTER(C.c_uint64)]),
    "p3x_kernel_times": (C.c_int, [_V, C.POINTER(C.c_float)]),
    "p3x_main": (C.c_int, [_V, C.POINTER(Runtime), C.POINTER(PrognosticState),
                           C.POINTER(DiagnosticInputs), C.POINTER(DiagnosticOutputs),
                           C.POINTER(Infrastructure), C.POINTER(HistoryOnly), _I, _I,
                           C.POINTER(Layout), _I, _V, C.POINTER(C.c_double)]),
    "p3x_main_host": (C.c_int, [_V, C.POINTER(Runtime), C.POINTER(PrognosticState),
                                C.POINTER(DiagnosticInputs), C.POINTER(DiagnosticOutputs),
                                C.POINTER(Infrastructure), C.POINTER(HistoryOnly), _I, _I,
                                C.POINTER(Layout), _I, _I, C.POINTER(C.c_double)]),
    "p3x_eam_tend_pre": (C.c_int, [C.POINTER(EamFields), C.POINTER(PrognosticState),
                                   C.POINTER(DiagnosticInputs), _I, _I, C.POINTER(Layout), _V]),
    "p3x_eam_tend_post": (C.c_int, [C.POINTER(EamFields), C.POINTER(PrognosticState),
                                    C.POINTER(DiagnosticInputs), C.POINTER(DiagnosticOutputs),
                                    C.POINTER(HistoryOnly), _I, _I, C.POINTER(Layout), C.c_double, _V]),
    "p3x_eam_micro_p3_tend": (C.c_int, [_V, C.POINTER(Runtime), C.POINTER(EamFields), C.POINTER(PrognosticState),
                                        C.POINTER(DiagnosticInputs), C.POINTER(DiagnosticOutputs),
                                        C.POINTER(Infrastructure), C.POINTER(HistoryOnly), _I, _I,
                                        C.POINTER(Layout), _I, _V]),
    "p3x_main_async": (C.c_int, [_V, C.POINTER(Runtime), C.POINTER(PrognosticState),
                                 C.POINTER(DiagnosticInputs), C.POINTER(DiagnosticOutputs),
                                 C.POINTER(Infrastructure), C.POINTER(HistoryOnly), _I, _I,
                                 C.POINTER(Layout), _I, _V]),
    "p3x_main_fixed_scratch": (C.c_int, [_V, C.POINTER(Runtime), C.POINTER(PrognosticState),
                                 C.POINTER(DiagnosticInputs), C.POINTER(DiagnosticOutputs),
                                 C.POINTER(Infrastructure), C.POINTER(HistoryOnly), _I, _I,
                                 C.POINTER(Layout), _I, _V]),
    "p3x_context_check": (C.c_int, [_V, _V]),
    "p3x_set_launch_config": (C.c_int, [_V, _I, C.POINTER(LaunchConfig)]),
    "p3x_get_launch_config": (C.c_int, [_V, _I, C.POINTER(LaunchConfig)]),
    "p3x_init": (C.c_int, [C.c_char_p, C.POINTER(C.c_int)]),
    "p3x_finalize": (C.c_int, []),
    "p3x_main_f": (C.c_int, [_dp] * 6 + [C.c_double] + [_dp] * 10 + [_I, _dp, _dp, _I, _I, _I, _I]
                   + [_dp] * 4 + [C.c_bool, C.c_bool] + [_dp] * 13 + [_dp]),
    "p3x_fixed_scratch_info": (C.c_int, [_V, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "p3x_handover_bytes": (C.c_int, [_I, C.c_int64, C.POINTER(C.c_int64)]),
    "p3x_set_check_values": (C.c_int, [_V, _I]),
    "p3x_check_values_report": (C.c_int, [_V, _V, C.POINTER(CheckReport)]),
    "p3x_main_stages": (C.c_int, [_V, C.POINTER(Runtime), C.POINTER(PrognosticState),
                                  C.POINTER(DiagnosticInputs), C.POINTER(DiagnosticOutputs),
                                  C.POINTER(Infrastructure), C.POINTER(HistoryOnly), _I, _I,
                                  C.POINTER(Layout), _I, _I, _V, _V]),
    "p3x_batch_create": (C.c_int, [_V, C.POINTER(Runtime), C.POINTER(InstanceDesc), _I, C.POINTER(_V)]),
    "p3x_batch_run": (C.c_int, [_V, _V]),
    "p3x_batch_capture_graph": (C.c_int, [_V, _V]),
    "p3x_batch_set_launch_config": (C.c_int, [_V, C.POINTER(LaunchConfig)]),
    "p3x_batch_destroy": (C.c_int, [_V]),
    "p3x_autotune_batch": (C.c_int, [_V, _V, _I, C.POINTER(LaunchConfig), C.POINTER(C.c_double)]),
    "p3x_workload_generate": (C.c_int, [_I, C.c_uint64, _I, _I, _I, C.POINTER(_V), C.c_int64]),
    "p3x_column_mass_energy": (C.c_int, [C.POINTER(ConservationFields), _I, _I, C.c_int64, _V, _V, _V]),
    "p3x_conservation_check": (C.c_int, [_V, C.POINTER(ConservationFields), _V, _V, _I, _I, C.c_int64,
                                         C.c_double, C.c_double, C.c_double, _V, _V,
                                         C.POINTER(ConservationReport), _V]),
    "p3x_column_budgets": (C.c_int, [C.POINTER(PrognosticState), _V, _V, _I, _I, C.c_int64, _V, _V, _V]),
    "p3x_preamble": (C.c_int, [C.POINTER(InterfaceFields), C.POINTER(PrognosticState),
                               C.POINTER(DiagnosticInputs), _I, _I, C.POINTER(Layout), _V]),
    "p3x_postamble": (C.c_int, [C.POINTER(InterfaceFields), C.POINTER(PrognosticState),
                                C.POINTER(DiagnosticInputs), C.POINTER(DiagnosticOutputs), _I, _I,
                                C.POINTER(Layout), C.c_double, _V]),
    "p3x_server_create": (C.c_int, [_V, C.POINTER(Runtime), C.c_int64, _I, C.POINTER(_V)]),
    "p3x_server_destroy": (C.c_int, [_V]),
    "p3x_server_submit": (C.c_int, [_V, C.c_int64, _I, _I, _I, _I, C.c_uint64, C.c_double, C.c_double]),
    "p3x_server_run_poisson": (C.c_int, [_V, C.c_double, _I, _I, C.c_uint64, C.POINTER(ServeStats)]),
    "p3x_server_read_field": (C.c_int, [_V, C.c_int64, _I, _dp, C.c_int64]),
    "p3x_server_drain": (C.c_int, [_V, C.POINTER(ServeStats)]),
    "p3x_server_calibrate": (C.c_int, [_V]),
    "p3x_server_set_latency_policy": (C.c_int, [_V, _I, C.c_double]),
    "p3x_server_set_sm_partition": (C.c_int, [_V, _I, C.c_int64, C.POINTER(C.c_int32)]),
    "p3x_server_set_dispatch_chunk": (C.c_int, [_V, C.c_int64]),
    "p3x_server_isolated_ms": (C.c_int, [_V, _I, _I, _I, _dp]),
    "p3x_server_export_instance": (C.c_int, [_V, C.c_int64, _dp, C.c_int64]),
    "p3x_server_import_instance": (C.c_int, [_V, C.c_int64, _I, _I, _I, C.c_double, _dp, C.c_int64]),
}

_lib = None


def load() -> C.CDLL:
    """Loads libp3x.so (built in-tree by scream_gb300.build); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: run scream_gb300.build.build() first "
                           "(there is no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class P3Error(RuntimeError):
    def __init__(self, fn: str, code: int):
        super().__init__(f"{fn} returned {STATUS_NAMES.get(code, code)}")
        self.code = code


def check(fn: str, code: int) -> int:
    if code != P3X_OK:
        raise P3Error(fn, code)
    return code


TABLE_SHAPES = {"ice": (5, 4, 50, 12), "collect": (5, 4, 50, 30, 2), "vn": (300, 10),
                "vm": (300, 10), "revap": (300, 10), "mu_r": (150,), "dnu": (16,)}


def host_tables(table_file=None):
    """P3LookupTables built on the host (no GPU), as numpy arrays."""
    import numpy as np
    out = {k: np.zeros(s) for k, s in TABLE_SHAPES.items()}
    args = [out[k].ctypes.data_as(_dp) for k in TABLE_SHAPES]
    check("p3x_tables_generate",
          load().p3x_tables_generate(table_file.encode() if table_file else None, *args))
    return out


def default_runtime() -> Runtime:
    rt = Runtime()
    load().p3x_runtime_defaults(C.byref(rt))
    return rt
