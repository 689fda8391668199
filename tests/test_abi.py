"""CPU checks of the C ABI: the library loads, exports every function that
include/p3x.h declares, and rejects bad arguments before touching a GPU."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "p3x.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(p3x_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(built):
    from scream_gb300 import _lib as L
    out = subprocess.run(["nm", "-D", "--defined-only", str(L.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (p3x_[a-z0-9_]+)\b", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert hasattr(built, n)


def test_python_prototypes_cover_header(built):
    from scream_gb300 import _lib as L
    missing = [n for n in declared_functions() if n not in L.PROTOTYPES and n != "p3x_incomplete_gamma_q"]
    assert not missing, missing


def test_runtime_defaults_match_reference(built):
    """P3Runtime defaults, components/eamxx/src/physics/p3/p3_functions.hpp:114-133."""
    from scream_gb300 import _lib as L
    rt = L.default_runtime()
    expect = dict(max_total_ni=740.0e3, autoconversion_prefactor=1350.0, autoconversion_qc_exponent=2.47,
                  autoconversion_nc_exponent=1.79, autoconversion_radius=25.0e-6, accretion_prefactor=67.0,
                  accretion_qc_exponent=1.15, accretion_qr_exponent=1.15, rain_selfcollection_prefactor=5.78,
                  rain_selfcollection_breakup_diameter=0.00028, constant_mu_rain=1.0, spa_ccn_to_nc_factor=1.0,
                  cldliq_to_ice_collection_factor=0.5, rain_to_ice_collection_factor=1.0, min_rime_rho=50.0,
                  max_rime_rho=900.0, immersion_freezing_exponent=0.65, deposition_nucleation_exponent=0.304,
                  ice_sedimentation_factor=1.0)
    for k, v in expect.items():
        assert getattr(rt, k) == v, k
    assert rt.do_ice_production == 1


def test_struct_layouts_match_header(built):
    from scream_gb300 import _lib as L
    assert C.sizeof(L.Runtime) == 19 * 8 + 8
    assert C.sizeof(L.PrognosticState) == 10 * 8
    assert C.sizeof(L.DiagnosticInputs) == 13 * 8
    assert C.sizeof(L.DiagnosticOutputs) == 11 * 8
    assert C.sizeof(L.HistoryOnly) == 3 * 8
    assert C.sizeof(L.Infrastructure) == 8 + 7 * 4 + 4 + 8
    # p3x_eam_fields: 62 pointers (state 6, q 9, pbuf 5, t_prev/qv_prev, ptend 10, diagnostics 30), 2 int32
    assert C.sizeof(L.EamFields) == 62 * 8 + 8
    assert L.EamFields.ptend_q.offset == 23 * 8
    assert L.EamFields.subgrid_clouds.offset == 62 * 8


def test_invalid_arguments_rejected_without_gpu(built):
    from scream_gb300 import _lib as L
    lib = built
    rt = L.default_runtime()
    prog, din, dout, hist = L.PrognosticState(), L.DiagnosticInputs(), L.DiagnosticOutputs(), L.HistoryOnly()
    infra = L.Infrastructure(300.0, 1, 1, 1, 1, 1, 1, 1, None)
    lay = L.Layout(0, 0)
    # null context
    assert lib.p3x_main(None, C.byref(rt), C.byref(prog), C.byref(din), C.byref(dout), C.byref(infra),
                        C.byref(hist), 1, 1, C.byref(lay), 0, None, None) == L.P3X_EINVAL
    assert lib.p3x_main_async(None, C.byref(rt), C.byref(prog), C.byref(din), C.byref(dout), C.byref(infra),
                              C.byref(hist), 1, 1, C.byref(lay), 0, None) == L.P3X_EINVAL
    assert lib.p3x_context_destroy(None) == L.P3X_EINVAL
    assert lib.p3x_batch_run(None, None) == L.P3X_EINVAL
    assert lib.p3x_batch_destroy(None) == L.P3X_EINVAL
    assert lib.p3x_server_destroy(None) == L.P3X_EINVAL
    assert lib.p3x_server_set_sm_partition(None, 8, 1 << 15, None) == L.P3X_EINVAL
    assert lib.p3x_server_set_dispatch_chunk(None, 1 << 18) == L.P3X_EINVAL
    # EAM driver: missing fields and a bad precipitation-fraction method
    e = L.EamFields()
    assert lib.p3x_eam_tend_pre(C.byref(e), C.byref(prog), C.byref(din), 1, 1, C.byref(lay), None) == L.P3X_EINVAL
    assert lib.p3x_eam_tend_post(C.byref(e), C.byref(prog), C.byref(din), C.byref(dout), C.byref(hist), 1, 1,
                                 C.byref(lay), 300.0, None) == L.P3X_EINVAL
    assert lib.p3x_eam_micro_p3_tend(None, C.byref(rt), C.byref(e), C.byref(prog), C.byref(din), C.byref(dout),
                                     C.byref(infra), C.byref(hist), 1, 1, C.byref(lay), 0, None) == L.P3X_EINVAL
    # workload generator argument checks (host only)
    arr = (C.c_void_p * 23)()
    assert lib.p3x_workload_generate(0, 1, 0, 4, 10, arr, 10) == L.P3X_EINVAL  # null fields
    bufs = [np.zeros((4, 10)) for _ in range(23)]
    arr = (C.c_void_p * 23)(*[b.ctypes.data for b in bufs])
    assert lib.p3x_workload_generate(0, 1, 0, 4, 10, arr, 5) == L.P3X_EINVAL   # ld < nlev
    assert lib.p3x_workload_generate(7, 1, 0, 4, 10, arr, 10) == L.P3X_EINVAL  # unknown kind
    assert lib.p3x_workload_generate(2, 1, 0, 4, 10, arr, 10) == L.P3X_EINVAL  # mixed IC needs >= 36 levels
    assert lib.p3x_workload_generate(0, 1, 0, 4, 10, arr, 10) == L.P3X_OK
    assert lib.p3x_version().decode().startswith("p3x")
