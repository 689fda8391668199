"""P3Microphysics pre/postamble (p3x_preamble / p3x_postamble) against a
NumPy restatement of the reference's formulas
(physics/p3/eamxx_p3_process_interface.hpp:63-269 and
share/util/scream_common_physics_functions_impl.hpp:88-426)."""
import ctypes as C

import numpy as np
import pytest

RD, G, EP2, P0, CP = 287.042, 9.80616, 18.016 / 28.966, 100000.0, 1004.64
SPECIES = ["qc", "nc", "qr", "nr", "qi", "ni", "qm", "bm", "qv"]


def np_preamble(h, s):
    out = {k: v.copy() for k, v in s.items()}
    c1 = -1.0 + 1.0 / EP2
    out["dz"] = (RD / G) * h["pseudo_density"] * (h["T_atm"] * (1.0 + c1 * s["qv"])) / h["pmid"]
    for n in SPECIES + ["qv_prev"]:
        out[n] = s[n] * h["pseudo_density"] / h["pseudo_density_dry"]
    exner = (h["pmid"] / P0) ** (RD * (1.0 / CP))
    out["inv_exner"] = 1.0 / exner
    out["th"] = h["T_atm"] / exner
    cl = np.maximum(h["cld_frac_t"], 1e-4)
    out["cld_frac_l"] = cl
    out["cld_frac_i"] = cl.copy()
    cr = cl.copy()
    cr[:, 1:] = np.where(h["cld_frac_t"][:, :-1] > cr[:, 1:], h["cld_frac_t"][:, :-1], cr[:, 1:])
    out["cld_frac_r"] = cr
    return out


def np_postamble(h, s, dt):
    hh = {k: v.copy() for k, v in h.items()}
    out = {k: v.copy() for k, v in s.items()}
    exner = (h["pmid"] / P0) ** (RD * (1.0 / CP))
    T = (s["th"] * exner - h["T_atm"]) * h["pseudo_density_dry"] / h["pseudo_density"]
    T = T + h["T_atm"]
    hh["T_atm"], hh["T_prev"] = T, T.copy()
    for n in SPECIES:
        out[n] = s[n] * h["pseudo_density_dry"] / h["pseudo_density"]
    out["qv_prev"] = out["qv"].copy()
    for n in ["diag_eff_radius_qc", "diag_eff_radius_qi", "diag_eff_radius_qr"]:
        out[n] = s[n] * 1e6
    liq, ice = s["precip_liq_surf"], s["precip_ice_surf"]
    hh["precip_liq_surf_mass"] = h["precip_liq_surf_mass"] + liq * 1000.0 * dt
    hh["precip_ice_surf_mass"] = h["precip_ice_surf_mass"] + ice * 1000.0 * dt
    hh["vapor_flux"] = np.zeros_like(liq)
    hh["water_flux"] = liq + ice
    hh["ice_flux"] = ice.copy()
    hh["heat_flux"] = np.zeros_like(liq)
    return hh, out


def test_interface_rejects_bad_arguments(built):
    from scream_gb300 import _lib as L
    lib = L.load()
    f = L.InterfaceFields()
    prog, din, dout = L.PrognosticState(), L.DiagnosticInputs(), L.DiagnosticOutputs()
    assert lib.p3x_preamble(None, C.byref(prog), C.byref(din), 4, 8, None, None) == L.P3X_EINVAL
    assert lib.p3x_preamble(C.byref(f), C.byref(prog), C.byref(din), 4, 8, None, None) == L.P3X_EINVAL
    assert lib.p3x_postamble(C.byref(f), C.byref(prog), C.byref(din), C.byref(dout), 4, 8, None, 0.0,
                             None) == L.P3X_EINVAL


def _host_state(ncol, nlev, seed):
    import scream_gb300 as p3
    inp = p3.generate_inputs(0, seed, ncol, nlev)
    rng = np.random.default_rng(seed)
    pdd = inp["dpres"]
    h = {"pmid": inp["pres"], "pseudo_density_dry": pdd, "pseudo_density": pdd * (1.0 + inp["qv"]),
         "cld_frac_t": rng.uniform(0.0, 1.0, (ncol, nlev)) * (rng.random((ncol, nlev)) < 0.6),
         "T_atm": inp["th"] / inp["inv_exner"], "T_prev": np.zeros((ncol, nlev)),
         "precip_liq_surf_mass": rng.uniform(0, 1, ncol), "precip_ice_surf_mass": rng.uniform(0, 1, ncol),
         "vapor_flux": np.full(ncol, 7.0), "water_flux": np.zeros(ncol), "ice_flux": np.zeros(ncol),
         "heat_flux": np.full(ncol, 7.0)}
    return inp, h


@pytest.mark.gpu
def test_preamble_and_postamble_match_numpy(gpu_ctx):
    import torch
    import scream_gb300 as p3
    ncol, nlev, dt = 300, 72, 300.0
    inp, h = _host_state(ncol, nlev, 2024)
    f = p3.P3Fields.from_inputs(inp)
    hd = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in h.items()}
    gpu_ctx.preamble(hd, f)
    torch.cuda.synchronize()
    got = f.to_host()
    exp = np_preamble(h, {k: v.copy() for k, v in inp.items()})
    for n in SPECIES + ["qv_prev", "dz", "inv_exner", "th", "cld_frac_l", "cld_frac_i", "cld_frac_r"]:
        np.testing.assert_allclose(got[n], exp[n], rtol=1e-15, atol=0, err_msg=n)

    # postamble on a state with outputs (one P3 step in between)
    gpu_ctx.p3_main(f, dt, p3.P3X_FP64)
    s = f.to_host()
    hh_exp, out_exp = np_postamble(h, s, dt)
    gpu_ctx.postamble(hd, f, dt)
    torch.cuda.synchronize()
    got = f.to_host()
    for n in SPECIES + ["qv_prev", "diag_eff_radius_qc", "diag_eff_radius_qi", "diag_eff_radius_qr"]:
        np.testing.assert_allclose(got[n], out_exp[n], rtol=1e-15, atol=0, err_msg=n)
    for n in ["T_atm", "T_prev", "precip_liq_surf_mass", "precip_ice_surf_mass", "vapor_flux", "water_flux",
              "ice_flux", "heat_flux"]:
        np.testing.assert_allclose(hd[n].cpu().numpy(), hh_exp[n], rtol=1e-15, atol=0, err_msg=n)


@pytest.mark.gpu
def test_preamble_then_postamble_restores_the_wet_state(gpu_ctx):
    import torch
    import scream_gb300 as p3
    ncol, nlev = 128, 128
    inp, h = _host_state(ncol, nlev, 77)
    f = p3.P3Fields.from_inputs(inp)
    hd = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in h.items()}
    gpu_ctx.preamble(hd, f)
    gpu_ctx.postamble(hd, f, 300.0)
    torch.cuda.synchronize()
    got = f.to_host()
    for n in SPECIES:
        np.testing.assert_allclose(got[n], inp[n], rtol=1e-15, atol=0, err_msg=n)
    np.testing.assert_allclose(hd["T_atm"].cpu().numpy(), h["T_atm"], rtol=1e-15, err_msg="T_atm")


def np_mass_energy(h, s, winds=None, ps=None, phis=None):
    """compute_total_mass_on_column / compute_total_energy_on_column
    (mass_and_energy_column_conservation_check.cpp:281-347)."""
    LV, LF = 2501000.0, 333700.0
    pd = h["pseudo_density"]
    m = ((s["qv"] + s["qc"] + s["qi"] + s["qr"]) * pd / G).sum(axis=1)
    ke = 0.0 if winds is None else 0.5 * (winds[:, 0] ** 2 + winds[:, 1] ** 2)
    e = ((h["T_atm"] * CP + ke + (LV + LF) * s["qv"] + LF * (s["qc"] + s["qr"])) * pd / G).sum(axis=1)
    if ps is not None:
        e = e + phis * ps / G
    return m, e


def _cons_fields(hd, f, extra=None):
    d = {"pseudo_density": hd["pseudo_density"], "T_mid": hd["T_atm"], "qv": f.t["qv"], "qc": f.t["qc"],
         "qi": f.t["qi"], "qr": f.t["qr"], "vapor_flux": hd["vapor_flux"], "water_flux": hd["water_flux"],
         "ice_flux": hd["ice_flux"], "heat_flux": hd["heat_flux"]}
    d.update(extra or {})
    return d


@pytest.mark.gpu
def test_conservation_totals_and_maxloc_match_numpy(gpu_ctx):
    """Column totals (with winds and surface geopotential), relative errors
    against planted fluxes, and the largest error's column."""
    import torch
    import scream_gb300 as p3
    ncol, nlev, dt = 257, 72, 300.0
    inp, h = _host_state(ncol, nlev, 5)
    rng = np.random.default_rng(5)
    winds = rng.normal(0, 10, (ncol, 2, nlev))
    ps, phis = rng.uniform(9e4, 1.02e5, ncol), rng.uniform(0, 3e4, ncol)
    # boundary fluxes of realistic size (kg/m2/s and m/s), so the planted
    # errors below are the largest
    h["vapor_flux"] = rng.uniform(0, 1e-5, ncol)
    h["water_flux"] = rng.uniform(0, 1e-7, ncol)
    h["ice_flux"] = 0.3 * h["water_flux"]
    h["heat_flux"] = rng.uniform(-1.0, 1.0, ncol)
    f = p3.P3Fields.from_inputs(inp)
    hd = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in h.items()}
    extra = {"horiz_winds": torch.from_numpy(winds).cuda(), "ps": torch.from_numpy(ps).cuda(),
             "phis": torch.from_numpy(phis).cuda()}
    m, e = gpu_ctx.column_mass_energy(_cons_fields(hd, f, extra))
    m_np, e_np = np_mass_energy(h, inp, winds, ps, phis)
    np.testing.assert_allclose(m.cpu().numpy(), m_np, rtol=1e-13)
    np.testing.assert_allclose(e.cpu().numpy(), e_np, rtol=1e-13)
    m0 = m_np * (1 + rng.uniform(-1e-9, 1e-9, ncol))
    e0 = e_np * (1 + rng.uniform(-1e-9, 1e-9, ncol))
    m0[101] *= 1 + 0.05   # the largest mass error, far above the flux terms
    e0[17] *= 1 - 0.05    # the largest energy error
    rep, me, ee = gpu_ctx.conservation_check(_cons_fields(hd, f, extra), torch.from_numpy(m0).cuda(),
                                            torch.from_numpy(e0).cuda(), dt, mass_tol=1e-6, energy_tol=1e-6)
    LV, LF = 2501000.0, 333700.0
    m_exp = m0 + (h["vapor_flux"] - h["water_flux"] * 1000.0) * dt
    e_exp = e0 + (h["vapor_flux"] * (LV + LF) - (h["water_flux"] - h["ice_flux"]) * 1000.0 * LF
                  + h["heat_flux"]) * dt
    np.testing.assert_allclose(me.cpu().numpy(), np.abs(m_np - m_exp) / m0, rtol=1e-6, atol=1e-15)
    np.testing.assert_allclose(ee.cpu().numpy(), np.abs(e_np - e_exp) / e0, rtol=1e-6, atol=1e-15)
    me_np, ee_np = np.abs(m_np - m_exp) / m0, np.abs(e_np - e_exp) / e0
    assert rep["mass_col"] == int(np.argmax(me_np)) == 101
    assert rep["energy_col"] == int(np.argmax(ee_np)) == 17
    assert rep["max_mass_err"] == float(me.max()) and not rep["pass"]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_process_step_passes_mass_conservation_check(gpu_ctx, precision):
    """preamble -> p3_main -> postamble (run_impl), then the check with the
    boundary fluxes the postamble set: column mass closes to round-off
    (the reference driver's default mass tolerance is 1e-10)."""
    import torch
    import scream_gb300 as p3
    ncol, nlev, dt = 512, 128, 300.0
    inp, h = _host_state(ncol, nlev, 11)
    f = p3.P3Fields.from_inputs(inp)
    hd = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in h.items()}
    m0, e0 = gpu_ctx.column_mass_energy(_cons_fields(hd, f))
    gpu_ctx.preamble(hd, f)
    gpu_ctx.p3_main(f, dt, precision)
    gpu_ctx.postamble(hd, f, dt)
    rep, me, ee = gpu_ctx.conservation_check(_cons_fields(hd, f), m0, e0, dt)
    print("conservation check after one process step, precision", precision, rep)
    assert rep["max_mass_err"] <= 1e-12, rep
    # the energy (cp T + (Lv+Lf) qv + Lf (qc+qr)) closes too in both forms: the
    # FP32-bulk form heats from the same FP64 condensate changes as the vapour
    assert rep["max_energy_err"] <= 1e-13, rep
