"""CPU oracle of EAM's P3 driver micro_p3_tend around p3_main -- TEST
INFRASTRUCTURE ONLY.

A NumPy restatement, column-vectorised and level by level where the driver
loops over levels, of components/eam/src/physics/p3/scream/
micro_p3_interface.F90: the preparation of the P3 inputs (:982-1047), its
get_cloud_fraction (:661-732) and the use of the P3 results (:1182-1431).
Fields are (ncol, nlev) arrays, level 0 at the model top; zi, flxprc and
flxsnw have nlev+1 interfaces.  The nine constituents are in the driver's
order: qv, cldliq, numliq, rain, numrain, cldice, numice, cldrim, rimvol.

EAM's constants (share/util/shr_const_mod.F90:21-49 through
components/eam/src/control/physconst.F90:38-86): R_dry = N_A k_B / M_dry,
cp_dry = 1004.64, g = 9.80616; the driver's literal 287.15 in the in-cloud
number concentrations is kept.  micro_p3_utils.F90:55 (mincld) and
micro_p3_interface.F90:873-875 (dcon, mucon, deicon).

Parity status: the driver is Fortran and gfortran is absent, so this
restatement is pinned by a literal scalar transcription of its cloud-fraction
loops (tests) and by the identities its outputs satisfy, not by the driver's
own output.
"""
from __future__ import annotations

from typing import Dict

import numpy as np

RGAS = 6.02214e26 * 1.38065e-23
RAIR = RGAS / 28.966
CPAIR = 1.00464e3
GRAVIT = 9.80616
MINCLD = 0.0001
QSMALL = 1.0e-14
MUCON, DCON, DEICON = 5.3, 25.e-6, 50.0
MAX_OVERLAP, IN_CLOUD = 0, 1
SPECIES = ("qv", "cldliq", "numliq", "rain", "numrain", "cldice", "numice", "cldrim", "rimvol")
# the P3 prognostic field holding each constituent
P3_NAME = {"qv": "qv", "cldliq": "qc", "numliq": "nc", "rain": "qr", "numrain": "nr", "cldice": "qi",
           "numice": "ni", "cldrim": "qm", "rimvol": "bm"}


def get_cloud_fraction(ast, qc, qr, qi, method):
    """get_cloud_fraction (micro_p3_interface.F90:661-732) with dry qc, qr, qi:
    floors at mincld, then the rain fraction down the column, level by level
    (each level reads the level above as already updated)."""
    cldm = np.maximum(ast, MINCLD)
    cld_i = cldm.copy()
    cld_l = cldm.copy()
    cld_r = cldm.copy()
    nlev = ast.shape[1]
    for k in range(1, nlev):
        if method == IN_CLOUD:
            cond = (qc[:, k] < QSMALL) & (qi[:, k] < QSMALL)
        else:
            cond = (qr[:, k - 1] >= QSMALL) | (qi[:, k - 1] >= QSMALL)
        cld_r[:, k] = np.where(cond, np.maximum(cld_r[:, k - 1], cld_r[:, k]), cld_r[:, k])
    return cld_i, cld_l, cld_r


def eam_pre(e: Dict[str, np.ndarray], subgrid: bool = True, method: int = MAX_OVERLAP) -> Dict[str, np.ndarray]:
    """P3 inputs from the EAM state (micro_p3_interface.F90:982-1047)."""
    ratio = e["pdel"] / e["pdeldry"]
    out = {}
    for s in SPECIES:
        out[P3_NAME[s]] = e[s] * ratio
    out["qv_prev"] = e["qv_prev"] * ratio
    inv_exner = 1.0 / np.power(e["pmid"] * 1.e-5, RAIR * (1.0 / CPAIR))
    out["inv_exner"] = inv_exner
    out["dz"] = e["zi"][:, :-1] - e["zi"][:, 1:]
    out["th"] = e["t"] * inv_exner
    out["pres"] = e["pmiddry"].copy()
    out["dpres"] = e["pdeldry"].copy()
    if subgrid:
        ci, cl, cr = get_cloud_fraction(e["ast"], out["qc"], out["qr"], out["qi"], method)
    else:
        ci = np.ones_like(e["ast"])
        cl = np.ones_like(e["ast"])
        cr = np.ones_like(e["ast"])
    out["cld_frac_i"], out["cld_frac_l"], out["cld_frac_r"] = ci, cl, cr
    out["nc_nuceat_tend"] = e["npccn"].copy()
    out["ni_activated"] = e["ni_activated"].copy()
    out["inv_qc_relvar"] = e["relvar"].copy()
    out["t_prev"] = e["t_prev"].copy()
    return out


def eam_post(e: Dict[str, np.ndarray], p3: Dict[str, np.ndarray], dt: float) -> Dict[str, np.ndarray]:
    """The driver's use of the P3 results (micro_p3_interface.F90:1182-1431).
    `p3` holds the P3 state after the step, its inputs (inv_exner and the
    cloud fractions) and outputs."""
    ratio = e["pdeldry"] / e["pdel"]
    w = {s: p3[P3_NAME[s]] * ratio for s in SPECIES}
    t = e["t"]
    dtemp = p3["th"] / p3["inv_exner"] - t
    dtemp = dtemp * ratio
    temp = dtemp + t
    out = {"ptend_s": CPAIR * (temp - t) / dt}
    for s in SPECIES:
        out["ptend_" + s] = (np.maximum(0.0, w[s]) - e[s]) / dt
    out["t_prev"] = temp
    out["qv_prev"] = w["qv"]
    out["qme"] = e["cmeliq"] + p3["qv2qi_depos_tend"]
    out["vap_liq_exchange"] = p3["vap_liq_exchange"] + e["cmeliq"]
    liq, ice = p3["precip_liq_surf"], p3["precip_ice_surf"]
    out["prec_pcw"] = liq + ice
    out["prec_str"] = out["prec_pcw"] + 0.0
    out["snow_pcw"] = ice.copy()
    out["snow_str"] = ice + 0.0
    pmid = e["pmid"]
    out["rho"] = pmid / (RAIR * temp)
    cl, ci, cr = p3["cld_frac_l"], p3["cld_frac_i"], p3["cld_frac_r"]
    out["icimrst"] = np.minimum(e["cldice"] / np.maximum(MINCLD, ci), 0.005)
    out["icwmrst"] = np.minimum(e["cldliq"] / np.maximum(MINCLD, cl), 0.005)
    out["icinc"] = e["numice"] / np.maximum(MINCLD, ci) * pmid / (287.15 * t)
    out["icwnc"] = e["numliq"] / np.maximum(MINCLD, cl) * pmid / (287.15 * t)
    rel = p3["diag_eff_radius_qc"] * 1e6
    rei = p3["diag_eff_radius_qi"] * 1e6
    dei = rei * 2.0
    low = e["ast"] < 1.e-4
    out["rel"], out["rei"] = rel, rei
    out["dei"] = np.where(low, DEICON, dei)
    out["mu"] = np.where(low, MUCON, 0.0)
    out["lambdac"] = np.where(low, (MUCON + 1.0) / DCON, 0.0)
    tot = w["rain"] + w["cldice"] + w["cldliq"]
    with np.errstate(divide="ignore", invalid="ignore"):
        out["nfice"] = np.where((w["cldice"] > QSMALL) & (tot > QSMALL), np.minimum(w["cldice"] / tot, 1.0), 0.0)
    out["cdnumc"] = np.sum(w["numliq"] * e["pdel"] / GRAVIT, axis=1)
    liqc = (cl > 0.01) & (out["icwmrst"] > 5.e-5)
    icec = (ci > 0.01) & (out["icimrst"] > 1.e-6)
    out["efcout"] = np.where(liqc, rel * cl, 0.0)
    out["ncout"] = np.where(liqc, out["icwnc"] * cl, 0.0)
    out["freql"] = np.where(liqc, cl, 0.0)
    out["efiout"] = np.where(icec, rei * ci, 0.0)
    out["niout"] = np.where(icec, out["icinc"] * ci, 0.0)
    out["freqi"] = np.where(icec, ci, 0.0)
    reff = p3["diag_eff_radius_qr"]
    out["deff_rain"] = reff * 2.0 * 1.e6
    rain = w["rain"] >= 1.e-7
    out["aqrain"] = np.where(rain, w["rain"] * cr, 0.0)
    out["anrain"] = np.where(rain, w["numrain"] * cr, 0.0)
    out["freqr"] = np.where(rain, cr, 0.0)
    out["reff_rain"] = np.where(rain, reff * 1.e6, reff)
    out["flxprc"] = p3["precip_liq_flux"] + p3["precip_ice_flux"]
    out["flxsnw"] = p3["precip_ice_flux"].copy()
    return out


def eam_state_from_p3_inputs(inp: Dict[str, np.ndarray], seed: int = 7) -> Dict[str, np.ndarray]:
    """An EAM physics state whose driver-prepared P3 inputs are close to the
    given P3 inputs (for tests): wet mixing ratios from the dry ones with
    pdel = pdeldry (1 + qv), pmid and pmiddry from the P3 pressure, T from th,
    interface heights from dz, ast from the liquid cloud fraction."""
    rng = np.random.default_rng(seed)
    ncol, nlev = inp["qc"].shape
    pdeldry = inp["dpres"].copy()
    qv = inp["qv"]
    pdel = pdeldry * (1.0 + qv)
    to_wet = pdeldry / pdel
    e = {}
    for s in SPECIES:
        e[s] = inp[P3_NAME[s]] * to_wet
    e["pdel"], e["pdeldry"] = pdel, pdeldry
    e["pmiddry"] = inp["pres"].copy()
    e["pmid"] = inp["pres"] * (1.0 + 0.6 * qv)
    e["t"] = inp["th"] / inp["inv_exner"]
    zi = np.zeros((ncol, nlev + 1))
    zi[:, :-1] = np.cumsum(inp["dz"][:, ::-1], axis=1)[:, ::-1]
    e["zi"] = zi
    ast = np.clip(inp["cld_frac_l"] * rng.uniform(0.2, 1.0, size=(ncol, nlev)), 0.0, 1.0)
    ast[rng.uniform(size=(ncol, nlev)) < 0.1] = 0.0
    e["ast"] = ast
    e["npccn"] = inp["nc_nuceat_tend"].copy()
    e["ni_activated"] = inp["ni_activated"].copy()
    e["relvar"] = inp["inv_qc_relvar"].copy()
    e["cmeliq"] = rng.normal(0.0, 1e-8, size=(ncol, nlev))
    e["t_prev"] = e["t"] + rng.normal(0.0, 0.3, size=(ncol, nlev))
    e["qv_prev"] = e["qv"] * (1.0 + rng.normal(0.0, 1e-3, size=(ncol, nlev)))
    return e
