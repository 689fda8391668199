"""EAM's P3 driver micro_p3_tend (components/eam/src/physics/p3/scream/
micro_p3_interface.F90:661-1431) around the step: the CPU restatement
against a literal transcription of the driver's cloud-fraction loops and
against the identities of a step that changes nothing, then the device
kernels against the restatement, and the device driver end to end against
the restatement around the CPU oracle's p3_main."""
import numpy as np
import pytest

from conftest import oracle_state, rel_l2

NCOL, NLEV, DT = 384, 72, 300.0


def literal_cloud_fraction(ast, qc, qr, qi, method):
    """get_cloud_fraction as written (micro_p3_interface.F90:676-727), one
    column and one level at a time, k = 1 the model top (Fortran index)."""
    from oracle import eam_driver as E
    ncol, nlev = ast.shape
    ci = np.empty_like(ast)
    cl = np.empty_like(ast)
    cr = np.empty_like(ast)
    ktop, kbot, kdir = 1, nlev, -1
    for i in range(ncol):
        cldm = [0.0] * (nlev + 1)
        for k in range(kbot, ktop - 1, kdir):
            cldm[k] = max(ast[i, k - 1], E.MINCLD)
            ci[i, k - 1] = max(ast[i, k - 1], E.MINCLD)
            cl[i, k - 1] = max(ast[i, k - 1], E.MINCLD)
            cr[i, k - 1] = cldm[k]
        for k in range(ktop - kdir, kbot + 1, -kdir):
            if method == E.IN_CLOUD:
                if qc[i, k - 1] < E.QSMALL and qi[i, k - 1] < E.QSMALL:
                    cr[i, k - 1] = max(cr[i, k - 2], cr[i, k - 1])
            else:
                if qr[i, k - 2] >= E.QSMALL or qi[i, k - 2] >= E.QSMALL:
                    cr[i, k - 1] = max(cr[i, k - 2], cr[i, k - 1])
    return ci, cl, cr


@pytest.mark.parametrize("method", [0, 1])
def test_cloud_fraction_restatement_matches_literal_loops(method):
    from oracle import eam_driver as E
    rng = np.random.default_rng(11 + method)
    ncol, nlev = 40, 30
    ast = rng.uniform(0, 1, (ncol, nlev))
    ast[rng.uniform(size=ast.shape) < 0.3] = 0.0
    ast[rng.uniform(size=ast.shape) < 0.05] = E.MINCLD
    def q():
        x = 10.0 ** rng.uniform(-18, -3, (ncol, nlev))
        x[rng.uniform(size=x.shape) < 0.4] = 0.0
        x[rng.uniform(size=x.shape) < 0.05] = E.QSMALL
        return x
    qc, qr, qi = q(), q(), q()
    got = E.get_cloud_fraction(ast, qc, qr, qi, method)
    want = literal_cloud_fraction(ast, qc, qr, qi, method)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)


def eam_case(seed=1003):
    from oracle import eam_driver as E
    from scream_gb300.p3 import generate_inputs
    inp = generate_inputs(0, seed, NCOL, NLEV)
    return inp, E.eam_state_from_p3_inputs(inp, seed)


def test_pre_then_post_of_an_unchanged_state_gives_zero_tendencies(built):
    """A step that changes nothing: the post's tendencies vanish to round-off
    and t_prev returns the state temperature (the driver's conversions are
    each other's inverses)."""
    from oracle import eam_driver as E
    inp, e = eam_case()
    p3 = E.eam_pre(e)
    ncol, nlev = inp["qc"].shape
    for n in ("qv2qi_depos_tend", "diag_eff_radius_qc", "diag_eff_radius_qi", "diag_eff_radius_qr",
              "vap_liq_exchange"):
        p3[n] = np.zeros((ncol, nlev))
    for n in ("precip_liq_surf", "precip_ice_surf"):
        p3[n] = np.zeros(ncol)
    for n in ("precip_liq_flux", "precip_ice_flux"):
        p3[n] = np.zeros((ncol, nlev + 1))
    out = E.eam_post(e, p3, DT)
    np.testing.assert_allclose(out["t_prev"], e["t"], rtol=1e-14)
    assert np.max(np.abs(out["ptend_s"])) <= 1e-12 * E.CPAIR * np.max(e["t"]) / DT * 10
    for s in E.SPECIES:
        scale = max(np.max(np.abs(e[s])), 1e-300)
        assert np.max(np.abs(out["ptend_" + s])) * DT <= 4e-16 * scale, s


def _device_state(e, torch):
    return {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in e.items()}


def _alloc_outputs(eam, ncol, nlev, torch):
    from scream_gb300 import _lib as L
    for s in L.EAM_SPECIES:
        eam["ptend_" + s] = torch.zeros(ncol, nlev, dtype=torch.float64, device="cuda")
    eam["ptend_s"] = torch.zeros(ncol, nlev, dtype=torch.float64, device="cuda")
    for n in L.EAM_DIAG:
        if n in ("flxprc", "flxsnw"):
            eam[n] = torch.zeros(ncol, nlev + 1, dtype=torch.float64, device="cuda")
        elif n in ("prec_pcw", "snow_pcw", "prec_str", "snow_str", "cdnumc"):
            eam[n] = torch.zeros(ncol, dtype=torch.float64, device="cuda")
        else:
            eam[n] = torch.zeros(ncol, nlev, dtype=torch.float64, device="cuda")


@pytest.mark.gpu
@pytest.mark.parametrize("subgrid,method", [(True, 0), (True, 1), (False, 0)])
def test_device_pre_matches_restatement(gpu_ctx, subgrid, method):
    import torch
    import scream_gb300 as p3
    from oracle import eam_driver as E
    inp, e = eam_case()
    want = E.eam_pre(e, subgrid, method)
    f = p3.P3Fields.from_inputs(inp)
    eam = _device_state(e, torch)
    gpu_ctx.eam_tend_pre(eam, f, subgrid, method)
    h = f.to_host()
    exact = ["qv", "qc", "nc", "qr", "nr", "qi", "ni", "qm", "bm", "qv_prev", "dz", "pres", "dpres",
             "cld_frac_l", "cld_frac_i", "cld_frac_r", "nc_nuceat_tend", "ni_activated", "inv_qc_relvar", "t_prev"]
    for n in exact:
        np.testing.assert_array_equal(h[n], want[n], err_msg=n)
    # inv_exner and th go through pow: the device's and the host's agree to an ulp or two
    for n in ("inv_exner", "th"):
        np.testing.assert_allclose(h[n], want[n], rtol=5e-16, atol=0, err_msg=n)
    # the rain fraction's recurrence does act on this workload
    if subgrid:
        assert np.any(h["cld_frac_r"] > h["cld_frac_l"])


@pytest.mark.gpu
def test_device_post_matches_restatement(gpu_ctx):
    import torch
    import scream_gb300 as p3
    from oracle import eam_driver as E
    inp, e = eam_case(1004)
    f = p3.P3Fields.from_inputs(inp)
    eam = _device_state(e, torch)
    _alloc_outputs(eam, NCOL, NLEV, torch)
    gpu_ctx.eam_tend_pre(eam, f)
    gpu_ctx.p3_main(f, DT, prescribedCCN=False)
    after = f.to_host()
    t_prev_in, qv_prev_in = eam["t_prev"].clone(), eam["qv_prev"].clone()
    gpu_ctx.eam_tend_post(eam, f, DT)
    torch.cuda.synchronize()
    e_in = dict(e)
    e_in["t_prev"], e_in["qv_prev"] = t_prev_in.cpu().numpy(), qv_prev_in.cpu().numpy()
    want = E.eam_post(e_in, after, DT)
    got = {k: v.cpu().numpy() for k, v in eam.items()}
    got["vap_liq_exchange"] = f.t["vap_liq_exchange"].cpu().numpy()
    for n, w in want.items():
        g = got[n]
        if n == "cdnumc":  # a warp sum on the device, a sequential one here
            np.testing.assert_allclose(g, w, rtol=1e-14, err_msg=n)
        elif n == "rho":
            np.testing.assert_allclose(g, w, rtol=4e-16, err_msg=n)
        else:
            np.testing.assert_array_equal(g, w, err_msg=n)


@pytest.mark.gpu
def test_device_driver_end_to_end(gpu_ctx, tables):
    """p3x_eam_micro_p3_tend equals its three parts run one by one, bit for
    bit, and the restatement around the CPU oracle's p3_main on the
    well-conditioned outputs (temperature and vapour/liquid tendencies,
    surface precipitation)."""
    import torch
    import scream_gb300 as p3
    from oracle import eam_driver as E
    from oracle import p3_oracle as O
    inp, e = eam_case(1005)
    # one call
    f1 = p3.P3Fields.from_inputs(inp)
    eam1 = _device_state(e, torch)
    _alloc_outputs(eam1, NCOL, NLEV, torch)
    gpu_ctx.eam_micro_p3_tend(eam1, f1, DT, prescribedCCN=False)
    torch.cuda.synchronize()
    # three calls
    f2 = p3.P3Fields.from_inputs(inp)
    eam2 = _device_state(e, torch)
    _alloc_outputs(eam2, NCOL, NLEV, torch)
    gpu_ctx.eam_tend_pre(eam2, f2)
    gpu_ctx.p3_main(f2, DT, prescribedCCN=False)
    gpu_ctx.eam_tend_post(eam2, f2, DT)
    torch.cuda.synchronize()
    for n in eam1:
        assert torch.equal(eam1[n], eam2[n]), n
    # the restatement around the oracle
    pre = E.eam_pre(e)
    st = oracle_state(inp)
    for n, v in pre.items():
        st[n] = v
    assert O.p3_main(st, tables, DT, prescribedCCN=False)[0] == 0
    want = E.eam_post(e, st, DT)
    got = {k: v.cpu().numpy() for k, v in eam1.items()}
    for n in ("ptend_s", "ptend_qv", "ptend_cldliq", "ptend_rain", "t_prev", "qv_prev"):
        r = rel_l2(got[n], want[n])
        assert r <= 1e-9, (n, r)
    r = rel_l2(got["prec_pcw"] - got["snow_pcw"], want["prec_pcw"] - want["snow_pcw"])
    assert r <= 1e-9, ("liquid surface precipitation", r)


@pytest.mark.gpu
def test_device_driver_rejects_before_touching_the_state(gpu_ctx):
    """An invalid step argument (precision, dt, leading dimension) fails the
    whole call before the preparation converts the state in place."""
    import torch
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    inp, e = eam_case(1007)
    f = p3.P3Fields.from_inputs(inp)
    eam = _device_state(e, torch)
    _alloc_outputs(eam, NCOL, NLEV, torch)
    before = {k: v.clone() for k, v in eam.items()}
    before_p3 = {k: v.clone() for k, v in f.t.items()}
    for kw in ({"precision": 7}, {"dt": 0.0}):
        args = {"dt": DT, **kw}
        with pytest.raises(L.P3Error, match="p3x_eam_micro_p3_tend") as err:
            gpu_ctx.eam_micro_p3_tend(eam, f, args.pop("dt"), **args)
        assert err.value.code == L.P3X_EINVAL
    torch.cuda.synchronize()
    for k in eam:
        assert torch.equal(eam[k], before[k]), k
    for k in f.t:
        assert torch.equal(f.t[k], before_p3[k]), k


@pytest.mark.gpu
def test_device_driver_fp32_bulk(gpu_ctx, tables):
    """The driver around the FP32-bulk step: the temperature, vapour and
    liquid tendencies and the liquid surface precipitation stay within the
    FP32-bulk form's one-step tolerance of the FP64 oracle chain (1e-4), and
    the driver's own kernels add nothing to that (its FP64 step agrees to 1e-9
    in the test above)."""
    import torch
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    from oracle import eam_driver as E
    from oracle import p3_oracle as O
    inp, e = eam_case(1006)
    f = p3.P3Fields.from_inputs(inp)
    eam = _device_state(e, torch)
    _alloc_outputs(eam, NCOL, NLEV, torch)
    gpu_ctx.eam_micro_p3_tend(eam, f, DT, precision=L.P3X_FP32_BULK, prescribedCCN=False)
    torch.cuda.synchronize()
    pre = E.eam_pre(e)
    st = oracle_state(inp)
    for n, v in pre.items():
        st[n] = v
    assert O.p3_main(st, tables, DT, prescribedCCN=False)[0] == 0
    want = E.eam_post(e, st, DT)
    got = {k: v.cpu().numpy() for k, v in eam.items()}
    for n in ("ptend_s", "ptend_qv", "ptend_cldliq", "ptend_rain", "t_prev", "qv_prev"):
        r = rel_l2(got[n], want[n])
        assert r <= 1e-4, (n, r)
    r = rel_l2(got["prec_pcw"] - got["snow_pcw"], want["prec_pcw"] - want["snow_pcw"])
    assert r <= 1e-4, ("liquid surface precipitation", r)
