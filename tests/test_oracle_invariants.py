"""CPU checks of the oracle against the reference's own invariant / known-answer tests.

Ports the intent of components/eamxx/src/physics/p3/tests:
  p3_upwind_unit_tests.cpp:26-200   upwind mass conservation + no new extrema
  p3_table3_unit_tests.cpp:23-170   Table3 interpolant is C0 (slope growth < 1.1)
  p3_unit_tests.cpp:27-131          conservation limiters scale sinks to the source
  p3_find_unit_tests.cpp            find_top / find_bottom
plus full-step invariants: column water conservation and the reference's
"mixed" initial condition (p3_ic_cases.cpp) run for 6 steps like p3_run_and_cmp.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import column_water, oracle_state

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def O(built):
    from oracle import p3_oracle
    return p3_oracle


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _extrema(r, eps):
    """True mixing ratio r[1]/r[0] extrema as the reference gathers them
    (p3_upwind_unit_tests.cpp:116-146): the maximum skips cells whose
    background r[0] fell below 1 (eps*r0 < eps), the minimum takes all."""
    with np.errstate(divide="ignore", invalid="ignore"):
        mr = r[1] / r[0]
    ok = r[0] * eps >= eps
    rmax = np.max(mr[ok]) if np.any(ok) else -np.inf
    rmin = np.nanmin(mr) if np.any(np.isfinite(mr)) else np.inf
    return rmin, rmax


@pytest.mark.parametrize("nk", [17, 32, 77, 128])
@pytest.mark.parametrize("kdir", [-1, 1])
def test_upwind_conserves_mass_and_extrema(O, nk, kdir):
    """p3_upwind_unit_tests.cpp:44-196 setup and checks (10 eps)."""
    lib = O.load()
    eps = np.finfo(float).eps
    max_speed, min_dz = 4.2, 0.33
    dt = min_dz / max_speed
    k = np.arange(nk, dtype=float)
    rho = 1 + k / nk
    inv_rho = 1 / rho
    inv_dz = 1 / (min_dz + k * k / (nk * nk))
    V = [0.5 * (1 + k / nk) * max_speed for _ in range(2)]
    r0 = np.ones(nk)
    r1 = np.where((k >= 2) & (k < nk - 2), k / nk, 0.0)
    r = [r0, r1]
    flux = [np.zeros(nk), np.zeros(nk)]
    kmin, kmax = 0, nk - 1
    k_bot = kmin if kdir == 1 else kmax
    k_top = kmax if kdir == 1 else kmin
    dp3 = C.POINTER(C.c_double) * 2
    for step in range(2 * nk):
        mass0 = np.sum(rho * r[1] / inv_dz)
        rmin0, rmax0 = _extrema(r, eps)
        if step == 0:
            for f, (kb, kt) in enumerate([(k_bot, k_top), (k_bot + kdir, k_top - kdir)]):
                lib.p3o_calc_first_order_upwind_step(nk, kb, kt, kdir, dt, _dp(rho), _dp(inv_rho), _dp(inv_dz), 1,
                                                     (C.POINTER(C.c_double) * 1)(_dp(flux[f])),
                                                     (C.POINTER(C.c_double) * 1)(_dp(V[f])),
                                                     (C.POINTER(C.c_double) * 1)(_dp(r[f])))
        else:
            lib.p3o_calc_first_order_upwind_step(nk, k_bot, k_top, kdir, dt, _dp(rho), _dp(inv_rho), _dp(inv_dz), 2,
                                                 dp3(_dp(flux[0]), _dp(flux[1])), dp3(_dp(V[0]), _dp(V[1])),
                                                 dp3(_dp(r[0]), _dp(r[1])))
        mass1 = np.sum(rho * r[1] / inv_dz)
        if step > 1:
            mass1 += flux[1][0 if kdir == 1 else nk - 1] * dt
        rmin1, rmax1 = _extrema(r, eps)
        assert abs(mass1 - mass0) / max(abs(mass0), abs(mass1)) <= 10 * eps
        assert rmin1 >= rmin0 - 10 * eps
        assert rmax1 <= rmax0 + 10 * eps


def test_find_top_bottom(O):
    lib = O.load()
    v = np.array([0, 0, 1e-10, 0, 2e-9, 0, 0, 0], dtype=float)
    p = C.c_int(0)
    assert lib.p3o_find_top(_dp(v), 1e-14, 7, 0, -1, C.byref(p)) == 2 and p.value == 1
    assert lib.p3o_find_bottom(_dp(v), 1e-14, 7, 2, -1, C.byref(p)) == 4 and p.value == 1
    z = np.zeros(8)
    lib.p3o_find_top(_dp(z), 1e-14, 7, 0, -1, C.byref(p))
    assert p.value == 0


def test_table3_is_continuous(O, tables):
    """p3_table3_unit_tests.cpp:76-170: max |d log(vm)/d alpha| converges under refinement."""
    lib = O.load()
    t, keep = O.make_tables(tables)

    def interp(mu, lam):
        mu = np.ascontiguousarray(mu, dtype=float)
        lam = np.ascontiguousarray(lam, dtype=float)
        out = np.zeros(mu.size)
        lib.p3o_table3_lookup_apply(C.byref(t), 1, mu.size, _dp(mu), _dp(lam), _dp(out))
        return out

    def calc_lamr(mu_r, alpha):
        lo, hi = 0.1 * 116.3, 1.5 * 0.2e6
        return (lo + alpha * (hi - lo)) * (1 + mu_r)

    slopes = []
    n = 1000
    for _ in range(2):
        n *= 10
        a = np.arange(n + 1) / n
        mu = a * 10
        lam = np.full_like(mu, calc_lamr(4.5, 0.5))
        v = np.log(interp(mu, lam))
        slopes.append(np.max(np.abs(np.diff(v) * n)))
    assert slopes[1] / slopes[0] <= 1.1
    slopes = []
    n = 4000
    for _ in range(2):
        n *= 2
        a = np.arange(n + 1) / n
        mu = np.full(n + 1, 3.5)
        lam = calc_lamr(3.5, a)
        v = np.log(interp(mu, lam))
        slopes.append(np.max(np.abs(np.diff(v) * n)))
    assert slopes[1] / slopes[0] <= 1.1


def test_conservation_limiters_known_answers(O):
    """Known-answer cases of p3_unit_tests.cpp:27-131 (inputs from the test file)."""
    lib = O.load()
    kat = json.loads((GOLDEN / "reference_kats.json").read_text())
    eps = np.finfo(float).eps
    c = kat["cloud_water_conservation"]
    t = np.array(c["tend_in"], dtype=float)
    lib.p3o_cloud_water_conservation(c["qc"], c["dt"], _dp(t))
    ratio = c["qc"] / (c["tend_in"][0] * c["dt"])
    assert abs(t[0] - c["tend_in"][0] * ratio) <= eps
    assert np.all(t[1:6] == 0.0)
    assert abs(t[6] - (1.0 - ratio)) <= eps and abs(t[7] - (1.0 - ratio)) <= eps
    assert t[0] * c["dt"] <= c["qc"]
    r = kat["rain_water_conservation"]
    t = np.array(r["tend_in"], dtype=float)
    lib.p3o_rain_water_conservation(r["qr"], r["dt"], _dp(t))
    ratio = r["qr"] / (r["tend_in"][4] * r["dt"])
    assert np.all(t[:4] == 0.0)
    assert abs(t[4] - r["tend_in"][4] * ratio) <= eps
    assert t[4] * r["dt"] <= r["qr"]
    i = kat["ice_water_conservation"]
    t = np.array(i["tend_in"], dtype=float)
    lib.p3o_ice_water_conservation(i["qi"], i["dt"], _dp(t))
    ratio = i["qi"] / (i["tend_in"][7] * i["dt"])
    assert abs(t[7] - i["tend_in"][7] * ratio) <= eps
    assert t[7] * i["dt"] <= i["qi"] * (1 + eps)


def test_saturation_known_values(O):
    """Murphy & Koop (2005) liquid/ice vapour pressure at 273.15 K and 250 K
    (p = 1e5 Pa), checked against the published formulas evaluated here."""
    lib = O.load()
    ep2 = 18.016 / 28.966

    def mk_liq(T):
        lt = np.log(T)
        return np.exp(54.842763 - 6763.22 / T - 4.210 * lt + 0.000367 * T +
                      np.tanh(0.0415 * (T - 218.8)) * (53.878 - 1331.22 / T - 9.44523 * lt + 0.014025 * T))

    def mk_ice(T):
        return np.exp(9.550426 - 5723.265 / T + 3.53068 * np.log(T) - 0.00728332 * T)

    for T in (273.15, 250.0, 300.0):
        assert lib.p3o_qv_sat_dry(T, 1e5, 0) == pytest.approx(ep2 * mk_liq(T) / 1e5, rel=1e-14)
    assert lib.p3o_qv_sat_dry(250.0, 1e5, 1) == pytest.approx(ep2 * mk_ice(250.0) / 1e5, rel=1e-14)
    # above freezing the "ice" request falls back to liquid (physics_saturation_impl.hpp:55-56)
    assert lib.p3o_qv_sat_dry(280.0, 1e5, 1) == lib.p3o_qv_sat_dry(280.0, 1e5, 0)
    # 611.2 Pa at the triple point within 0.1 %
    assert mk_liq(273.16) == pytest.approx(611.657, rel=1e-3)


@pytest.mark.parametrize("kind,seed,ncol,nlev", [(0, 1000, 64, 72), (1, 1002, 48, 128)])
def test_oracle_step_conserves_column_water(O, tables, kind, seed, ncol, nlev):
    from scream_gb300.p3 import generate_inputs
    st = oracle_state(generate_inputs(kind, seed, ncol, nlev))
    w0 = column_water(st)
    err, _ = O.p3_main(st, tables, 300.0)
    assert err == 0
    w1 = column_water(st)
    p = (st["precip_liq_surf"] + st["precip_ice_surf"]) * 1000.0 * 300.0
    assert np.max(np.abs(w1 + p - w0) / w0) <= 1e-12
    for n in ["qc", "qr", "qi", "qv", "nc", "nr", "ni", "th"]:
        assert np.all(np.isfinite(st[n])), n
    for n in ["qc", "qr", "qi", "qv"]:
        assert st[n].min() >= 0.0, n


def test_mixed_ic_six_steps(O, tables):
    """The reference's p3_run_and_cmp case: mixed IC, 3 columns x 72 levels,
    dt = 300 s, 6 steps, predict_nc and prescribed_CCN both on
    (p3_run_and_cmp.cpp:238-247).  The oracle stays finite and conserves water."""
    from scream_gb300.p3 import generate_inputs
    st = oracle_state(generate_inputs(2, 0, 3, 72))
    for it in range(1, 7):
        w0 = column_water(st)
        err, _ = O.p3_main(st, tables, 300.0, it=it)
        assert err == 0
        p = (st["precip_liq_surf"] + st["precip_ice_surf"]) * 1000.0 * 300.0
        assert np.max(np.abs(column_water(st) + p - w0) / w0) <= 1e-12
    for n in st:
        assert np.all(np.isfinite(st[n])), n


def test_mixed_ic_matches_committed_oracle_fixture(O, tables):
    """Regression pin of the oracle: tests/golden/mixed_ic_oracle.npz was made
    by tests/golden/make_golden.py (same inputs, 6 steps)."""
    from scream_gb300.p3 import generate_inputs
    ref = np.load(GOLDEN / "mixed_ic_oracle.npz")
    for pn, pc in [(1, 1), (0, 0), (1, 0)]:
        st = oracle_state(generate_inputs(2, 0, 3, 72))
        for it in range(1, 7):
            O.p3_main(st, tables, 300.0, predictNc=bool(pn), prescribedCCN=bool(pc), it=it)
        for n in ["qc", "nc", "qr", "nr", "qi", "qm", "ni", "bm", "qv", "th", "precip_liq_surf",
                  "precip_ice_surf", "diag_eff_radius_qc", "diag_eff_radius_qr", "diag_eff_radius_qi"]:
            a, b = st[n], ref[f"p{pn}{pc}_{n}"]
            assert np.allclose(a, b, rtol=1e-9, atol=0.0), (pn, pc, n)


# Murphy & Koop (2005), Table C1, "values recommended for checking computer
# codes" -- the check points the reference's saturation test names
# (components/eamxx/src/physics/share/tests/physics_saturation_run_and_cmp.cpp:91-101),
# whose expected values live in a generated baseline file, not in the source.
# Published to five significant figures: (T in K, over ice?, vapour pressure in Pa as printed).
MK_TABLE_C1 = [
    (150.0, True, "6.1061e-6"), (180.0, True, "0.0053975"), (210.0, True, "0.70202"),
    (240.0, True, "27.272"), (273.16, True, "611.66"),
    (240.0, False, "37.667"), (273.16, False, "611.66"), (300.0, False, "3536.8"),
]


def _half_unit(printed):
    """Half a unit in the last printed significant digit."""
    low = printed.lower()
    mant = low.split("e")[0]
    exp = int(low.split("e")[1]) if "e" in low else 0
    decimals = len(mant.split(".")[1]) if "." in mant else 0
    return 0.5 * 10.0 ** (exp - decimals)


@pytest.mark.parametrize("T,ice,printed", MK_TABLE_C1)
def test_saturation_matches_published_check_values(O, T, ice, printed):
    """The oracle's Murphy-Koop vapour pressure rounds to the published
    five-figure check values (e = qv_sat p / ep_2 at p = 1e5 Pa)."""
    lib = O.load()
    ep2 = 18.016 / 28.966
    e = lib.p3o_qv_sat_dry(T, 1e5, int(ice)) * 1e5 / ep2
    assert abs(e - float(printed)) <= _half_unit(printed), (T, ice, e, printed)


@pytest.mark.parametrize("T,ice,printed", MK_TABLE_C1)
def test_saturation_table_matches_published_check_values(built, T, ice, printed):
    """The FP32-bulk form's tabulated vapour pressure (cubic per 1/64 K) at
    the same check points."""
    import ctypes as C
    from scream_gb300 import _lib as L
    lib = L.load()
    n, t0, inv_h = C.c_int32(0), C.c_double(0), C.c_double(0)
    assert lib.p3x_saturation_table(None, C.byref(n), C.byref(t0), C.byref(inv_h)) == 0
    coef = np.zeros(2 * n.value * 4)
    lib.p3x_saturation_table(coef.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n), C.byref(t0), C.byref(inv_h))
    x = (T - t0.value) * inv_h.value
    i = int(np.floor(x))
    u = x - i
    row = n.value + i if (ice and T < 273.15) else i
    c = coef[row * 4: row * 4 + 4]
    e = c[0] + u * (c[1] + u * (c[2] + u * c[3]))
    assert abs(e - float(printed)) <= _half_unit(printed), (T, ice, e, printed)
