"""CPU checks of the synthetic workload generator (standard, RH-stress and mixed-IC columns)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def gen(built):
    from scream_gb300.p3 import generate_inputs
    return generate_inputs


def test_columns_are_independent_of_range(gen):
    a = gen(0, 1000, 40, 72)
    b = gen(0, 1000, 15, 72, col0=25)
    for n in a:
        np.testing.assert_array_equal(a[n][25:], b[n], err_msg=n)


def test_seed_changes_draws(gen):
    a = gen(0, 1000, 8, 72)
    b = gen(0, 1001, 8, 72)
    assert not np.array_equal(a["qc"], b["qc"])


def test_standard_atmosphere_distributions(gen):
    nlev = 128
    a = gen(0, 1000, 2000, nlev)
    p_int_bot = a["pres"][:, -1] + 0.5 * a["dpres"][:, -1]
    ps = p_int_bot
    assert abs(ps.mean() - 1e5) < 100 and 350 < ps.std() < 650
    assert np.all(np.diff(a["pres"], axis=1) > 0)          # monotone downward
    assert np.allclose(a["pres"][:, 0] - 0.5 * a["dpres"][:, 0], 200.0)  # 2 hPa top
    T = a["th"] / a["inv_exner"]
    assert 150 < T.min() and T.max() < 320
    # cloud layer: q in [1e-7, 1e-3] where present, zero outside
    for n in ["qc", "qr", "qi"]:
        v = a[n][a[n] > 0]
        assert v.min() >= 1e-7 * (1 - 1e-12) and v.max() <= 1e-3
    inside = a["qc"] > 0
    assert np.all(a["cld_frac_l"][inside] == 1.0)
    assert np.all(a["cld_frac_l"][~inside] == 1e-4)
    assert np.all(a["nc"][inside] >= 5e7) and np.all(a["nc"][inside] <= 2e8)
    assert np.all(a["qm"] <= 0.5 * a["qi"] + 1e-30)
    # rain fraction: max overlap with the level above
    cr = a["cld_frac_r"]
    ct = np.where(inside, 1.0, 0.0)
    expect = np.maximum(np.maximum(ct, 1e-4), np.concatenate([np.zeros((ct.shape[0], 1)), ct[:, :-1]], axis=1))
    np.testing.assert_array_equal(cr, expect)
    assert np.all(a["nccn"] == 1e8) and np.all(a["inv_qc_relvar"] == 1.0)
    np.testing.assert_array_equal(a["qv_prev"], a["qv"])
    # RH ~ U(0.3, 1.05): qv / qsat_liq within bounds
    ep2 = 18.016 / 28.966
    lt = np.log(T)
    es = np.exp(54.842763 - 6763.22 / T - 4.210 * lt + 0.000367 * T +
                np.tanh(0.0415 * (T - 218.8)) * (53.878 - 1331.22 / T - 9.44523 * lt + 0.014025 * T))
    rh = a["qv"] / (ep2 * es / a["pres"])
    assert rh.min() >= 0.3 - 1e-9 and rh.max() <= 1.05 + 1e-9


def test_supersaturation_stress_columns(gen):
    a = gen(1, 1002, 64, 128)
    T = a["th"] / a["inv_exner"]
    ep2 = 18.016 / 28.966
    lt = np.log(T)
    es = np.exp(54.842763 - 6763.22 / T - 4.210 * lt + 0.000367 * T +
                np.tanh(0.0415 * (T - 218.8)) * (53.878 - 1331.22 / T - 9.44523 * lt + 0.014025 * T))
    rh = a["qv"] / (ep2 * es / a["pres"])
    assert rh[0::2].min() >= 0.9 - 1e-9          # even columns: U(0.9, 1.05)
    assert rh[1::2].min() < 0.6                    # odd columns keep U(0.3, 1.05)


def test_mixed_case_matches_reference_ic(gen):
    """Spot values of physics/p3/p3_ic_cases.cpp:11-120 (nk = 72)."""
    a = gen(2, 0, 3, 72)
    nk = 72
    assert a["qc"][0, nk - 20] == 1e-4 and a["qc"][0, 35] == 1e-7 and a["qc"][0, nk - 1] == 1e-6
    assert a["qi"][0, nk - 1] == 1e-9 and a["qi"][0, nk - 25] == 5e-8
    assert a["qv"][0, nk - 1] == 5e-2 and a["qv"][0, 33] == 1e-4
    assert a["pres"][0, 0] == 100.0 and np.all(a["nccn"] == 1e8)
    T = 150 + 150 / nk * np.arange(nk)
    np.testing.assert_allclose(a["t_prev"][0], T)
    T1 = T + ((1 % 3) - 0.5) / nk * np.arange(nk)
    np.testing.assert_allclose(a["t_prev"][1], T1)
