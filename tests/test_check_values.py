"""check_values (components/eamxx/src/physics/p3/impl/p3_check_values_impl.hpp,
called after part3 at p3_main_impl.hpp:316-323 in the reference's debug
builds): T = th / inv_exner must lie in (173, 323) K and qv in (0, 0.04) on
every level of every column that went on past part2.  The library counts the
out-of-range levels and keeps the first location; in fail mode a temperature
out of range makes the step return P3X_ERANGE instead of the reference's
device abort.  Nothing traps: the bad values are planted in the inputs, on
the host."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = 300.0


@pytest.fixture(scope="module")
def bad_inputs(built):
    from scream_gb300.p3 import generate_inputs
    inp = generate_inputs(0, 1000, 64, 72)
    inp["th"][5, 70] = 330.0 * inp["inv_exner"][5, 70]   # hot surface level: T > 323 K
    inp["th"][9, 71] = 335.0 * inp["inv_exner"][9, 71]
    inp["qv"][7, 60] = 0.05                               # qv above 0.04
    return inp


def expected(ctx, inp):
    """Counts and first (column, level) from the step's own outputs, over the
    columns that go on past part2 (flag from the staged entry)."""
    import scream_gb300 as p3
    ncol, nlev = inp["qc"].shape
    f = p3.P3Fields.from_inputs(inp)
    ho = ctx.allocate_handover(ncol, nlev)
    ctx.p3_main_stages(f, DT, p3.P3X_STAGE_PART12, ho)
    go_on = ctx.handover_views(ho, ncol, nlev)[1].cpu().numpy().astype(bool)
    ctx.p3_main_stages(f, DT, p3.P3X_STAGE_SED | p3.P3X_STAGE_PART3, ho)
    h = f.to_host()
    T = h["th"] * (1.0 / h["inv_exner"])
    t_bad = ~((T > 173.0) & (T < 323.0)) & go_on[:, None]
    q_bad = ~((h["qv"] > 0.0) & (h["qv"] < 0.04)) & go_on[:, None]

    def first(mask):
        idx = np.argwhere(mask)
        return (-1, -1) if idx.size == 0 else tuple(int(x) for x in idx[0])
    return int(t_bad.sum()), int(q_bad.sum()), first(t_bad), first(q_bad)


def test_check_values_modes(gpu_ctx, bad_inputs):
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    nt, nq, ft, fq = expected(gpu_ctx, bad_inputs)
    assert nt >= 2 and nq >= 1
    try:
        # off: nothing recorded
        gpu_ctx.set_check_values(L.P3X_CHECK_OFF)
        gpu_ctx.check_values_report()
        gpu_ctx.p3_main(p3.P3Fields.from_inputs(bad_inputs), DT)
        r = gpu_ctx.check_values_report()
        assert r["t_out_of_range"] == 0 and r["qv_out_of_range"] == 0 and r["t_first_column"] == -1
        # record: counted, first locations, the step succeeds
        gpu_ctx.set_check_values(L.P3X_CHECK_RECORD)
        for precision in (L.P3X_FP64, L.P3X_FP32_BULK):
            gpu_ctx.p3_main(p3.P3Fields.from_inputs(bad_inputs), DT, precision)
            r = gpu_ctx.check_values_report()
            # the planted cells stay far from the bounds in both forms
            assert r["t_out_of_range"] == nt and r["qv_out_of_range"] == nq, (precision, r, nt, nq)
            assert (r["t_first_column"], r["t_first_level"]) == ft
            assert (r["qv_first_column"], r["qv_first_level"]) == fq
            assert r["t_first_instance"] == 0
        # the report clears
        r = gpu_ctx.check_values_report()
        assert r["t_out_of_range"] == 0 and r["qv_first_level"] == -1
        # fail: P3X_ERANGE, and the context keeps working
        gpu_ctx.set_check_values(L.P3X_CHECK_FAIL)
        with pytest.raises(L.P3Error) as ei:
            gpu_ctx.p3_main(p3.P3Fields.from_inputs(bad_inputs), DT)
        assert ei.value.code == L.P3X_ERANGE
        assert gpu_ctx.check_values_report()["t_out_of_range"] == nt
        good = {k: v.copy() for k, v in bad_inputs.items()}
        good["th"][5, 70] = good["th"][5, 69]
        good["th"][9, 71] = good["th"][9, 70]
        gpu_ctx.p3_main(p3.P3Fields.from_inputs(good), DT)
    finally:
        gpu_ctx.set_check_values(L.P3X_CHECK_OFF)
        gpu_ctx.check_values_report()


def test_check_values_batched_reports_instance(gpu_ctx, bad_inputs):
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    from scream_gb300.p3 import generate_inputs
    clean = generate_inputs(0, 1001, 40, 72)
    try:
        gpu_ctx.set_check_values(L.P3X_CHECK_RECORD)
        gpu_ctx.check_values_report()
        fields = [p3.P3Fields.from_inputs(clean), p3.P3Fields.from_inputs(bad_inputs)]
        b = p3.P3Batch(gpu_ctx, fields, [DT, DT], L.P3X_FP64)
        b.run()
        r = gpu_ctx.check_values_report()
        nt, _, ft, _ = expected(gpu_ctx, bad_inputs)
        assert r["t_out_of_range"] == nt
        assert (r["t_first_instance"], r["t_first_column"], r["t_first_level"]) == (1,) + ft
        b.close()
    finally:
        gpu_ctx.set_check_values(L.P3X_CHECK_OFF)
        gpu_ctx.check_values_report()
