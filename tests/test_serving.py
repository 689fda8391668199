"""Serving loop (p3x_server_*): continuous batching under a memory budget.

Each instance's result must be the same alone and in a mix: columns are
independent and the kernels' arithmetic does not depend on batching, so the
tolerance is exact equality.  A one-step instance must also equal a direct
p3_main of the same inputs (the server's instance data is a column slice of
its synthetic workload, seed 5000).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TEMPLATE_SEED = 5000
TEMPLATE_COLS = 65536
PROG = ["qc", "nc", "qr", "nr", "qi", "qm", "ni", "bm", "qv", "th"]


def read_state(srv, iid, ncol, nlev):
    out = {n: srv.read_field(iid, f, ncol * nlev).reshape(ncol, nlev) for f, n in enumerate(PROG)}
    out["precip_liq_surf"] = srv.read_field(iid, -1, ncol)
    out["precip_ice_surf"] = srv.read_field(iid, -2, ncol)
    return out


@pytest.fixture(scope="module")
def server_cls(built):
    import scream_gb300 as p3
    return p3.P3Server


def test_one_step_equals_direct_p3_main(gpu_ctx, server_cls):
    import scream_gb300 as p3
    srv = server_cls(gpu_ctx, budget_bytes=4 * 10**9, max_inflight=2)
    try:
        cases = [(1, 257, 128, p3.P3X_FP64, 11), (2, 1000, 72, p3.P3X_FP32_BULK, 77777)]
        for iid, ncol, nlev, prec, seed in cases:
            srv.submit(iid, ncol, nlev, prec, total_steps=1, seed=seed)
        srv.drain()
        for iid, ncol, nlev, prec, seed in cases:
            c0 = seed % (TEMPLATE_COLS - ncol + 1)
            inp = p3.generate_inputs(0, TEMPLATE_SEED, ncol, nlev, col0=c0)
            f = p3.P3Fields.from_inputs(inp)
            gpu_ctx.p3_main(f, 300.0, prec)
            ref = f.to_host()
            got = read_state(srv, iid, ncol, nlev)
            for n in PROG + ["precip_liq_surf", "precip_ice_surf"]:
                assert np.array_equal(got[n], ref[n]), n
    finally:
        srv.close()


@pytest.mark.parametrize("policy", ["latency", "throughput", "latency+partition", "latency+chunks"])
def test_result_alone_equals_result_in_mix(gpu_ctx, server_cls, policy):
    """Bitwise the same alone and in a mix, under both dispatch policies (the
    latency policy also shrinks large steps' grids and reserves a slot) and
    under an SM partition (probe 7, 21,600 column-levels, runs on the small
    partition's green context, the others on the rest of the SMs) and with
    dispatches launched in chunks of 2^18 column-levels (probe 9 alone is
    1.15e6)."""
    import scream_gb300 as p3
    probes = [(7, 300, 72, p3.P3X_FP64, 3, 123), (8, 2000, 128, p3.P3X_FP32_BULK, 4, 456),
              (9, 9000, 128, p3.P3X_FP32_BULK, 2, 789)]

    def run(mix):
        srv = server_cls(gpu_ctx, budget_bytes=6 * 10**9, max_inflight=4)
        srv.set_latency_policy(policy != "throughput")
        if policy.endswith("partition"):
            small, rest = srv.set_sm_partition(16, 1 << 15)
            assert small >= 16 and rest > 0
        if policy.endswith("chunks"):
            srv.set_dispatch_chunk(1 << 18)
        try:
            rng = np.random.default_rng(3)
            if mix:
                for j in range(40):
                    ncol = int(np.exp(rng.uniform(0, np.log(8192))))
                    nlev = 72 if rng.random() < 0.5 else 128
                    prec = p3.P3X_FP64 if rng.random() < 0.5 else p3.P3X_FP32_BULK
                    steps = int(rng.integers(1, 4))
                    for s in range(steps):
                        srv.submit(1000 + j, ncol, nlev, prec, steps, seed=int(rng.integers(1 << 30)),
                                   arrival_s=float(rng.uniform(0, 0.05)))
            for iid, ncol, nlev, prec, steps, seed in probes:
                for s in range(steps):
                    srv.submit(iid, ncol, nlev, prec, steps, seed=seed, arrival_s=0.01 * s if mix else 0.0)
            st = srv.drain()
            return {iid: read_state(srv, iid, ncol, nlev) for iid, ncol, nlev, _, _, _ in probes}, st
        finally:
            srv.close()

    alone, st_alone = run(False)
    mixed, st_mix = run(True)
    assert st_mix["completed"] > st_alone["completed"]
    for iid in alone:
        for n in alone[iid]:
            assert np.array_equal(alone[iid][n], mixed[iid][n]), (iid, n)


def test_sm_partition_arguments_and_removal(gpu_ctx, server_cls):
    """set_sm_partition: argument checks, SM counts that add up to the
    device's, and removal (0) back to an unpartitioned server that still runs
    requests."""
    import torch
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    srv = server_cls(gpu_ctx, budget_bytes=2 * 10**9, max_inflight=2)
    try:
        for bad in ((-1, 1 << 15), (8, 0), (sms, 1 << 15)):
            with pytest.raises(L.P3Error):
                srv.set_sm_partition(*bad)
        small, rest = srv.set_sm_partition(8, 1 << 15)
        assert small >= 8 and small + rest <= sms
        srv.submit(1, 16, 72, p3.P3X_FP64, total_steps=1, seed=1)
        srv.submit(2, 1024, 128, p3.P3X_FP32_BULK, total_steps=1, seed=2)
        assert srv.drain()["completed"] == 2
        assert srv.set_sm_partition(0) == (0, 0)
        srv.submit(3, 16, 72, p3.P3X_FP64, total_steps=1, seed=3)
        assert srv.drain()["completed"] == 3  # counted since the server started
    finally:
        srv.close()
    one = server_cls(gpu_ctx, budget_bytes=10**9, max_inflight=1)
    try:
        with pytest.raises(L.P3Error):  # the partition needs a second slot
            one.set_sm_partition(8, 1 << 15)
    finally:
        one.close()


def test_budget_admission_and_rejection(gpu_ctx, server_cls):
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    # one 8192 x 128 instance needs ~400 MB: a 600 MB budget holds one at a time
    srv = server_cls(gpu_ctx, budget_bytes=600 * 10**6, max_inflight=4)
    try:
        for iid in range(3):
            srv.submit(iid, 8192, 128, p3.P3X_FP32_BULK, total_steps=1, seed=iid)
        st = srv.drain()
        assert st["completed"] == 3
        assert 0 < st["peak_bytes"] <= 600 * 10**6
        with pytest.raises(L.P3Error):
            srv.submit(99, 65536, 128, p3.P3X_FP64, total_steps=1, seed=1)
    finally:
        srv.close()


def test_poisson_load_reports_latency(gpu_ctx, server_cls):
    srv = server_cls(gpu_ctx, budget_bytes=20 * 10**9, max_inflight=4)
    try:
        st = srv.run_poisson(rate_hz=100.0, n_sessions=30, max_ncol=4096, seed=9)
        assert st["completed"] >= 30
        assert st["rejected"] == 0
        assert 0 < st["p50_ms"] <= st["p90_ms"] <= st["p99_ms"] <= st["max_ms"]
        assert st["column_levels_per_s"] > 0
        assert st["peak_bytes"] <= 20 * 10**9
    finally:
        srv.close()


def test_requests_carry_data_and_report_per_class(gpu_ctx, server_cls):
    """Every step downloads its result (10 prognostic fields + 2 surface
    rates) and every session's first step uploads its 23 input fields; the
    statistics count those bytes, split latency by size class and, after
    calibration, report slowdowns."""
    import scream_gb300 as p3
    srv = server_cls(gpu_ctx, budget_bytes=20 * 10**9, max_inflight=4)
    try:
        srv.calibrate()
        for prec in (p3.P3X_FP64, p3.P3X_FP32_BULK):
            t_small = srv.isolated_ms(prec, 128, 8)
            t_big = srv.isolated_ms(prec, 128, 65536)
            assert 0 < t_small < t_big
        srv.submit(5, 300, 72, p3.P3X_FP64, total_steps=2, seed=1)
        srv.submit(5, 300, 72, p3.P3X_FP64, total_steps=2, seed=1)
        srv.submit(6, 20, 128, p3.P3X_FP32_BULK, total_steps=1, seed=2)
        st = srv.drain()
        assert st["completed"] == 3
        assert st["h2d_bytes"] == 23 * 8 * (300 * 72 + 20 * 128)
        assert st["d2h_bytes"] == 8 * (2 * 300 * (10 * 72 + 2) + 20 * (10 * 128 + 2))
        cls = st["by_size_class"]
        assert cls["10-99"]["count"] == 1 and cls["100-999"]["count"] == 2
        assert st["slowdown_p50"] > 0
    finally:
        srv.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_checkpoint_export_import_resumes_bitwise(gpu_ctx, server_cls, precision):
    """Step N, export, import into another server, step N+1 .. M: the same
    bits as M uninterrupted steps."""
    ncol, nlev, seed, total = 777, 72, 31, 4

    def run(steps, srv, iid=3):
        for _ in range(steps):
            srv.submit(iid, ncol, nlev, precision, total_steps=total, seed=seed)
        srv.drain()

    a = server_cls(gpu_ctx, budget_bytes=4 * 10**9, max_inflight=2)
    try:
        run(total, a)
        ref = read_state(a, 3, ncol, nlev)
    finally:
        a.close()
    b = server_cls(gpu_ctx, budget_bytes=4 * 10**9, max_inflight=2)
    try:
        run(2, b)
        ckpt = b.export_instance(3, ncol, nlev)
    finally:
        b.close()
    c = server_cls(gpu_ctx, budget_bytes=4 * 10**9, max_inflight=2)
    try:
        c.import_instance(3, ckpt, precision)
        np.testing.assert_array_equal(c.export_instance(3, ncol, nlev), ckpt)
        run(total - 2, c)
        got = read_state(c, 3, ncol, nlev)
        for n in ref:
            assert np.array_equal(got[n], ref[n]), n
    finally:
        c.close()
