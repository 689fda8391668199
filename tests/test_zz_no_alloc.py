"""p3x_main_fixed_scratch: the P3 step with its hand-over scratch in static
device storage (no device allocation by the call).

Called through the C ABI and compared with p3x_main (scratch from the
context's pool) on the same inputs for two steps in a row.  Both run the same
kernels on the same data, so the tolerance is exact equality.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIXED_SCRATCH_BYTES = 64 << 20


def call_fixed(ctx, f, dt, precision, it):
    from scream_gb300 import _lib as L
    rt = L.default_runtime()
    infra = L.Infrastructure(dt, it, 1, f.ncol, 1, f.nlev, 1, 1, None)
    prog, din, dout, hist = f.prog(), f.din(), f.dout(), f.hist()
    lay = L.Layout(f.nlev, f.nlev + 1)
    return ctx.lib.p3x_main_fixed_scratch(ctx.h, C.byref(rt), C.byref(prog), C.byref(din), C.byref(dout),
                                          C.byref(infra), C.byref(hist), f.ncol, f.nlev, C.byref(lay),
                                          precision, None)


@pytest.mark.parametrize("precision", [0, 1])
def test_fixed_scratch_matches_pooled_entry_two_steps(gpu_ctx, precision):
    import torch
    import scream_gb300 as p3
    inp = p3.generate_inputs(1, 1002, 1500, 128)
    ref = p3.P3Fields.from_inputs(inp)
    got = p3.P3Fields.from_inputs(inp)
    for it in (1, 2):
        gpu_ctx.p3_main(ref, 300.0, precision, it=it)
        assert call_fixed(gpu_ctx, got, 300.0, precision, it) == 0
        torch.cuda.synchronize()
        gpu_ctx.check()
        a, b = ref.to_host(), got.to_host()
        for name in a:
            assert np.array_equal(a[name], b[name]), (it, name)


def test_fixed_scratch_reserved_at_context_creation(gpu_ctx):
    """The static array is reserved, and its address looked up, when the
    context is created, so a host that fills the device right after creating
    the context cannot meet an out-of-memory error on the first call."""
    import scream_gb300 as p3
    cap, res = C.c_int64(0), C.c_int32(0)
    ctx = p3.P3Context()
    try:
        assert ctx.lib.p3x_fixed_scratch_info(ctx.h, C.byref(cap), C.byref(res)) == 0
        assert cap.value == FIXED_SCRATCH_BYTES
        assert res.value == 1
    finally:
        ctx.close()


def test_fixed_scratch_rejects_oversize_call(gpu_ctx):
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    ncol, nlev = 14000, 128  # 40 * ncol * nlev + 4 * ncol > 64 MiB
    assert 40 * ncol * nlev + 4 * ncol > FIXED_SCRATCH_BYTES
    f = p3.P3Fields.allocate(ncol, nlev)
    before = f.t["qc"].clone()
    assert call_fixed(gpu_ctx, f, 300.0, 0, 1) == L.P3X_ENOMEM
    assert bool((f.t["qc"] == before).all())
