"""p3x_main_host: the P3 step on host arrays, columns in chunks through a ring
of device buffers with the copies overlapped with the kernels.

Columns are independent, so every output must equal, bit for bit, the device
entry p3x_main on the same data, for any chunking (including a ragged last
chunk and a single chunk), in both arithmetic forms and over two steps with
the state carried.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_fields(inputs):
    import torch
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    ncol, nlev = inputs["qc"].shape
    h = p3.P3Fields.allocate_host(ncol, nlev)
    for n in L.INPUT_FIELDS:
        h.t[n].copy_(torch.from_numpy(np.ascontiguousarray(inputs[n])))
    return h


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("chunk_cols", [256, 0])
def test_host_entry_matches_device_entry(gpu_ctx, precision, chunk_cols):
    import scream_gb300 as p3
    inputs = p3.generate_inputs(1, 1002, 1500, 72)
    dev = p3.P3Fields.from_inputs(inputs)
    host = _host_fields(inputs)
    for it in (1, 2):
        gpu_ctx.p3_main(dev, 300.0, precision, it=it)
        us = gpu_ctx.p3_main_host(host, 300.0, precision, it=it, chunk_cols=chunk_cols)
        assert us > 0
        a = dev.to_host()
        for name, v in host.t.items():
            assert np.array_equal(a[name], v.numpy()), (it, name)


def test_host_entry_arguments(gpu_ctx):
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    host = _host_fields(p3.generate_inputs(0, 5, 8, 16))
    with pytest.raises(L.P3Error) as e:
        gpu_ctx.p3_main_host(host, 300.0, 1, chunk_cols=-1)
    assert e.value.code == L.P3X_EINVAL
    empty = p3.P3Fields.allocate_host(0, 16)
    assert gpu_ctx.p3_main_host(empty, 300.0, 1) == 0.0


def test_host_entry_concurrent_calls_on_one_context(gpu_ctx):
    """Two threads stepping different host arrays through one context (the
    calls are serialised on its chunk buffers) each get the device entry's
    result."""
    import threading
    import scream_gb300 as p3
    ins = [p3.generate_inputs(1, 900 + s, 700, 72) for s in range(2)]
    hosts = [_host_fields(i) for i in ins]
    errors = []

    def work(h):
        try:
            for it in (1, 2):
                gpu_ctx.p3_main_host(h, 300.0, 1, it=it, chunk_cols=128)
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=work, args=(h,)) for h in hosts]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for inp, h in zip(ins, hosts):
        dev = p3.P3Fields.from_inputs(inp)
        for it in (1, 2):
            gpu_ctx.p3_main(dev, 300.0, 1, it=it)
        a = dev.to_host()
        for name, v in h.t.items():
            assert np.array_equal(a[name], v.numpy()), name


def test_host_entry_pageable_arrays(gpu_ctx):
    """Pageable (not page-locked) host arrays give the same result."""
    import torch
    import scream_gb300 as p3
    from scream_gb300 import _lib as L
    inputs = p3.generate_inputs(1, 77, 600, 72)
    dev = p3.P3Fields.from_inputs(inputs)
    host = p3.P3Fields.allocate_host(600, 72, pinned=False)
    for n in L.INPUT_FIELDS:
        host.t[n].copy_(torch.from_numpy(np.ascontiguousarray(inputs[n])))
    gpu_ctx.p3_main(dev, 300.0, 1)
    gpu_ctx.p3_main_host(host, 300.0, 1, chunk_cols=200)
    a = dev.to_host()
    for name, v in host.t.items():
        assert np.array_equal(a[name], v.numpy()), name
