"""Asynchronous host transfers (gpumhd_upload_async / gpumhd_download_async).

Each asynchronous upload / download is ordered with the context's steps
exactly as the synchronous call is; only its host copy runs on a copy stream
of its own.  So a queue of (upload, step, download) triples over different
host buffers must give, bit for bit, what the synchronous calls give one
triple at a time, in both precisions, with pinned and with pageable host
memory, and mixed with synchronous calls.
"""
import numpy as np
import pytest
import torch

import helpers as H
from muram_main_gb300 import gpumhd, initial

pytestmark = pytest.mark.gpu

NX, NY, NZ = 32, 24, 16


def _inputs(n):
    tab = initial.EosTable(H.EOS_SMALL)
    return [np.ascontiguousarray(np.moveaxis(initial.periodic_box(tab, NX, NY, NZ, seed=11 + s), 0, -1))
            for s in range(n)]


def _ctx(precision):
    return gpumhd.MuramGPU(gpumhd.default_params(NX, NY, NZ, 3.2e6, precision=precision), eos_path=H.EOS_SMALL)


def _sync_results(g, ins):
    out = []
    for a in ins:
        r = np.empty_like(a)
        g.upload_ptr(gpumhd.FIELD_U, a.ctypes.data)
        g.run_steps(1)
        g.download_ptr(gpumhd.FIELD_U, r.ctypes.data)
        out.append(r)
    return out


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("precision", [64, 32])
def test_queued_transfers_equal_synchronous_calls(gpu_lib, precision, pinned):
    ins = _inputs(4)
    g = _ctx(precision)
    ref = _sync_results(g, ins)
    if pinned:
        h_in = [torch.from_numpy(a.reshape(-1)).pin_memory() for a in ins]
        h_out = [torch.empty_like(t).pin_memory() for t in h_in]
        ptr_in = [t.data_ptr() for t in h_in]
        ptr_out = [t.data_ptr() for t in h_out]
        result = lambda s: h_out[s].numpy().reshape(ins[s].shape)  # noqa: E731
    else:
        outs = [np.full_like(a, np.nan) for a in ins]
        ptr_in = [a.ctypes.data for a in ins]
        ptr_out = [o.ctypes.data for o in outs]
        result = lambda s: outs[s]  # noqa: E731
    # every triple queued before any wait; each step starts from its own input
    for s in range(len(ins)):
        g.upload_ptr_async(gpumhd.FIELD_U, ptr_in[s])
        g.enqueue_steps(1)
        g.download_ptr_async(gpumhd.FIELD_U, ptr_out[s])
    g.synchronize()
    for s in range(len(ins)):
        assert np.array_equal(result(s), ref[s]), (precision, pinned, s)
    g.close()


def test_async_and_synchronous_calls_mix(gpu_lib):
    ins = _inputs(2)
    g = _ctx(64)
    ref = _sync_results(g, ins)
    h_in = [torch.from_numpy(a.reshape(-1)).pin_memory() for a in ins]
    h_out = torch.empty_like(h_in[0]).pin_memory()
    # asynchronous upload, synchronous download
    g.upload_ptr_async(gpumhd.FIELD_U, h_in[0].data_ptr())
    g.enqueue_steps(1)
    r0 = np.empty_like(ins[0])
    g.download_ptr(gpumhd.FIELD_U, r0.ctypes.data)
    assert np.array_equal(r0, ref[0])
    # synchronous upload, asynchronous download, then a second asynchronous
    # upload queued behind it
    g.upload_ptr(gpumhd.FIELD_U, ins[1].ctypes.data)
    g.enqueue_steps(1)
    g.download_ptr_async(gpumhd.FIELD_U, h_out.data_ptr())
    g.upload_ptr_async(gpumhd.FIELD_U, h_in[0].data_ptr())
    g.enqueue_steps(1)
    g.synchronize()
    assert np.array_equal(h_out.numpy().reshape(ins[1].shape), ref[1])
    r2 = np.empty_like(ins[0])
    g.download_ptr(gpumhd.FIELD_U, r2.ctypes.data)
    assert np.array_equal(r2, ref[0])
    g.close()


@pytest.mark.parametrize("precision", [64, 32])
def test_float_host_layout_equals_double_layout(gpu_lib, precision):
    """gpumhd_upload_f32 / gpumhd_download_f32 (and the asynchronous pair):
    a float32 cState array, as MURaM built with SINGLE_PRECISION holds it,
    gives the device state that the float64 array of the same values gives,
    and a float32 download is the float64 download rounded to nearest."""
    ins = [a.astype(np.float32) for a in _inputs(3)]
    g = _ctx(precision)
    ref = _sync_results(g, [a.astype(np.float64) for a in ins])
    # synchronous float32 transfers
    for a, r in zip(ins, ref):
        g.upload_ptr(gpumhd.FIELD_U, a.ctypes.data, np.float32)
        g.run_steps(1)
        out = np.full_like(a, np.nan)
        g.download_ptr(gpumhd.FIELD_U, out.ctypes.data, np.float32)
        assert np.array_equal(out, r.astype(np.float32)), precision
        d64 = g.download(gpumhd.FIELD_U)
        assert np.array_equal(d64.reshape(r.shape), r), precision
    # queued float32 transfers from pinned memory
    h_in = [torch.from_numpy(a.reshape(-1)).pin_memory() for a in ins]
    h_out = [torch.full_like(t, float("nan")).pin_memory() for t in h_in]
    for s in range(len(ins)):
        g.upload_ptr_async(gpumhd.FIELD_U, h_in[s].data_ptr(), np.float32)
        g.enqueue_steps(1)
        g.download_ptr_async(gpumhd.FIELD_U, h_out[s].data_ptr(), np.float32)
    g.synchronize()
    for s in range(len(ins)):
        assert np.array_equal(h_out[s].numpy().reshape(ins[s].shape), ref[s].astype(np.float32)), (precision, s)
    # a one-value field (the pressure) through the numpy wrappers
    p64 = g.download(gpumhd.FIELD_PRES)
    p32 = g.download(gpumhd.FIELD_PRES, dtype=np.float32)
    assert np.array_equal(p32, p64.astype(np.float32))
    g.upload(gpumhd.FIELD_PRES, p32)
    assert np.array_equal(g.download(gpumhd.FIELD_PRES), p32.astype(np.float64))
    g.close()
