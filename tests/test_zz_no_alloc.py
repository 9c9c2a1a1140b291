"""crv_pulses_static (scratch in a static device array, no caller workspace) against crv_pulses, through the C ABI.

Two calls in a row on different inputs (FP64 with 64-bit samples, then FP32-mixed with 16-bit samples): each must equal
crv_pulses on the same input bit for bit, so nothing left in the shared scratch by the first call leaks into the second.
A request larger than the static maximum is refused with CRV_ERR_TOO_LARGE before anything is launched.  Around a
later static call with every buffer allocated beforehand, neither the device's free memory nor torch's allocator
changes: the call itself allocates nothing.
The file is collected last so the test also runs after every other GPU test in one process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(seed, n_wf, adc16):
    import torch
    from tests.helpers import uneven_waveforms
    adc, n, start, ped, area, height = uneven_waveforms(np.random.default_rng(seed), n_wf)
    W, L = adc.shape
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a).astype(dt))).cuda()  # noqa: E731
    samples = d(adc, np.int16) if adc16 else d(adc, np.int64)
    return dict(nw=W, ns=W * L, off=d(np.arange(W) * L, np.int64), n=d(n, np.int32), start=d(start, np.int64),
                ped=d(ped, np.float64), area=d(area, np.float64), height=d(height, np.float64),
                adc16=samples if adc16 else None, adc64=None if adc16 else samples,
                max_pulses=int(max(8, int(np.max(n)))))


def _buffers(P, x, static):
    import torch
    from crvgpu import _capi
    L = _capi.load()
    nw, cap = x["nw"], 16 * x["nw"] + 1024
    out = {k: torch.full((cap,), -7, dtype=torch.int64, device="cuda") for k in _capi.PULSE_INT}
    out.update({k: torch.full((cap,), np.nan, dtype=torch.float64, device="cuda") for k in _capi.PULSE_FLOAT})
    out.update({k: torch.full((cap,), 9, dtype=torch.uint8, device="cuda") for k in _capi.PULSE_BOOL})
    near = torch.full((nw,), 9, dtype=torch.uint8, device="cuda")
    n_out = torch.zeros(1, dtype=torch.int64, device="cuda")
    status = _capi.DeviceStatus("cuda")
    status.reset()
    O = _capi.CrvPulses(*[_capi.ptr(out[k]) for k in _capi.PULSE_INT + _capi.PULSE_FLOAT + _capi.PULSE_BOOL])
    args = [ctypes.byref(P), nw, x["ns"], _capi.ptr(x["off"]), _capi.ptr(x["n"]), _capi.ptr(x["start"]),
            _capi.ptr(x["ped"]), _capi.ptr(x["area"]), _capi.ptr(x["height"]), _capi.ptr(x["adc16"]),
            _capi.ptr(x["adc64"]), x["max_pulses"], ctypes.byref(O), cap, _capi.ptr(n_out), _capi.ptr(near)]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ws = None
    if not static:
        ws = torch.empty(L.crv_pulses_workspace(ctypes.byref(P), nw, x["ns"]), dtype=torch.uint8, device="cuda")
    return dict(L=L, args=args, stream=stream, status=status, ws=ws, out=out, near=near, n_out=n_out, O=O)


def _launch(b, static):
    from crvgpu import _capi
    if static:
        rc = b["L"].crv_pulses_static(*b["args"], b["stream"], b["status"].ptr)
    else:
        rc = b["L"].crv_pulses(*b["args"], _capi.ptr(b["ws"]), b["ws"].numel(), b["stream"], b["status"].ptr)
    _capi.check(rc, "crv_pulses_static" if static else "crv_pulses")


def _results(b, static):
    import torch
    torch.cuda.synchronize()
    flags, need = b["status"].read()
    assert flags == 0, (static, flags, need)
    m = int(b["n_out"].item())
    res = {k: v[:m].cpu().numpy() for k, v in b["out"].items()}
    res["wf_near_threshold"] = b["near"].cpu().numpy()
    return res


def _call(P, x, static):
    b = _buffers(P, x, static)
    _launch(b, static)
    return _results(b, static)


def test_static_scratch_matches_workspace_entry_point_on_two_calls():
    from crvgpu import _capi
    from crvgpu.params import make_params
    L = _capi.load()
    cases = [(make_params(precision="fp64"), _inputs(11, 600, adc16=False)),
             (make_params(precision="fp32"), _inputs(12, 900, adc16=True))]
    for P, x in cases:
        assert L.crv_pulses_workspace(ctypes.byref(P), x["nw"], x["ns"]) <= _capi.PULSES_STATIC_MAX_BYTES
    got = [_call(P, x, static=True) for P, x in cases]          # two static calls in a row
    for (P, x), g in zip(cases, got):
        ref = _call(P, x, static=False)
        assert len(ref["wf"]) > x["nw"]                          # several pulses per waveform on average
        assert set(g) == set(ref)
        for k in ref:
            assert g[k].dtype == ref[k].dtype and np.array_equal(g[k], ref[k], equal_nan=True), k


def test_static_scratch_refuses_requests_above_its_maximum():
    import torch
    from crvgpu import _capi
    from crvgpu.params import make_params
    L = _capi.load()
    P = make_params(precision="fp64")
    nw, ns = 1 << 20, 64 << 20
    assert L.crv_pulses_workspace(ctypes.byref(P), nw, ns) > _capi.PULSES_STATIC_MAX_BYTES
    one = torch.zeros(8, dtype=torch.int64, device="cuda")
    O = _capi.CrvPulses(*[_capi.ptr(one)] * len(_capi.PULSE_INT + _capi.PULSE_FLOAT + _capi.PULSE_BOOL))
    status = _capi.DeviceStatus("cuda")
    status.reset()
    p = _capi.ptr(one)
    rc = L.crv_pulses_static(ctypes.byref(P), nw, ns, p, p, p, p, p, p, None, p, 8, ctypes.byref(O), 8, p, p,
                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), status.ptr)
    assert rc == _capi.CRV_ERR_TOO_LARGE
    with pytest.raises(ValueError, match="static maximum"):
        _capi.check(rc, "crv_pulses_static")


def test_static_call_allocates_nothing():
    """With its inputs, outputs and status block allocated beforehand, a static call changes neither the device's
    free memory (cudaMemGetInfo) nor torch's allocator: the entry point itself allocates nothing."""
    import torch
    from crvgpu import _capi
    from crvgpu.params import make_params
    _capi.profile(False)
    P = make_params(precision="fp32")
    x = _inputs(13, 700, adc16=True)
    first = _call(P, x, static=True)                       # warm-up: module loaded, scratch address known
    b = _buffers(P, x, static=True)
    torch.cuda.synchronize()
    free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    _launch(b, static=True)
    torch.cuda.synchronize()
    free1, alloc1 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    assert (free1, alloc1) == (free0, alloc0), (free0 - free1, alloc1 - alloc0)
    again = _results(b, static=True)
    for k in first:
        assert np.array_equal(again[k], first[k], equal_nan=True), k
