"""Pulse reconstruction on the GPU.

Drop-in counterparts of crv/crvfastsim/reco/pulsefit.py: reconstruct (:236), reconstruct_full (:222),
filter_channels (:228), concat_waveforms (:319).  reconstruct returns the same flat per-pulse dict (wf, seq, pe, peph,
time, height, beta, chi2, letime, failed, zerondf, ped, pedfromdb, fit_A, fit_mu, fit_b) plus the per-waveform
wf_near_threshold, in (waveform, sequence) order.
"""
from __future__ import annotations

import ctypes
from dataclasses import replace

import numpy as np

from . import _capi
from .config import PERIOD, RecoConfig
from .params import make_params
from .response import _stream, _torch, raise_status


class PulseEngine:
    def __init__(self, device="cuda"):
        self.device = device
        self.ws = None
        self.out_factor = 2.0
        self.status = _capi.DeviceStatus(device)

    def run(self, P, off, n, start_tdc, ped, area, height, adc16=None, adc64=None, max_pulses=8, nsamples=None,
            max_tries=4):
        torch = _torch()
        L = _capi.load()
        dev = self.device
        nw = int(n.numel())
        ns = int(nsamples if nsamples is not None else (adc16 if adc16 is not None else adc64).numel())
        for _ in range(max_tries):
            cap = int(max(1024, self.out_factor * nw))
            wsb = L.crv_pulses_workspace(ctypes.byref(P), nw, ns)
            if self.ws is None or self.ws.numel() < wsb:
                self.ws = torch.empty(int(wsb * 1.1) + 1024, dtype=torch.uint8, device=dev)
            out = {k: torch.empty(cap, dtype=torch.int64, device=dev) for k in _capi.PULSE_INT}
            out.update({k: torch.empty(cap, dtype=torch.float64, device=dev) for k in _capi.PULSE_FLOAT})
            out.update({k: torch.empty(cap, dtype=torch.uint8, device=dev) for k in _capi.PULSE_BOOL})
            near = torch.empty(max(nw, 1), dtype=torch.uint8, device=dev)
            n_out = torch.zeros(1, dtype=torch.int64, device=dev)
            self.status.reset()
            O = _capi.CrvPulses(*[_capi.ptr(out[k]) for k in _capi.PULSE_INT + _capi.PULSE_FLOAT + _capi.PULSE_BOOL])
            r = L.crv_pulses(ctypes.byref(P), nw, ns, _capi.ptr(off), _capi.ptr(n), _capi.ptr(start_tdc),
                             _capi.ptr(ped), _capi.ptr(area), _capi.ptr(height), _capi.ptr(adc16), _capi.ptr(adc64),
                             int(min(max_pulses, 2 ** 31 - 1)), ctypes.byref(O), cap, _capi.ptr(n_out),
                             _capi.ptr(near), _capi.ptr(self.ws), self.ws.numel(), _stream(), self.status.ptr)
            _capi.check(r, "crv_pulses")
            flags, need = self.status.read()
            npo = need[_capi.NEED["PULSES_OUT"]]
            if flags == _capi.ST_CAPACITY and npo:
                self.out_factor = 1.3 * npo / max(nw, 1)
                continue
            raise_status(flags, need, "crv_pulses")
            m = int(n_out.item())
            res = {k: v[:m] for k, v in out.items()}
            res["wf_near_threshold"] = near[:nw]
            return res
        raise RuntimeError("crv_pulses: capacities did not converge")


DEFAULT_SHAPE = (128, 16, 0)           # threads per block, blocks per SM, rounds (0: one persistent launch)


def set_shape(shape):
    """Launch shape of the pulse fit for later calls: threads 64 or 128, blocks per SM 1..32, and rounds (0: one
    persistent launch whose lanes claim waveforms as they finish; 1..32: round launches before a tail launch)."""
    _capi.check(_capi.load().crv_pulses_shape(*[int(v) for v in shape]), "crv_pulses_shape")


SHAPES = tuple((t, b, 0) for t in (64, 128) for b in (4, 8, 16, 32)) + ((128, 16, 8), (128, 16, 16))


class ShapeTuner:
    """Picks the launch shape of the pulse fit per size bucket by timing every candidate once on the first batch of
    that bucket; results do not depend on the shape.  A bucket is (waveform count rounded up to a power of two,
    longest waveform rounded up to a power of two): the count sets how many lanes the launch can fill, the length how
    long a lane's waveform keeps it (pulses per waveform and the peak searches grow with it)."""

    def __init__(self, shapes=SHAPES):
        self.shapes = tuple(shapes)
        self.best = {}                 # bucket -> (shape, {shape: ms})

    @staticmethod
    def bucket(nw, max_len=0):
        return (max(0, int(nw - 1).bit_length()), max(0, int(max_len - 1).bit_length()))

    def shape_for(self, eng, P, batch, max_len=None):
        """Shape for this batch's bucket, tuning it first when unseen; batch = the keyword arguments of eng.run."""
        torch = _torch()
        if max_len is None:
            max_len = int(batch["n"].max().item()) if batch["n"].numel() else 0
        b = self.bucket(int(batch["n"].numel()), max_len)
        if b not in self.best:
            times = {}
            for sh in self.shapes:
                set_shape(sh)
                eng.run(P, **batch)                           # warm (workspace, capacities)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                eng.run(P, **batch)
                e1.record()
                torch.cuda.synchronize()
                times[sh] = e0.elapsed_time(e1)
            self.best[b] = (min(times, key=times.get), times)
        return self.best[b][0]


class GraphFitter:
    """Fits batches of up to nw_cap waveforms / ns_cap samples (int16) by replaying one captured CUDA graph of
    crv_pulses: each batch is copied into static device buffers and padded with zero-length waveforms (which find no
    pulses), so every replay has the captured shape.  The launch shape is the one in force at capture."""

    def __init__(self, P, nw_cap, ns_cap, out_cap, max_pulses=2 ** 31 - 1, device="cuda"):
        torch = _torch()
        L = _capi.load()
        self.P, self.nw_cap, self.ns_cap, self.out_cap, self.device = P, int(nw_cap), int(ns_cap), int(out_cap), device
        i64, i32, f64 = torch.int64, torch.int32, torch.float64
        self.inp = dict(off=torch.zeros(self.nw_cap, dtype=i64, device=device),
                        n=torch.zeros(self.nw_cap, dtype=i32, device=device),
                        start=torch.zeros(self.nw_cap, dtype=i64, device=device),
                        ped=torch.zeros(self.nw_cap, dtype=f64, device=device),
                        area=torch.ones(self.nw_cap, dtype=f64, device=device),
                        height=torch.ones(self.nw_cap, dtype=f64, device=device),
                        adc=torch.zeros(self.ns_cap, dtype=torch.int16, device=device))
        self.out = {k: torch.empty(self.out_cap, dtype=i64, device=device) for k in _capi.PULSE_INT}
        self.out.update({k: torch.empty(self.out_cap, dtype=f64, device=device) for k in _capi.PULSE_FLOAT})
        self.out.update({k: torch.empty(self.out_cap, dtype=torch.uint8, device=device) for k in _capi.PULSE_BOOL})
        self.near = torch.empty(self.nw_cap, dtype=torch.uint8, device=device)
        self.n_out = torch.zeros(1, dtype=i64, device=device)
        self.status = _capi.DeviceStatus(device)
        wsb = L.crv_pulses_workspace(ctypes.byref(P), self.nw_cap, self.ns_cap)
        self.ws = torch.empty(int(wsb) + 1024, dtype=torch.uint8, device=device)
        self.O = _capi.CrvPulses(*[_capi.ptr(self.out[k]) for k in _capi.PULSE_INT + _capi.PULSE_FLOAT +
                                   _capi.PULSE_BOOL])
        self.max_pulses = int(min(max_pulses, 2 ** 31 - 1))
        self._call()                                          # warm-up outside the capture
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(self.graph, stream=side):
                self.status.t.zero_()
                self._call()
        torch.cuda.current_stream().wait_stream(side)

    def _call(self):
        L = _capi.load()
        x = self.inp
        _capi.check(L.crv_pulses(ctypes.byref(self.P), self.nw_cap, self.ns_cap, _capi.ptr(x["off"]),
                                 _capi.ptr(x["n"]), _capi.ptr(x["start"]), _capi.ptr(x["ped"]), _capi.ptr(x["area"]),
                                 _capi.ptr(x["height"]), _capi.ptr(x["adc"]), None, self.max_pulses,
                                 ctypes.byref(self.O), self.out_cap, _capi.ptr(self.n_out), _capi.ptr(self.near),
                                 _capi.ptr(self.ws), self.ws.numel(), _stream(), self.status.ptr), "crv_pulses")

    def fit(self, off, n, start_tdc, ped, area, height, adc16):
        """Pulses of one batch (device tensors as PulseEngine.run takes them); returns the same dict."""
        adc16 = adc16.reshape(-1)
        nw, ns = int(n.numel()), int(adc16.numel())
        if nw > self.nw_cap or ns > self.ns_cap:
            raise ValueError(f"GraphFitter: batch of {nw} waveforms / {ns} samples exceeds its capacity")
        x = self.inp
        x["n"][nw:].zero_()
        for k, v in (("off", off), ("n", n), ("start", start_tdc), ("ped", ped), ("area", area), ("height", height)):
            x[k][:nw].copy_(v)
        x["adc"][:ns].copy_(adc16)
        self.graph.replay()
        flags, need = self.status.read()
        raise_status(flags, need, "crv_pulses (graph)")
        m = int(self.n_out.item())
        res = {k: v[:m] for k, v in self.out.items()}
        res["wf_near_threshold"] = self.near[:nw]
        return res


_ENGINE = {}


def engine(device="cuda"):
    if device not in _ENGINE:
        _ENGINE[device] = PulseEngine(device)
    return _ENGINE[device]


def _to_host(res):
    out = {}
    for k, v in res.items():
        a = v.cpu().numpy()
        out[k] = a.astype(bool) if k in _capi.PULSE_BOOL or k == "wf_near_threshold" else a
    return out


def reconstruct(adc, n, start_tdc, pedestal_db, calib_area, calib_height, cfg=RecoConfig(), precision="fp64",
                max_pulses=None):
    """Pulses of a batch of (already concatenated) waveforms: adc [W, L] (padded), n [W] valid samples."""
    torch = _torch()
    adc = np.asarray(adc)
    W = adc.shape[0]
    L = adc.shape[1] if adc.ndim == 2 else 0
    period = getattr(cfg, "period", PERIOD)
    P = make_params(reco=cfg, precision=precision)
    P.period = period
    if W == 0:
        out = {k: np.zeros(0) for k in _capi.PULSE_FLOAT}
        out.update({k: np.zeros(0, np.int64) for k in _capi.PULSE_INT})
        out.update({k: np.zeros(0, bool) for k in _capi.PULSE_BOOL + ("wf_near_threshold",)})
        return out
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a).astype(dt))).to("cuda")  # noqa: E731
    off = d(np.arange(W, dtype=np.int64) * L, np.int64)
    res = engine().run(P, off, d(n, np.int32), d(start_tdc, np.int64), d(pedestal_db, np.float64),
                       d(calib_area, np.float64), d(calib_height, np.float64), adc64=d(adc, np.int64),
                       max_pulses=cfg.max_pulses if max_pulses is None else max_pulses)
    return _to_host(res)


def reconstruct_full(adc, n, start_tdc, pedestal_db, calib_area, calib_height, cfg=RecoConfig(), precision="fp64"):
    """Full-length recovery: rounds bounded by the longest waveform."""
    mp = max(cfg.max_pulses, int(np.max(n, initial=0)))
    return reconstruct(adc, n, start_tdc, pedestal_db, calib_area, calib_height, replace(cfg, max_pulses=mp),
                       precision=precision)


def filter_channels(pulses, channels, status, cfg=RecoConfig()):
    """Drop pulses of status-bit-1 (ignored) channels; per-waveform diagnostics are kept."""
    if not cfg.ignore_channels:
        return pulses
    keep = (np.asarray(status)[np.asarray(channels)[pulses["wf"]]] & 0b010) == 0
    return {k: v if k == "wf_near_threshold" else v[keep] for k, v in pulses.items()}


def concat_waveforms(key, bar, sipm, start_tdc, adc_flat, lens):
    """Consecutive digis of one channel whose TDCs continue are one waveform: (group id per digi, padded ADC matrix,
    valid lengths, start TDC and first digi index per group).  Digis of one length L (the digitizer's fixed sample
    count) are copied as whole rows of L samples into a (groups, digis per group, L) view of the matrix."""
    nd = len(bar)
    lens = np.asarray(lens, np.int64)
    cont = np.zeros(nd, bool)
    if nd > 1:
        cont[1:] = ((key[1:] == key[:-1]) & (bar[1:] == bar[:-1]) & (sipm[1:] == sipm[:-1])
                    & (start_tdc[1:] == start_tdc[:-1] + lens[:-1]))
    gid = np.cumsum(~cont) - 1
    G = int(gid[-1]) + 1 if nd else 0
    first = np.flatnonzero(~cont)
    adc_flat = np.asarray(adc_flat)
    if nd and int(lens.min()) == int(lens.max()) and int(lens[0]) > 0 and adc_flat.size == nd * int(lens[0]):
        L = int(lens[0])
        ndig = np.diff(np.append(first, nd))
        glen = ndig * L
        rows = adc_flat.reshape(nd, L)
        if int(ndig.max()) == 1:
            mat = rows.astype(np.int64)
        else:
            pos = np.arange(nd) - np.repeat(first, ndig)
            mat = np.zeros((G, int(ndig.max()), L), np.int64)
            mat[gid, pos] = rows
            mat = mat.reshape(G, -1)
        return gid, mat, glen, start_tdc[first], first
    glen = np.bincount(gid, weights=lens, minlength=G).astype(np.int64)
    begin = np.cumsum(lens) - lens
    offs = begin - begin[first][gid] if nd else np.zeros(0, np.int64)
    mat = np.zeros((G, int(glen.max()) if G else 0), np.int64)
    inner = np.arange(int(lens.sum())) - np.repeat(begin, lens)
    mat[np.repeat(gid, lens), np.repeat(offs, lens) + inner] = np.asarray(adc_flat, np.int64)
    return gid, mat, glen, start_tdc[first], first
