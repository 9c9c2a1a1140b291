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
    valid lengths, start TDC and first digi index per group)."""
    nd = len(bar)
    lens = np.asarray(lens, np.int64)
    cont = np.zeros(nd, bool)
    if nd > 1:
        cont[1:] = ((key[1:] == key[:-1]) & (bar[1:] == bar[:-1]) & (sipm[1:] == sipm[:-1])
                    & (start_tdc[1:] == start_tdc[:-1] + lens[:-1]))
    gid = np.cumsum(~cont) - 1
    G = int(gid[-1]) + 1 if nd else 0
    glen = np.bincount(gid, weights=lens, minlength=G).astype(np.int64)
    first = np.flatnonzero(~cont)
    begin = np.cumsum(lens) - lens
    offs = begin - begin[first][gid] if nd else np.zeros(0, np.int64)
    mat = np.zeros((G, int(glen.max()) if G else 0), np.int64)
    inner = np.arange(int(lens.sum())) - np.repeat(begin, lens)
    mat[np.repeat(gid, lens), np.repeat(offs, lens) + inner] = np.asarray(adc_flat, np.int64)
    return gid, mat, glen, start_tdc[first], first
