"""Waveform stage on the GPU: SiPM charges -> zero-suppressed digis.

Drop-in counterparts of the reference functions:
  single_pe_template(...)   crv/crvfastsim/reco/waveform.py:46-62  (the template file is optional: by default the
                            workload's Gumbel single-PE shape is sampled on the template grid)
  synthesize(chan, time, charge, tdc0_of_chan, cfg, window, rng, ...)   crv/crvfastsim/reco/waveform.py:74
  digis(Q, cond, cfg, rng, key, ...)                                    crv/crvfastsim/chain.py:234

TDC0 per (event, FEB) and the electronics noise are keyed draws (seed, run, subrun, event, FEB / channel, tick).
"""
from __future__ import annotations

import ctypes
import time as _time

import numpy as np

from . import _capi
from .config import CHAN_MULT, ChainConfig, WaveformConfig
from .params import make_params, validate_window
from .response import DeviceTables, _stream, _torch, raise_status, seed_of


def gumbel_raw(peak, mu, beta, precision=0.5, max_time=100.0):
    """(t, v) of the Gumbel single-PE shape peak * e * exp(-z - exp(-z)), z = (t - mu) / beta."""
    t = np.arange(0.0, max_time + precision / 2, precision)
    z = (t - mu) / beta
    return t, peak * np.e * np.exp(-z - np.exp(-z))


def resample(t_raw, v_raw, precision, stretch, max_time):
    """Linear resampling of a (t, v) single-PE table to `precision` ns steps up to max_time (the reference's
    LoadSinglePEWaveform port: first value kept, then one interpolated value per grid point)."""
    t = np.asarray(t_raw, float) * stretch
    v = np.asarray(v_raw, float)
    out = [v[0]]
    k = 1
    for i in range(1, len(t)):
        while t[i] >= k * precision and k * precision < max_time:
            w = (k * precision - t[i - 1]) / (t[i] - t[i - 1])
            out.append((v[i] - v[i - 1]) * w + v[i - 1])
            k += 1
        if k * precision >= max_time:
            break
    return np.asarray(out)


def single_pe_template(cfg: WaveformConfig):
    if cfg.single_pe_file:
        raw = np.loadtxt(cfg.single_pe_file)
        t, v = raw[:, 0], raw[:, 1]
    else:
        t, v = gumbel_raw(cfg.gumbel_peak, cfg.gumbel_mu, cfg.gumbel_beta, cfg.single_pe_precision,
                          cfg.single_pe_max_time)
    return resample(t, v, cfg.single_pe_precision, cfg.single_pe_stretch, cfg.single_pe_max_time)


DIGI_KEYS = ("chan", "start", "tdc0", "starttdc", "volt", "adc")


class DigiEngine:
    """Workspace + launcher of crv_digis on device tensors (fail-closed capacity growth)."""

    def __init__(self, device="cuda"):
        self.device = device
        self.ws = None
        self.slot_factor = 0.5
        self.status = _capi.DeviceStatus(device)

    def run(self, P, tabs: DeviceTables, label, time, charge, tmpl_dev, ev_keys=None, ev_runs=None, max_tries=4):
        torch = _torch()
        L = _capi.load()
        dev = self.device
        nq = int(label.numel())
        zs = int(P.samples_zs)
        for _ in range(max_tries):
            slots = int(max(256, self.slot_factor * nq))
            wsb = L.crv_digis_workspace(ctypes.byref(P), nq, slots)
            if self.ws is None or self.ws.numel() < wsb:
                self.ws = torch.empty(int(wsb * 1.1) + 1024, dtype=torch.uint8, device=dev)
            out = dict(chan=torch.empty(slots, dtype=torch.int64, device=dev),
                       start=torch.empty(slots, dtype=torch.float64, device=dev),
                       tdc0=torch.empty(slots, dtype=torch.float64, device=dev),
                       starttdc=torch.empty(slots, dtype=torch.int64, device=dev),
                       volt=torch.empty((slots, zs), dtype=torch.float64, device=dev),
                       adc=torch.empty((slots, zs), dtype=torch.int16, device=dev))
            n_out = torch.zeros(1, dtype=torch.int64, device=dev)
            self.status.reset()
            D = _capi.CrvDigis(*[_capi.ptr(out[k]) for k in DIGI_KEYS])
            rc = L.crv_digis(ctypes.byref(P), ctypes.byref(tabs.c_channels()), nq, _capi.ptr(label), _capi.ptr(time),
                             _capi.ptr(charge), _capi.ptr(tmpl_dev), int(tmpl_dev.numel()), _capi.ptr(ev_keys),
                             _capi.ptr(ev_runs), 0 if ev_keys is None else int(ev_keys.numel()), slots,
                             ctypes.byref(D), slots, _capi.ptr(n_out), _capi.ptr(self.ws), self.ws.numel(), _stream(),
                             self.status.ptr)
            _capi.check(rc, "crv_digis")
            flags, need = self.status.read()
            nd = need[_capi.NEED["DIGIS"]]
            if flags == _capi.ST_CAPACITY and nd and not need[_capi.NEED["SAMPLES"]]:
                self.slot_factor = 1.2 * nd / max(nq, 1)
                continue
            raise_status(flags, need, "crv_digis")
            n = int(n_out.item())
            return {k: v[:n] for k, v in out.items()}
        raise RuntimeError("crv_digis: capacities did not converge")


_ENGINE = {}


def engine(device="cuda"):
    if device not in _ENGINE:
        _ENGINE[device] = DigiEngine(device)
    return _ENGINE[device]


def _host(D):
    out = {k: v.cpu().numpy() for k, v in D.items()}
    return out


def digis(Q, cond, cfg: ChainConfig, rng, key=None, timers=None, *, stock_scan=False, caps=None, geom=None,
          runs=None):
    """chain.digis: SiPM charges (label-sorted, time-sorted per label) -> digis dict chan, start, tdc0, starttdc,
    volt [D, 12], adc [D, 12].  runs: optional {event key: run} for the draw keys (default run 0)."""
    torch = _torch()
    if stock_scan or caps is not None:
        raise ValueError("stock_scan / caps are options of the reference's JAX synthesis only")
    validate_window(cfg.window)
    timers = timers if timers is not None else {}
    wcfg = cfg.waveform if cfg.waveform is not None else WaveformConfig()
    ccfg = ChainConfig(**{**cfg.__dict__, "waveform": wcfg})
    seed = seed_of(rng, key)
    t0 = _time.perf_counter()
    tmpl = single_pe_template(wcfg)
    if geom is None:
        from .geometry import module_geometry
        nb = max(1, len(np.asarray(cond.status)) // 4)
        geom = module_geometry(n_modules=max(1, (nb + 63) // 64))
    tabs = DeviceTables(geom, cond, ccfg)
    P = make_params(ccfg, seed, template_len=len(tmpl))
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a).astype(dt))).to("cuda")  # noqa: E731
    lab = np.asarray(Q["chan"], np.int64)
    if len(lab) > 1 and np.any(np.diff(lab) < 0):
        raise ValueError("charges must be sorted by SiPM label (as chain.charges returns them)")
    ek = er = None
    if runs:
        keys = np.array(sorted(runs), np.int64)
        ek = d(keys, np.int64)
        er = d(np.array([runs[int(k)] for k in keys], np.int64).astype(np.uint32).view(np.int32), np.int32)
    D = engine().run(P, tabs, d(lab, np.int64), d(Q["time"], np.float64), d(Q["charge"], np.float64),
                     d(tmpl, np.float64), ek, er)
    out = _host(D)
    timers["waveforms_s"] = timers.get("waveforms_s", 0.0) + _time.perf_counter() - t0
    timers["digis"] = timers.get("digis", 0) + len(out["chan"])
    return out


def synthesize(chan, time, charge, tdc0_of_chan, cfg=WaveformConfig(), window=(0.0, 1e5), rng=None,
               max_charges=2_000_000, key=None, cond=None):
    """waveform.synthesize with the engine's keyed TDC0 and noise: tdc0_of_chan is accepted for signature
    compatibility but the TDC0 of every label is the keyed draw of its (event, FEB) (cond gives the FEB map;
    default: 64 channels per FEB).  rng None = no noise."""
    from .geometry import default_conditions, module_geometry
    nb = int(np.max(np.asarray(chan) % CHAN_MULT)) // 4 + 1 if len(chan) else 64
    geom = module_geometry(n_modules=max(1, (nb + 63) // 64))
    cond = cond if cond is not None else default_conditions(geom)
    cc = ChainConfig(waveform=cfg, window=window, noise=rng is not None or key is not None)
    return digis({"chan": chan, "time": time, "charge": charge}, cond, cc, rng, key=key, geom=geom)
