"""Chain glue with the reference's entry points (crv/crvfastsim/chain.py): charges (:151), digis (:234),
reco_waveforms (:273), clusters (:296); plus ChainEngine, the device-resident chain steps -> coincidence clusters
stage by stage (every stage a CUDA launch sequence behind the C ABI; host reads only of the stage sizes).  The
resident engine (crvgpu.resident, crv_chain) runs the same kernels in one call without those reads.

Event key = (subrun << 20) | event; SiPM label = event key * CHAN_MULT + channel (CHAN_MULT 32768).
"""
from __future__ import annotations

import ctypes
import time as _time
from dataclasses import dataclass, replace

import numpy as np

from . import _capi
from .coinc import CoincEngine, FinderTables, rows_of  # noqa: F401
from .config import (CHAN_MULT, PERIOD, ChainConfig, Conditions, FinderConfig, RecoConfig, WaveformConfig,  # noqa: F401
                     from_reference, workload_finder)
from .params import make_params, validate_sipm, validate_window
from .pulsefit import PulseEngine, filter_channels, concat_waveforms
from .pulsefit import engine as _pulse_engine
from .pulsefit import reconstruct_full as _reconstruct_full
from .response import (DeviceSteps, DeviceTables, ResponseEngine, _stream, _torch, charges, raise_status,  # noqa: F401
                       seed_of, upload_steps)
from .waveform import DigiEngine, digis, single_pe_template  # noqa: F401


def tdc0_per_feb(labels, cond, rng, width=PERIOD, key="roc_feb", *, seed=None, runs=None, geom=None):
    """chain.tdc0_per_feb (crv/crvfastsim/chain.py:219-231): TDC0 [ns] of every SiPM label, one uniform x width per
    (event, ROC, FEB) (key "roc_feb") or per (event, FEB) (key "feb").  The draw is the engine's keyed one (seed, run,
    subrun, event, FEB key), the TDC0 chain.digis uses, so it does not depend on which labels are asked for or in which
    order; seed = `seed`, else a draw from rng (the reference draws sequentially from rng in sorted-key order).
    runs: optional {event key: run}.  Same ValueErrors as the reference for the width and the key."""
    from .params import validate_feb_phase
    from .waveform import _dev, _geometry_for, _tdc0_device
    validate_feb_phase(width, key, PERIOD)
    labels = np.asarray(labels, np.int64)
    if len(labels) == 0:
        return np.zeros(0)
    if int(labels.min()) < 0 or int((labels % CHAN_MULT).max()) >= len(np.asarray(cond.status)):
        raise ValueError("labels must be event key * 32768 + a channel of the conditions' channel table")
    cfg = ChainConfig(feb_phase_width=float(width), feb_phase_key=key)
    geom = geom if geom is not None else _geometry_for(cond)
    tabs = DeviceTables(geom, cond, cfg)
    P = make_params(cfg, seed_of(rng, seed))
    ek = er = None
    if runs:
        keys = np.array(sorted(runs), np.int64)
        ek = _dev(keys, np.int64)
        er = _dev(np.array([runs[int(k)] for k in keys], np.int64).astype(np.uint32).view(np.int32), np.int32)
    return _tdc0_device(P, tabs, _dev(labels, np.int64), ek, er)


def reco_waveforms(D, cond):
    """Digis -> reco waveform rows with calibration, sorted by (event, channel, start) (pulsefit.concat_waveforms'
    grouping; host glue as in the reference)."""
    lab, std = np.asarray(D["chan"]), np.asarray(D["starttdc"])
    ev, ch = lab // CHAN_MULT, lab % CHAN_MULT
    # (event, channel) order is label order; chain.digis returns (label, start) order already, which the stable sort
    # would keep as it is
    ordered = len(lab) < 2 or bool(np.all((lab[1:] > lab[:-1]) | ((lab[1:] == lab[:-1]) & (std[1:] >= std[:-1]))))
    if ordered:
        st, adc = std, np.asarray(D["adc"])
    else:
        o = np.lexsort((std, ch, ev))
        ev, ch, st = ev[o], ch[o], std[o]
        adc = np.asarray(D["adc"])[o]
    lens = np.full(len(lab), adc.shape[1] if adc.ndim == 2 else 12, np.int64)
    gid, mat, n, start, first = concat_waveforms(ev, ch // 4, ch % 4, st, adc.ravel(), lens)
    c0 = ch[first]
    return {"ev": ev[first], "bar": c0 // 4, "sipm": c0 % 4, "chan": c0, "adc": mat, "n": n, "start": start,
            "ped": cond.pedestal[c0], "area": cond.pulsearea[c0], "height": cond.pulseheight[c0],
            "toff": cond.timeoffset[c0]}


def clusters(W, cond, geom, counters_cfg, cfg: ChainConfig, timers=None, detail=False, rng=None, caps=None):
    """Reco waveforms -> pulses (GPU) -> coincidence clusters (GPU).  counters_cfg: the SectorGeom of the geometry (or
    None to build it from geom).  Returns ([dict of cl_* arrays (+ members with detail)], timers)."""
    from . import coinc as CO
    from .geometry import sector_geom
    timers = timers if timers is not None else {}
    if caps is not None:
        raise ValueError("capacities are managed by the engine")
    if getattr(cfg, "background", None) is not None:
        raise NotImplementedError("background pulse overlays are not part of the GPU chain")
    if "toff" not in W:
        W = {**W, "toff": cond.timeoffset[W["bar"] * 4 + W["sipm"]]}
    G = counters_cfg if counters_cfg is not None and hasattr(counters_cfg, "sector_type") else sector_geom(geom)
    fcfg = cfg.finder if cfg.finder is not None else workload_finder(G.sector_names)
    rcfg = cfg.pulse_reco if cfg.pulse_reco is not None else RecoConfig()
    adc = np.asarray(W["adc"])
    if adc.ndim != 2 or adc.shape[0] == 0:
        return _clusters_host(W, cond, G, fcfg, rcfg, cfg, timers, detail)
    torch = _torch()
    up = lambda a, dt: torch.from_numpy(np.ascontiguousarray(  # noqa: E731
        np.asarray(a).astype(dt, copy=False))).to("cuda")
    t0 = _time.perf_counter()
    # reconstruct_full (pulsefit.py:222) -> filter_channels (:228) -> DB time offsets and event t0 (chain.py:317-323),
    # on the device: the fit returns its pulses in (waveform, sequence) order, so the reference's
    # lexsort((seq, wf, event)) is a stable sort by event, and none when the waveforms are in event order
    nw, L = adc.shape
    n = np.asarray(W["n"])
    Pp = make_params(reco=rcfg, precision=cfg.precision)
    Pp.period = getattr(rcfg, "period", PERIOD)
    res = _pulse_engine().run(Pp, torch.arange(nw, dtype=torch.int64, device="cuda") * L, up(n, np.int32),
                              up(W["start"], np.int64), up(W["ped"], np.float64), up(W["area"], np.float64),
                              up(W["height"], np.float64), adc64=up(adc, np.int64),
                              max_pulses=max(rcfg.max_pulses, int(n.max(initial=0))))
    wf, time, pe, seq = res["wf"], res["time"], res["pe"], res["seq"]
    if rcfg.ignore_channels:
        keep = (up(cond.status, np.int64)[up(W["bar"] * 4 + W["sipm"], np.int64)[wf]] & 0b010) == 0
        wf, time, pe, seq = wf[keep], time[keep], pe[keep], seq[keep]
    if rcfg.use_time_offset_db:
        time = time + up(W["toff"], np.float64)[wf] * rcfg.time_offset_scale
    if "event_t0" in W:
        time = time + up(W["event_t0"], np.float64)[wf]
    ev = up(W["ev"], np.int64)[wf]
    if ev.numel() > 1 and bool((ev[1:] < ev[:-1]).any()):
        o = torch.sort(ev, stable=True).indices
        ev, wf, time, pe, seq = ev[o], wf[o], time[o], pe[o], seq[o]
    torch.cuda.synchronize()
    timers["pulses_s"] = timers.get("pulses_s", 0.0) + _time.perf_counter() - t0
    t0 = _time.perf_counter()
    u, cnt = torch.unique_consecutive(ev, return_counts=True)
    start = torch.cumsum(cnt, 0) - cnt
    status = up(cond.status, np.int32)
    cl, mem = CO.engine().run(make_params(finder=fcfg), CO.FinderTables(G, fcfg), start, cnt.to(torch.int32), u,
                              up(W["bar"], np.int32)[wf], up(W["sipm"], np.int32)[wf], seq.to(torch.int32), time, pe,
                              status)
    cl = {k: v.cpu().numpy() for k, v in cl.items()}
    mem = {k: v.cpu().numpy() for k, v in mem.items()}
    timers["coinc_s"] = timers.get("coinc_s", 0.0) + _time.perf_counter() - t0
    timers["pulses"] = timers.get("pulses", 0) + int(ev.numel())
    pulses = None
    if detail:
        wf_h, ev_h = wf.cpu().numpy(), ev.cpu().numpy()
        st_h, cnt_h = start.cpu().numpy(), cnt.cpu().numpy()
        pulses = dict(ev=ev_h, idx=np.arange(len(ev_h)) - np.repeat(st_h, cnt_h), bar=W["bar"][wf_h],
                      sipm=W["sipm"][wf_h], seq=seq.cpu().numpy(), pe=pe.cpu().numpy(), time=time.cpu().numpy())
    return [_cluster_out(cl, mem, detail, pulses)], timers


def _clusters_host(W, cond, G, fcfg, rcfg, cfg, timers, detail):
    """clusters for a batch with no reco waveforms (or a non-matrix ADC table): the host sequence of the reference's
    calls, each on the GPU."""
    from . import coinc as CO
    t0 = _time.perf_counter()
    P = _reconstruct_full(W["adc"], W["n"], W["start"], W["ped"], W["area"], W["height"], rcfg,
                          precision=cfg.precision)
    P = filter_channels(P, W["bar"] * 4 + W["sipm"], cond.status, rcfg)
    if rcfg.use_time_offset_db:
        P["time"] = P["time"] + W["toff"][P["wf"]] * rcfg.time_offset_scale
    if "event_t0" in W:
        P["time"] = P["time"] + W["event_t0"][P["wf"]]
    timers["pulses_s"] = timers.get("pulses_s", 0.0) + _time.perf_counter() - t0
    wf = P["wf"]
    ev = W["ev"][wf]
    o = np.lexsort((P["seq"], wf, ev))
    ev, wf = ev[o], wf[o]
    idx = np.arange(len(ev)) - np.searchsorted(ev, ev)
    bar, sipm, time, pe, seq = W["bar"][wf], W["sipm"][wf], P["time"][o], P["pe"][o], P["seq"][o]
    t0 = _time.perf_counter()
    cl, mem = CO.find_events(ev, idx, bar, sipm, time, pe, seq, G, cond.status, fcfg)
    timers["coinc_s"] = timers.get("coinc_s", 0.0) + _time.perf_counter() - t0
    timers["pulses"] = timers.get("pulses", 0) + len(ev)
    pulses = dict(ev=ev, idx=idx, bar=bar, sipm=sipm, seq=seq, pe=pe, time=time) if detail else None
    return [_cluster_out(cl, mem, detail, pulses)], timers


def _cluster_out(cl, mem, detail, pulses):
    out = {"cl_event": cl["event"], "cl_type": cl["type"].astype(np.int64), "cl_pe": cl["pe"], "cl_start": cl["start"],
           "cl_end": cl["end"], "cl_slope": cl["slope"], "cl_avgtime": cl["avgtime"],
           "cl_poscalc": cl["poscalc"].astype(bool)}
    if detail:
        out.update({"mem_cl": mem["cl"], "mem_idx": mem["idx"].astype(np.int64), "mem_event": mem["event"],
                    "cl_pos": cl["pos"], "cl_sidepe": cl["sidepe"], "cl_sidetime": cl["sidetime"],
                    "cl_sidehits": cl["sidehits"], "cl_nlayers": cl["nlayers"], "pulses": pulses})
    return out


# ---------------------------------------------------------------------------------------------------------------------
# device-resident chain

class _Ws:
    """Grow-only device workspace."""

    def __init__(self, device):
        self.device, self.t = device, None

    def get(self, nbytes):
        torch = _torch()
        if self.t is None or self.t.numel() < nbytes:
            self.t = torch.empty(int(nbytes * 1.1) + 1024, dtype=torch.uint8, device=self.device)
        return self.t


@dataclass
class ChainResult:
    n_events: int
    n_charges: int
    n_digis: int
    n_waveforms: int
    n_pulses: int
    n_hits: int
    n_clusters: int
    n_members: int
    clusters: dict
    members: dict
    n_photons: int = 0
    n_sipms: int = 0
    charges: object = None
    seed: int = 0
    ev_keys: object = None
    ev_runs: object = None
    digis: dict = None
    waveforms: dict = None
    pulses: dict = None
    hits: dict = None


class ChainEngine:
    """steps (DeviceSteps) -> charges -> digis -> reco waveforms -> pulses -> coincidence clusters, on the device."""

    def __init__(self, geom, cond, cfg: ChainConfig, G=None, device="cuda", pmap=None):
        from .coinc import FinderTables
        from .geometry import sector_geom
        torch = _torch()
        validate_sipm(cfg.sipm)
        validate_window(cfg.window)
        self.cfg = cfg
        self.device = device
        self.geom, self.cond, self.pmap = geom, cond, pmap
        self.G = G if G is not None else sector_geom(geom)
        self.wcfg = cfg.waveform if cfg.waveform is not None else WaveformConfig()
        self.rcfg = cfg.pulse_reco if cfg.pulse_reco is not None else RecoConfig()
        self.fcfg = cfg.finder if cfg.finder is not None else workload_finder(self.G.sector_names)
        self.ccfg = replace(cfg, waveform=self.wcfg, pulse_reco=self.rcfg, finder=self.fcfg)
        self.tabs = DeviceTables(geom, cond, self.ccfg, device, pmap)
        self.fin = FinderTables(self.G, self.fcfg, device)
        tm = single_pe_template(self.wcfg)
        self.tmpl = torch.from_numpy(tm).to(device)
        self.tlen = len(tm)
        self.resp, self.dig, self.pul, self.coi = (ResponseEngine(device), DigiEngine(device), PulseEngine(device),
                                                   CoincEngine(device))
        self.ws_w, self.ws_h = _Ws(device), _Ws(device)
        self.status = _capi.DeviceStatus(device)

    def configure(self, cfg: ChainConfig):
        """Switch to another design point: knobs carried in the launch parameters change freely; the finder tables
        and the single-PE template are rebuilt when their settings change, the channel tables when the response
        scales or SiPM settings do."""
        from .coinc import FinderTables
        torch = _torch()
        validate_sipm(cfg.sipm)
        validate_window(cfg.window)
        wcfg = cfg.waveform if cfg.waveform is not None else WaveformConfig()
        rcfg = cfg.pulse_reco if cfg.pulse_reco is not None else RecoConfig()
        fcfg = cfg.finder if cfg.finder is not None else workload_finder(self.G.sector_names)
        ccfg = replace(cfg, waveform=wcfg, pulse_reco=rcfg, finder=fcfg)
        old = self.ccfg
        if (cfg.sipm != old.sipm or cfg.response.photon_yield_scale != old.response.photon_yield_scale
                or cfg.response.photon_yield_variation_scale != old.response.photon_yield_variation_scale):
            self.tabs = DeviceTables(self.geom, self.cond, ccfg, self.device, self.pmap)
        if fcfg != self.fcfg and not self.fin.update(self.G, fcfg):
            self.fin = FinderTables(self.G, fcfg, self.device)
        shape = ("single_pe_file", "single_pe_precision", "single_pe_stretch", "single_pe_max_time", "gumbel_peak",
                 "gumbel_mu", "gumbel_beta")
        if any(getattr(wcfg, k) != getattr(self.wcfg, k) for k in shape):
            tm = single_pe_template(wcfg)
            self.tmpl = torch.from_numpy(tm).to(self.device)
            self.tlen = len(tm)
        self.cfg, self.ccfg, self.wcfg, self.rcfg, self.fcfg = cfg, ccfg, wcfg, rcfg, fcfg

    def release(self):
        """Drop the stage workspaces (tables, configuration and the sizes learned so far stay; the next run allocates
        again)."""
        for e in (self.resp, self.dig, self.pul, self.coi):
            e.ws = None
        self.ws_w.t = self.ws_h.t = None

    def params(self, seed):
        P = make_params(self.ccfg, seed, template_len=self.tlen, uniform_map=self.tabs.uniform_map)
        P.period = self.wcfg.period
        return P

    def run(self, ds: DeviceSteps, seed, keep=False, diagnostics=False, charges=None):
        """One pass of the chain over ds.  diagnostics: also count photons and hit SiPMs (n_photons, n_sipms).
        charges: the batch's SiPM charges from elsewhere (device columns label, time, charge, pe, photon in label and
        time order, e.g. chain.charges with lookup tables), which replace the response stage."""
        torch = _torch()
        L = _capi.load()
        dev = self.device
        P = self.params(seed)
        if charges is None:
            R = self.resp.run(P, ds, self.tabs, diagnostics=diagnostics)
        else:
            from types import SimpleNamespace
            R = SimpleNamespace(**{k: charges[k] for k in ("label", "time", "charge", "pe", "photon")},
                                n=int(charges["label"].numel()), nsipm=0, sipm_photons=None)
            diagnostics = False
        evk = ((ds.ev_subrun.to(torch.int64) & 0xFFFFFFFF) << 20) | (ds.ev_event.to(torch.int64) & 0xFFFFFFFF)
        D = self.dig.run(P, self.tabs, R.label, R.time, R.charge, self.tmpl, evk, ds.ev_run)
        nd = int(D["chan"].numel())
        # reco waveforms
        W = {k: torch.empty(max(nd, 1), dtype=dt, device=dev) for k, dt in
             (("label", torch.int64), ("off", torch.int64), ("n", torch.int32), ("start", torch.int64),
              ("ped", torch.float64), ("area", torch.float64), ("height", torch.float64), ("toff", torch.float64))}
        nw_t = torch.zeros(1, dtype=torch.int64, device=dev)
        self.status.reset()
        ws = self.ws_w.get(L.crv_reco_waveforms_workspace(nd))
        _capi.check(L.crv_reco_waveforms(ctypes.byref(P), ctypes.byref(self.tabs.c_channels()), nd,
                                         _capi.ptr(D["chan"]), _capi.ptr(D["starttdc"]),
                                         *[_capi.ptr(W[k]) for k in ("label", "off", "n", "start", "ped", "area",
                                                                      "height", "toff")],
                                         _capi.ptr(nw_t), _capi.ptr(ws), ws.numel(), _stream(), self.status.ptr),
                    "crv_reco_waveforms")
        nw = int(nw_t.item())
        W = {k: v[:nw] for k, v in W.items()}
        adc16 = D["adc"].reshape(-1)
        Pu = self.pul.run(P, W["off"], W["n"], W["start"], W["ped"], W["area"], W["height"], adc16=adc16,
                          max_pulses=2 ** 31 - 1, nsamples=adc16.numel())
        npu = int(Pu["wf"].numel())
        # finder input
        H = dict(ev_start=torch.empty(max(npu, 1), dtype=torch.int64, device=dev),
                 ev_count=torch.empty(max(npu, 1), dtype=torch.int32, device=dev),
                 ev_key=torch.empty(max(npu, 1), dtype=torch.int64, device=dev),
                 bar=torch.empty(max(npu, 1), dtype=torch.int32, device=dev),
                 sipm=torch.empty(max(npu, 1), dtype=torch.int32, device=dev),
                 seq=torch.empty(max(npu, 1), dtype=torch.int32, device=dev),
                 time=torch.empty(max(npu, 1), dtype=torch.float64, device=dev),
                 pe=torch.empty(max(npu, 1), dtype=torch.float64, device=dev))
        nn = torch.zeros(2, dtype=torch.int64, device=dev)
        ws = self.ws_h.get(L.crv_pulse_hits_workspace(npu))
        _capi.check(L.crv_pulse_hits(ctypes.byref(P), _capi.ptr(self.tabs.status), nw, _capi.ptr(W["label"]),
                                     _capi.ptr(W["toff"]), None, npu, _capi.ptr(Pu["wf"]), _capi.ptr(Pu["seq"]),
                                     _capi.ptr(Pu["time"]), _capi.ptr(Pu["pe"]),
                                     *[_capi.ptr(H[k]) for k in ("ev_start", "ev_count", "ev_key", "bar", "sipm",
                                                                  "seq", "time", "pe")],
                                     _capi.ptr(nn[0:1]), _capi.ptr(nn[1:2]), _capi.ptr(ws), ws.numel(), _stream(),
                                     self.status.ptr), "crv_pulse_hits")
        flags, need = self.status.read()
        raise_status(flags, need, "chain glue")
        nev, nh = (int(v) for v in nn.cpu().numpy())
        H = {k: (v[:nev] if k.startswith("ev_") else v[:nh]) for k, v in H.items()}
        cl, mem = self.coi.run(P, self.fin, H["ev_start"], H["ev_count"], H["ev_key"], H["bar"], H["sipm"],
                               H["seq"], H["time"], H["pe"], self.tabs.status)
        res = ChainResult(ds.nevents, R.n, nd, nw, npu, nh, int(cl["pe"].numel()), int(mem["cl"].numel()), cl, mem,
                          int(R.sipm_photons.sum().item()) if diagnostics and R.nsipm else 0,
                          R.nsipm if diagnostics else 0)
        if keep:
            res.charges, res.digis, res.waveforms, res.pulses, res.hits = R, D, W, Pu, H
            res.seed, res.ev_keys, res.ev_runs = seed, evk, ds.ev_run
        return res
