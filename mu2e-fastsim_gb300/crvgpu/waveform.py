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

N_DIGI_PERIODS_GAP = 4        # cluster gap: template length + 4 sampling periods (waveform.py:24, :67)


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

    def run(self, P, tabs: DeviceTables, label, time, charge, tmpl_dev, ev_keys=None, ev_runs=None, max_tries=4,
            tdc0_rows=None):
        """Digis of label-sorted charges.  tdc0_rows (optional, per charge row): the caller's TDC0 of each charge's
        cluster (crv_synthesize); without it TDC0 is the keyed per-(event, FEB) draw (crv_digis)."""
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
            if tdc0_rows is None:
                rc = L.crv_digis(ctypes.byref(P), ctypes.byref(tabs.c_channels()), nq, _capi.ptr(label),
                                 _capi.ptr(time), _capi.ptr(charge), _capi.ptr(tmpl_dev), int(tmpl_dev.numel()),
                                 _capi.ptr(ev_keys), _capi.ptr(ev_runs), 0 if ev_keys is None else int(ev_keys.numel()),
                                 slots, ctypes.byref(D), slots, _capi.ptr(n_out), _capi.ptr(self.ws), self.ws.numel(),
                                 _stream(), self.status.ptr)
                _capi.check(rc, "crv_digis")
            else:
                rc = L.crv_synthesize(ctypes.byref(P), ctypes.byref(tabs.c_channels()), nq, _capi.ptr(label),
                                      _capi.ptr(time), _capi.ptr(charge), _capi.ptr(tdc0_rows), _capi.ptr(tmpl_dev),
                                      int(tmpl_dev.numel()), slots, ctypes.byref(D), slots, _capi.ptr(n_out),
                                      _capi.ptr(self.ws), self.ws.numel(), _stream(), self.status.ptr)
                _capi.check(rc, "crv_synthesize")
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


def charge_clusters(chan, time, wcfg: WaveformConfig):
    """Cluster id of every charge and the first charge row of every cluster (waveform.charge_clusters,
    crv/crvfastsim/reco/waveform.py:65-71): a new cluster where the channel changes or consecutive times are more than
    the template length + 4 periods apart.  The device splits clusters by the same comparisons."""
    chan, time = np.asarray(chan), np.asarray(time, np.float64)
    gap = wcfg.single_pe_max_time + N_DIGI_PERIODS_GAP * wcfg.period
    new = np.ones(len(time), bool)
    if len(time) > 1:
        new[1:] = (chan[1:] != chan[:-1]) | (time[1:] - time[:-1] > gap)
    return np.cumsum(new) - 1, np.flatnonzero(new)


def cluster_table(chan, time, tdc0_cluster, wcfg: WaveformConfig, tmpl, clusters=None):
    """The reference's per-cluster outputs (waveform.py:118-121, 169-172): cluster_chan, cluster_tstart (the first
    FEB tick after the first charge - one period: ceil((t_first - P - TDC0) / P) P + TDC0) and cluster_keep (charges x
    template maximum >= min_voltage), for every cluster, kept or not.  The device forms the same start with the same
    operations for the clusters it synthesises.  clusters: charge_clusters' result when the caller has it."""
    cid, first = clusters if clusters is not None else charge_clusters(chan, time, wcfg)
    P = wcfg.period
    nq = np.bincount(cid, minlength=len(first)) if len(first) else np.zeros(0, np.int64)
    t_first = np.asarray(time, np.float64)[first] - P
    tdc0_cluster = np.asarray(tdc0_cluster, np.float64)
    return {"cluster_chan": np.asarray(chan)[first], "cluster_tstart": np.ceil((t_first - tdc0_cluster) / P) * P
            + tdc0_cluster, "cluster_keep": nq * float(np.max(tmpl)) >= wcfg.min_voltage}


def digis(Q, cond, cfg: ChainConfig, rng, key=None, timers=None, *, stock_scan=False, caps=None, geom=None,
          runs=None):
    """chain.digis: SiPM charges (label-sorted, time-sorted per label) -> digis dict chan, start, tdc0, starttdc,
    volt [D, 12], adc [D, 12], and per charge cluster cluster_chan, cluster_tstart, cluster_keep (as the reference's
    synthesis returns them).  TDC0 is the keyed draw per (event, FEB) (chain.tdc0_per_feb); runs: optional {event
    key: run} for the draw keys (default run 0)."""
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
        geom = _geometry_for(cond)
    tabs = DeviceTables(geom, cond, ccfg)
    P = make_params(ccfg, seed, template_len=len(tmpl))
    lab = np.asarray(Q["chan"], np.int64)
    ek = er = None
    if runs:
        keys = np.array(sorted(runs), np.int64)
        ek = _dev(keys, np.int64)
        er = _dev(np.array([runs[int(k)] for k in keys], np.int64).astype(np.uint32).view(np.int32), np.int32)
    lab_d = _dev(lab, np.int64)
    if lab_d.numel() > 1 and bool((lab_d[1:] < lab_d[:-1]).any()):
        raise ValueError("charges must be sorted by SiPM label (as chain.charges returns them)")
    time_d = _dev(Q["time"], np.float64)
    D = engine().run(P, tabs, lab_d, time_d, _dev(Q["charge"], np.float64), _dev(tmpl, np.float64), ek, er)
    out = _host(D)
    # per-cluster outputs, formed on the device from the uploaded columns with cluster_table's operations
    out.update(_cluster_table_device(P, tabs, lab_d, time_d, wcfg, tmpl, ek, er))
    timers["waveforms_s"] = timers.get("waveforms_s", 0.0) + _time.perf_counter() - t0
    timers["digis"] = timers.get("digis", 0) + len(out["chan"])
    return out


def _dev(a, dt):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).astype(dt, copy=False))).to("cuda")


def _cluster_table_device(P, tabs, lab_d, time_d, wcfg: WaveformConfig, tmpl, ek=None, er=None):
    """cluster_table on device columns (label-sorted charges): the same splits and the same FP64 operations, in
    order, on the device; the keyed TDC0 of each cluster's label (crv_tdc0_per_feb).  Host arrays."""
    torch = _torch()
    n = int(lab_d.numel())
    if n == 0:
        return {"cluster_chan": np.zeros(0, np.int64), "cluster_tstart": np.zeros(0),
                "cluster_keep": np.zeros(0, bool)}
    gap = wcfg.single_pe_max_time + N_DIGI_PERIODS_GAP * wcfg.period
    new = torch.ones(n, dtype=torch.bool, device=lab_d.device)
    new[1:] = (lab_d[1:] != lab_d[:-1]) | ((time_d[1:] - time_d[:-1]) > gap)
    first = torch.nonzero(new).squeeze(1)
    nq = torch.diff(torch.cat([first, torch.tensor([n], device=first.device)]))
    cl_lab = lab_d[first].contiguous()
    tdc0 = _tdc0_device(P, tabs, cl_lab, ek, er, host=False)
    Pd = float(wcfg.period)
    t_first = time_d[first] - Pd
    tstart = torch.ceil((t_first - tdc0) / Pd) * Pd + tdc0
    keep = nq.to(torch.float64) * float(np.max(tmpl)) >= wcfg.min_voltage
    return {"cluster_chan": cl_lab.cpu().numpy(), "cluster_tstart": tstart.cpu().numpy(),
            "cluster_keep": keep.cpu().numpy()}


def _geometry_for(cond):
    from .geometry import module_geometry
    nb = max(1, len(np.asarray(cond.status)) // 4)
    return module_geometry(n_modules=max(1, (nb + 63) // 64))


def _tdc0_device(P, tabs, labels_d, ek=None, er=None, host=True):
    """Keyed TDC0 of device labels (crv_tdc0_per_feb) -> host array (or the device tensor)."""
    torch = _torch()
    L = _capi.load()
    n = int(labels_d.numel())
    out = torch.empty(max(n, 1), dtype=torch.float64, device=labels_d.device)
    st = _capi.DeviceStatus(labels_d.device)
    st.reset()
    _capi.check(L.crv_tdc0_per_feb(ctypes.byref(P), ctypes.byref(tabs.c_channels()), n, _capi.ptr(labels_d),
                                   _capi.ptr(ek), _capi.ptr(er), 0 if ek is None else int(ek.numel()),
                                   _capi.ptr(out), _stream(), st.ptr), "crv_tdc0_per_feb")
    flags, need = st.read()
    raise_status(flags, need, "crv_tdc0_per_feb")
    return out[:n].cpu().numpy() if host else out[:n]


def _part_starts(cid, first, max_charges):
    """Charge rows where synthesize's batches start: whole clusters, a new batch at the first cluster start at or
    after every multiple of max_charges (waveform.py:88-98)."""
    cuts = [0]
    for v in range(max_charges, len(cid), max_charges):
        j = np.searchsorted(first, v)
        if j < len(first) and first[j] > cuts[-1]:
            cuts.append(int(first[j]))
    return cuts + [len(cid)]


def synthesize(chan, time, charge, tdc0_of_chan, cfg=WaveformConfig(), window=(0.0, 1e5), rng=None,
               max_charges=2_000_000, key=None, cond=None):
    """waveform.synthesize (crv/crvfastsim/reco/waveform.py:74-172): zero-suppressed digis of charges grouped by
    channel label (any non-negative integer) and time-ordered within a label.

    tdc0_of_chan: callable or array mapping labels to TDC0 [ns]; as in the reference it is evaluated on the labels of
    the charge clusters, once per batch of whole clusters of at most max_charges charges.  rng None and key None: no
    electronics noise; otherwise noise is keyed by (seed, event, channel, sample tick) with seed = key or a draw from
    rng (the reference draws sequential normals from rng).  Returns per digi chan, start, tdc0, starttdc,
    volt [D, 12], adc [D, 12] sorted by (label, start), and per cluster cluster_chan, cluster_tstart, cluster_keep in
    input order."""
    chan = np.asarray(chan)
    time = np.asarray(time, np.float64)
    charge = np.asarray(charge, np.float64)
    if not (len(chan) == len(time) == len(charge)):
        raise ValueError("chan, time and charge must have the same length")
    if len(chan) and int(np.min(chan)) < 0:
        raise ValueError("channel labels must be non-negative")
    tmpl = single_pe_template(cfg)
    cid, first = charge_clusters(chan, time, cfg)
    # the caller's TDC0 per cluster, evaluated batch by batch as the reference does
    tdc0_cl = np.zeros(len(first))
    cuts = _part_starts(cid, first, int(max_charges)) if len(cid) else [0, 0]
    for a, b in zip(cuts[:-1], cuts[1:]):
        ca, cb = cid[a], cid[b - 1] + 1
        cch = chan[first[ca:cb]]
        tdc0_cl[ca:cb] = tdc0_of_chan(cch) if callable(tdc0_of_chan) else np.asarray(tdc0_of_chan)[cch]
    table = cluster_table(chan, time, tdc0_cl, cfg, tmpl, clusters=(cid, first))
    # the device wants labels ascending: a stable sort keeps every label's time order and its clusters
    lab = chan.astype(np.int64)
    order = None
    if len(lab) > 1 and np.any(np.diff(lab) < 0):
        runs = 1 + int(np.count_nonzero(lab[1:] != lab[:-1]))
        if runs != len(np.unique(lab)):
            raise ValueError("charges must be grouped by channel label (each label's charges contiguous)")
        order = np.argsort(lab, kind="stable")
    rows = tdc0_cl[cid] if len(cid) else np.zeros(0)
    if order is not None:
        lab, time, charge, rows = lab[order], time[order], charge[order], rows[order]
    from .geometry import default_conditions, module_geometry
    nb = int(np.max(lab % CHAN_MULT)) // 4 + 1 if len(lab) else 64
    geom = module_geometry(n_modules=max(1, (nb + 63) // 64))
    cond = cond if cond is not None else default_conditions(geom)
    cc = ChainConfig(waveform=cfg, window=window, noise=rng is not None or key is not None)
    validate_window(cc.window)
    seed = seed_of(rng, key)
    tabs = DeviceTables(geom, cond, cc)
    P = make_params(cc, seed, template_len=len(tmpl))
    D = engine().run(P, tabs, _dev(lab, np.int64), _dev(time, np.float64), _dev(charge, np.float64),
                     _dev(tmpl, np.float64), tdc0_rows=_dev(rows, np.float64))
    out = _host(D)
    out.update(table)
    return out
