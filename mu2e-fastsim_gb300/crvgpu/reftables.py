"""The CrvRecoTableDumper trees (crv/art/CrvFastSim/src/CrvRecoTableDumper_module.cc, read by
crv/art/CrvFastSim/src/CrvRecoTable.hh): directory ``crvdump/``, rows keyed by (run, subrun, event), channel rows
with ``idx`` (row index in its art collection), ``bar`` and ``sipm``; jagged columns (ADC samples, voltages, charges,
waveform and member indices) as std::vector branches (the art dumper) or counted arrays n<name> (the uproot writer).

The reference reads them with crvfastsim.reco.reftables (read, calib, event_key: crv/crvfastsim/reco/reftables.py:
17-50) into awkward arrays through uproot; here they come back as Tables whose jagged columns are
crvgpu.rootio.JaggedArray.  On top: `write` (counted arrays, the layout CrvRecoTable.hh's Jagged<T> reads),
`conditions` (the chain's Conditions from the calib tree, as Conditions.from_csv takes the CSV dumped from it),
`digis_table`, `pulses_table`, `clusters_table` and `events_table` (the engine's digis, pulses, clusters and
per-event counts in the
dumper's layouts) and `waveforms` (dumped digis -> reco waveforms with
their calibration, the grouping crv/crvfastsim/reco/cli.py:52-74 makes before the pulse fit), so a dumped digi table
goes into chain.clusters / pulsefit.reconstruct_full as it is.
"""
from __future__ import annotations

import numpy as np

from . import rootio
from .config import CHAN_MULT, Conditions
from .tables import KEY, Table, expand

DIR = "crvdump"
TREES = ("events", "charges", "digimc", "digis", "pulses", "clusters", "calib")
NCHAN_PER_BAR = 4


def _concat(parts):
    out = Table()
    for k in parts[0]:
        vs = [p[k] for p in parts]
        if isinstance(vs[0], rootio.JaggedArray):
            vals = np.concatenate([v.values for v in vs])
            offs = np.concatenate([[0]] + [v.offsets[1:] + s for v, s in
                                           zip(vs, np.cumsum([0] + [len(v.values) for v in vs[:-1]]))])
            out[k] = rootio.JaggedArray(vals, offs)
        else:
            out[k] = np.concatenate(vs)
    return out


def read(paths, tree, columns=None, entry_stop=None):
    """One tree concatenated over files (patterns expanded; files without it are skipped); None when no file has it."""
    parts = []
    for p in expand(paths if isinstance(paths, (list, tuple)) else [paths]):
        with rootio.RootFile(p) as f:
            try:
                T = f[f"{DIR}/{tree}"]
            except KeyError:
                continue
            cols = T.arrays(columns)
        if entry_stop is not None:
            cols = {k: (v.take(slice(0, entry_stop)) if isinstance(v, rootio.JaggedArray) else v[:entry_stop])
                    for k, v in cols.items()}
        parts.append(Table(cols))
    return _concat(parts) if parts else None


def calib(paths):
    """Per-channel conditions as dense arrays indexed by offline channel (bar*4 + SiPM): pedestal, pulsearea,
    pulseheight, timeoffset (float, 0 where absent) and status, roc, feb, febch (int64, -1 where absent)."""
    c = read(paths, "calib")
    if c is None:
        raise KeyError(f"no {DIR}/calib tree in {paths}")
    ch = np.asarray(c["channel"], np.int64)
    n = int(ch.max()) + 1 if len(ch) else 0
    out = {k: np.zeros(n, float) for k in ("pedestal", "pulsearea", "pulseheight", "timeoffset")}
    for k in ("status", "roc", "feb", "febch"):
        out[k] = np.full(n, -1, np.int64)
    for k in out:
        out[k][ch] = np.asarray(c[k])
    return out


def event_key(a):
    """One int64 per row combining (run, subrun, event), for joins."""
    return (np.asarray(a["run"]).astype(np.int64) << 40) | (np.asarray(a["subrun"]).astype(np.int64) << 20) | \
        np.asarray(a["event"]).astype(np.int64)


def conditions(paths, deviation=None):
    """The chain's Conditions from the calib tree (the columns Conditions.from_csv reads from its CSV dump)."""
    c = calib(paths)
    n = len(c["pedestal"])
    dev = np.zeros(n) if deviation is None else np.asarray(deviation, float)
    return Conditions(c["pedestal"], c["pulsearea"], c["pulseheight"], c["timeoffset"], c["status"], c["roc"],
                      c["feb"], dev)


def write(path, trees):
    """{tree name: table} into directory crvdump/ of a new ROOT file (jagged columns as counted arrays)."""
    return rootio.write(path, {f"{DIR}/{k}": v for k, v in trees.items()})


def calib_table(cond, febch=None):
    """The calib tree (one row per channel) of a Conditions."""
    n = len(cond.pedestal)
    fc = np.full(n, -1, np.int32) if febch is None else np.asarray(febch, np.int32)
    return {"channel": np.arange(n, dtype=np.int32), "pedestal": np.asarray(cond.pedestal, np.float32),
            "pulsearea": np.asarray(cond.pulsearea, np.float32),
            "pulseheight": np.asarray(cond.pulseheight, np.float32),
            "timeoffset": np.asarray(cond.timeoffset, np.float32), "status": np.asarray(cond.status, np.int32),
            "roc": np.asarray(cond.roc, np.int32), "feb": np.asarray(cond.feb, np.int32), "febch": fc}


def digis_table(D, cond, run=1, febch=None):
    """The digis tree of the engine's digis (chain.digis / waveform.synthesize output: SiPM label, start TDC, ADC
    samples): one row per digi in the given order, idx = its index among its event's digis, nzs 0 (zero-suppressed
    digis), roc/feb/febch of the channel (febch -1 unless given per channel).  run: one run number for every event,
    or {event key: run}."""
    lab = np.asarray(D["chan"], np.int64)
    evk, ch = lab // CHAN_MULT, lab % CHAN_MULT
    if isinstance(run, dict):
        r = np.array([run[int(k)] for k in evk], np.int64)
    else:
        r = np.full(len(lab), int(run), np.int64)
    key = (r << 40) | evk
    o = np.argsort(key, kind="stable")
    new = np.ones(len(lab), bool)
    if len(lab) > 1:
        new[1:] = key[o][1:] != key[o][:-1]
    first = np.flatnonzero(new)
    idx = np.empty(len(lab), np.int64)
    idx[o] = np.arange(len(lab)) - np.repeat(first, np.diff(np.r_[first, len(lab)]))
    adc = np.asarray(D["adc"])
    per = adc.shape[1] if adc.ndim == 2 else 0
    fc = np.full(len(np.asarray(cond.roc)), -1) if febch is None else np.asarray(febch)
    return {"run": r.astype(np.uint32), "subrun": (evk >> 20).astype(np.uint32),
            "event": (evk & ((1 << 20) - 1)).astype(np.uint32), "idx": idx.astype(np.int32),
            "bar": (ch // NCHAN_PER_BAR).astype(np.int32), "sipm": (ch % NCHAN_PER_BAR).astype(np.int32),
            "starttdc": np.asarray(D["starttdc"]).astype(np.int32), "nzs": np.zeros(len(lab), np.int32),
            "roc": np.asarray(cond.roc)[ch].astype(np.int32), "feb": np.asarray(cond.feb)[ch].astype(np.int32),
            "febch": fc[ch].astype(np.int32),
            "adc": rootio.JaggedArray(adc.reshape(-1).astype(np.int16), np.arange(len(lab) + 1, dtype=np.int64) * per)}


def _run_of(evk, run):
    if isinstance(run, dict):
        return np.array([run[int(k)] for k in evk], np.int64)
    return np.full(len(evk), int(run), np.int64)


def clusters_table(out, G, run=1):
    """The clusters tree (crv/art/CrvFastSim/src/CrvRecoTableDumper_module.cc:155-170) of a chain.clusters(...,
    detail=True) result: one row per cluster, in event order; idx = its index among its event's clusters; pulses = its
    member pulses' indices in the event's pulse list, in member order; layers = the distinct layers of their counters,
    increasing; position, side PE, side times and side hit counts as the finder gives them.  G: the SectorGeom (layer
    per counter); run: one run number, or {event key: run}."""
    ev = np.asarray(out["cl_event"], np.int64)
    n = len(ev)
    new = np.ones(n, bool)
    if n > 1:
        new[1:] = ev[1:] != ev[:-1]
    first = np.flatnonzero(new)
    idx = np.arange(n) - np.repeat(first, np.diff(np.r_[first, n]))
    mcl = np.asarray(out["mem_cl"], np.int64)
    o = np.argsort(mcl, kind="stable")
    mcl, midx, mev = mcl[o], np.asarray(out["mem_idx"], np.int64)[o], np.asarray(out["mem_event"], np.int64)[o]
    offs = np.searchsorted(mcl, np.arange(n + 1))
    P = out["pulses"]
    pev = np.asarray(P["ev"], np.int64)
    pstart = np.searchsorted(pev, mev)                  # pulses are grouped by event, idx = position in the event
    layer = np.asarray(G.layer)[np.asarray(P["bar"], np.int64)[pstart + midx]]
    layers = [np.unique(layer[offs[c]:offs[c + 1]]).astype(np.int32) for c in range(n)]
    pos = np.asarray(out["cl_pos"], float).reshape(-1, 3)
    spe = np.asarray(out["cl_sidepe"], float).reshape(-1, 2)
    stm = np.asarray(out["cl_sidetime"], float).reshape(-1, 2)
    shi = np.asarray(out["cl_sidehits"]).reshape(-1, 2)
    return {"run": _run_of(ev, run).astype(np.uint32), "subrun": (ev >> 20).astype(np.uint32),
            "event": (ev & ((1 << 20) - 1)).astype(np.uint32), "idx": idx.astype(np.int32),
            "sectortype": np.asarray(out["cl_type"]).astype(np.int32),
            "start": np.asarray(out["cl_start"], np.float64), "end": np.asarray(out["cl_end"], np.float64),
            "pe": np.asarray(out["cl_pe"]).astype(np.float32), "slope": np.asarray(out["cl_slope"]).astype(np.float32),
            "layers": rootio.JaggedArray.from_rows(layers, np.int32) if n else rootio.JaggedArray(
                np.zeros(0, np.int32), np.zeros(1, np.int64)),
            "pulses": rootio.JaggedArray(midx.astype(np.int32), offs.astype(np.int64)),
            "poscalc": np.asarray(out["cl_poscalc"]).astype(np.int32),
            "avgtime": np.asarray(out["cl_avgtime"], np.float64), "x": pos[:, 0].astype(np.float32),
            "y": pos[:, 1].astype(np.float32), "z": pos[:, 2].astype(np.float32),
            "sidepe0": spe[:, 0].astype(np.float32), "sidepe1": spe[:, 1].astype(np.float32),
            "sidetime0": stm[:, 0], "sidetime1": stm[:, 1], "sidehits0": shi[:, 0].astype(np.int32),
            "sidehits1": shi[:, 1].astype(np.int32)}


def pulses_table(W, P, run=1, digi_len=12):
    """The pulses tree (crv/art/CrvFastSim/src/CrvRecoTableDumper_module.cc:143-154) of reco waveforms W
    (chain.reco_waveforms or waveforms() above) and their pulses P (pulsefit.reconstruct_full, after
    filter_channels and the time offsets as chain.clusters applies them): one row per pulse in (event, waveform,
    sequence) order; idx = its index among its event's pulses; flags bit 0 = failed fit (the bit the reference's reco
    reads); wfidx = the indices of the waveform's digis in their event's digi list (W["digi0"] onwards, one per
    digi_len samples, the digitizer's samples per digi; empty when W has no digi0)."""
    wf = np.asarray(P["wf"], np.int64)
    evw = np.asarray(W["ev"], np.int64)
    ev = evw[wf] & ((1 << 40) - 1)
    o = np.lexsort((np.asarray(P["seq"]), wf, ev))
    wf, ev = wf[o], ev[o]
    n = len(wf)
    new = np.ones(n, bool)
    if n > 1:
        new[1:] = ev[1:] != ev[:-1]
    first = np.flatnonzero(new)
    idx = np.arange(n) - np.repeat(first, np.diff(np.r_[first, n]))
    chan = np.asarray(W["bar"], np.int64)[wf] * NCHAN_PER_BAR + np.asarray(W["sipm"], np.int64)[wf]
    if "digi0" in W:
        L = int(digi_len)
        nd = -(-np.asarray(W["n"], np.int64)[wf] // L)
        d0 = np.asarray(W["digi0"], np.int64)[wf]
        wfidx = rootio.JaggedArray((np.repeat(d0, nd) + np.arange(int(nd.sum())) -
                                    np.repeat(np.cumsum(nd) - nd, nd)).astype(np.int32), np.r_[0, np.cumsum(nd)])
    else:
        wfidx = rootio.JaggedArray(np.zeros(0, np.int32), np.zeros(n + 1, np.int64))
    col = lambda k, dt: np.asarray(P[k])[o].astype(dt)  # noqa: E731
    return {"run": _run_of(ev, run).astype(np.uint32), "subrun": (ev >> 20).astype(np.uint32),
            "event": (ev & ((1 << 20) - 1)).astype(np.uint32), "idx": idx.astype(np.int32),
            "bar": (chan // NCHAN_PER_BAR).astype(np.int32), "sipm": (chan % NCHAN_PER_BAR).astype(np.int32),
            "pe": col("pe", np.float32), "peph": col("peph", np.float32), "height": col("height", np.float32),
            "beta": col("beta", np.float32), "chi2": col("chi2", np.float32), "ped": col("ped", np.float32),
            "time": col("time", np.float64), "letime": col("letime", np.float64), "seq": col("seq", np.int32),
            "flags": col("failed", bool).astype(np.int32), "pedfromdb": col("pedfromdb", bool).astype(np.int32),
            "wfidx": wfidx}


def events_table(event_keys, run=1, ndigi=None, npulse=None, ncluster=None):
    """The events tree (one row per event; spill -1, event length and proton-bunch time 0 for the fast chain's
    off-spill events) with the per-event digi, pulse and cluster counts ({event key: count} or arrays by event)."""
    evk = np.asarray(event_keys, np.int64)

    def per(c):
        if c is None:
            return np.zeros(len(evk), np.int32)
        if isinstance(c, dict):
            return np.array([c.get(int(k), 0) for k in evk], np.int32)
        return np.asarray(c).astype(np.int32)
    return {"run": _run_of(evk, run).astype(np.uint32), "subrun": (evk >> 20).astype(np.uint32),
            "event": (evk & ((1 << 20) - 1)).astype(np.uint32), "spill": np.full(len(evk), -1, np.int32),
            "evlen": np.zeros(len(evk)), "pbtime": np.zeros(len(evk)), "ndigi": per(ndigi), "npulse": per(npulse),
            "ncluster": per(ncluster)}


def waveforms(paths, reco_cfg=None, max_events=None, cond=None):
    """Dumped digis -> reco waveforms: zero-suppressed digis grouped per channel into waveforms in collection order
    (pulsefit.concat_waveforms), status-ignored channels dropped when the reco configuration ignores them,
    calibration from the calib tree (or `cond`).  The keys of chain.reco_waveforms (ev = event_key, bar, sipm, chan,
    adc, n, start, ped, area, height, toff) and of the reference's grouping (digi0 = the first digi's idx, mat = adc,
    events = every event key of the digis)."""
    from .config import RecoConfig
    from .pulsefit import concat_waveforms
    cfg = reco_cfg or RecoConfig()
    d = read(paths, "digis")
    if d is None:
        raise KeyError(f"no {DIR}/digis tree in {paths}")
    ev = event_key(d)
    if max_events:
        keep = np.isin(ev, np.unique(ev)[:max_events])
        d = Table({k: (v.take(keep) if isinstance(v, rootio.JaggedArray) else np.asarray(v)[keep])
                   for k, v in d.items()})
        ev = ev[keep]
    C = calib(paths) if cond is None else {"status": np.asarray(cond.status), "pedestal": np.asarray(cond.pedestal),
                                           "pulsearea": np.asarray(cond.pulsearea),
                                           "pulseheight": np.asarray(cond.pulseheight),
                                           "timeoffset": np.asarray(cond.timeoffset)}
    zs = np.asarray(d["nzs"]) == 0
    adc = d["adc"]
    lens = adc.counts[zs]
    flat = adc.values[np.repeat(zs, adc.counts)]
    bar, sipm = np.asarray(d["bar"])[zs], np.asarray(d["sipm"])[zs]
    gid, mat, n, start, first = concat_waveforms(ev[zs], bar, sipm, np.asarray(d["starttdc"])[zs], flat, lens)
    chan = bar[first] * NCHAN_PER_BAR + sipm[first]
    ok = np.ones(len(first), bool)
    if cfg.ignore_channels:
        ok = ~((np.asarray(C["status"])[chan] >> 1) & 1).astype(bool)
    c = chan[ok]
    key = ev[zs][first][ok]
    return {"ev": key, "bar": c // NCHAN_PER_BAR, "sipm": c % NCHAN_PER_BAR, "chan": c,
            "digi0": np.asarray(d["idx"])[zs][first][ok], "adc": mat[ok], "mat": mat[ok], "n": n[ok],
            "start": start[ok], "ped": np.asarray(C["pedestal"])[c], "area": np.asarray(C["pulsearea"])[c],
            "height": np.asarray(C["pulseheight"])[c], "toff": np.asarray(C["timeoffset"])[c],
            "events": np.unique(ev)}


__all__ = ["DIR", "TREES", "KEY", "read", "calib", "event_key", "conditions", "write", "calib_table", "digis_table",
           "pulses_table", "clusters_table", "events_table", "waveforms"]
