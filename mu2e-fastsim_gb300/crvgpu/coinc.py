"""Coincidence finder on the GPU (crv/crvfastsim/reco/coinc.py: find_event :289, type limits :112-122, SectorCuts,
FinderConfig, SectorGeom :29-79).

find_events runs every event of a flat pulse table in one launch; find_event keeps the reference's one-event
signature and returns the same list of cluster dicts (sectortype, start, end, pe, slope, layers, pulses, poscalc,
avgtime, pos, sidepe, sidetime, sidehits).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from .config import FinderConfig, SectorCuts  # noqa: F401
from .params import make_params
from .response import _stream, _torch, raise_status

CUT_FIELDS = ("pe_threshold", "max_dt_adjacent", "max_dt", "min_slope", "max_slope", "max_slope_diff",
              "coincidence_layers", "min_cluster_pes", "initial_max_distance", "final_max_distance")


def type_limits(G, cfg):
    """Per sector type: readout-end extremes, half length, largest max_dt and instrumented sides."""
    out = {}
    for tt in np.unique(G.sector_type):
        secs = np.flatnonzero(np.asarray(G.sector_type) == tt)
        cuts = [cfg.cuts[G.sector_names[s]] for s in secs if G.sector_names[s] in cfg.cuts]
        if not cuts:
            continue
        p0, p1 = np.asarray(G.pos_side0)[secs].min(), np.asarray(G.pos_side1)[secs].max()
        out[int(tt)] = dict(p0=p0, p1=p1, half=(p1 - p0) / 2, max_dt=max(c.max_dt for c in cuts),
                            side0=bool(np.asarray(G.sipms_side0)[secs].any()),
                            side1=bool(np.asarray(G.sipms_side1)[secs].any()))
    return out


class FinderTables:
    """SectorGeom + cuts flattened on the device (CrvFinderGeom)."""

    def __init__(self, G, cfg: FinderConfig, device="cuda"):
        torch = _torch()
        i32 = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.int32))).to(device)    # noqa: E731
        f64 = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float64))).to(device)  # noqa: E731
        names = list(G.sector_names)
        cut_names = [n for n in names if n in cfg.cuts]
        for n in cut_names:
            if cfg.cuts[n].final_max_distance < 0 or cfg.cuts[n].initial_max_distance < 0:
                raise ValueError("coincidence max distances must be non-negative")
        cut_index = {n: i for i, n in enumerate(cut_names)}
        # the device keeps bar and counter indices in 16 bits, cut-set and type indices in 8 bits
        if len(G.sector) > 65535 or int(np.max(G.counter_in_type, initial=0)) > 65535 or len(cut_names) > 255:
            raise ValueError("coincidence finder: more than 65535 bars or counters per type, or 255 cut sets")
        cuts = np.array([[float(getattr(cfg.cuts[n], f)) for f in CUT_FIELDS] for n in cut_names], float)
        lim = type_limits(G, cfg)
        types = sorted(lim)
        self.bar_sector, self.bar_layer = i32(G.sector), i32(G.layer)
        self.bar_counter = i32(G.counter_in_type)
        self.bar_x, self.bar_y, self.bar_pos = f64(G.x), f64(G.y), f64(np.asarray(G.pos, float).reshape(-1, 3))
        self.sec_type = i32(G.sector_type)
        self.sec_cut = i32([cut_index.get(n, -1) for n in names])
        self.sec_length_dir = i32(G.length_dir)
        self.sec_pos0, self.sec_pos1 = f64(G.pos_side0), f64(G.pos_side1)
        self.cuts = f64(cuts.reshape(-1) if len(cuts) else np.zeros(10))
        self.type_id = i32(types if types else [0])
        self.type_p0 = f64([lim[t]["p0"] for t in types] or [0.0])
        self.type_p1 = f64([lim[t]["p1"] for t in types] or [0.0])
        self.type_half = f64([lim[t]["half"] for t in types] or [0.0])
        self.type_maxdt = f64([lim[t]["max_dt"] for t in types] or [0.0])
        self.type_side0 = i32([lim[t]["side0"] for t in types] or [0])
        self.type_side1 = i32([lim[t]["side1"] for t in types] or [0])
        self.ntypes = len(types)
        if self.ntypes > 255:
            raise ValueError("coincidence finder: more than 255 sector types")

    def update(self, G, cfg: FinderConfig) -> bool:
        """Take the cuts of another finder configuration in place (same device buffers, so a captured chain graph
        that reads them stays valid); False when the tables would change shape (then build new tables)."""
        other = FinderTables(G, cfg, device=self.cuts.device)
        keys = ("sec_cut", "cuts", "type_id", "type_p0", "type_p1", "type_half", "type_maxdt", "type_side0",
                "type_side1")
        if other.ntypes != self.ntypes or any(getattr(other, k).shape != getattr(self, k).shape for k in keys):
            return False
        for k in keys:
            getattr(self, k).copy_(getattr(other, k))
        return True

    def c_geom(self):
        keys = ("bar_sector", "bar_layer", "bar_counter", "bar_x", "bar_y", "bar_pos", "sec_type", "sec_cut",
                "sec_length_dir", "sec_pos0", "sec_pos1", "cuts", "type_id", "type_p0", "type_p1", "type_half",
                "type_maxdt", "type_side0", "type_side1")
        return _capi.CrvFinderGeom(*[_capi.ptr(getattr(self, k)) for k in keys], self.ntypes, 0)


CL_FLOAT = ("pe", "start", "end", "slope", "avgtime")


class CoincEngine:
    def __init__(self, device="cuda"):
        self.device = device
        self.ws = None
        self.status = _capi.DeviceStatus(device)

    def run(self, P, tabs: FinderTables, ev_start, ev_count, ev_key, bar, sipm, seq, time, pe, status):
        torch = _torch()
        L = _capi.load()
        dev = self.device
        nev, np_ = int(ev_start.numel()), int(bar.numel())
        wsb = L.crv_coincidences_workspace(nev, np_)
        if self.ws is None or self.ws.numel() < wsb:
            self.ws = torch.empty(int(wsb * 1.1) + 1024, dtype=torch.uint8, device=dev)
        cap = max(np_, 1)
        out = dict(event=torch.empty(cap, dtype=torch.int64, device=dev),
                   type=torch.empty(cap, dtype=torch.int32, device=dev),
                   **{k: torch.empty(cap, dtype=torch.float64, device=dev) for k in CL_FLOAT},
                   poscalc=torch.empty(cap, dtype=torch.uint8, device=dev),
                   pos=torch.empty((cap, 3), dtype=torch.float64, device=dev),
                   sidepe=torch.empty((cap, 2), dtype=torch.float64, device=dev),
                   sidetime=torch.empty((cap, 2), dtype=torch.float64, device=dev),
                   sidehits=torch.empty((cap, 2), dtype=torch.int32, device=dev),
                   nlayers=torch.empty(cap, dtype=torch.int32, device=dev))
        mem = dict(cl=torch.empty(cap, dtype=torch.int64, device=dev), idx=torch.empty(cap, dtype=torch.int32, device=dev),
                   event=torch.empty(cap, dtype=torch.int64, device=dev))
        n = torch.zeros(2, dtype=torch.int64, device=dev)
        self.status.reset()
        C = _capi.CrvClusters(*[_capi.ptr(out[k]) for k in ("event", "type", "pe", "start", "end", "slope", "avgtime",
                                                            "poscalc", "pos", "sidepe", "sidetime", "sidehits",
                                                            "nlayers")])
        M = _capi.CrvMembers(_capi.ptr(mem["cl"]), _capi.ptr(mem["idx"]), _capi.ptr(mem["event"]))
        r = L.crv_coincidences(ctypes.byref(P), ctypes.byref(tabs.c_geom()), nev, _capi.ptr(ev_start),
                               _capi.ptr(ev_count), _capi.ptr(ev_key), np_, _capi.ptr(bar), _capi.ptr(sipm),
                               _capi.ptr(seq), _capi.ptr(time), _capi.ptr(pe), _capi.ptr(status), ctypes.byref(C),
                               cap, _capi.ptr(n[0:1]), ctypes.byref(M), cap, _capi.ptr(n[1:2]), _capi.ptr(self.ws),
                               self.ws.numel(), _stream(), self.status.ptr)
        _capi.check(r, "crv_coincidences")
        flags, need = self.status.read()
        raise_status(flags, need, "crv_coincidences")
        ncl, nm = (int(v) for v in n.cpu().numpy())
        return {k: v[:ncl] for k, v in out.items()}, {k: v[:nm] for k, v in mem.items()}


_ENGINE = {}


def engine(device="cuda"):
    if device not in _ENGINE:
        _ENGINE[device] = CoincEngine(device)
    return _ENGINE[device]


def find_events(ev, idx, bar, sipm, time, pe, seq, G, status, cfg=FinderConfig(), tabs=None):
    """Clusters of every event of a flat pulse table sorted by event (idx = position inside the event).
    Returns (cluster dict of host arrays, member dict cl/idx/event)."""
    torch = _torch()
    ev = np.asarray(ev, np.int64)
    n = len(ev)
    if n > 1 and np.any(np.diff(ev) < 0):
        raise ValueError("pulses must be grouped by event in increasing order")
    u, start, cnt = np.unique(ev, return_index=True, return_counts=True)
    if n and not np.array_equal(np.asarray(idx, np.int64), np.arange(n) - np.repeat(start, cnt)):
        raise ValueError("idx must be the position of each pulse inside its event")
    T = tabs if tabs is not None else FinderTables(G, cfg)
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a).astype(dt))).to("cuda")  # noqa: E731
    P = make_params(finder=cfg)
    cl, mem = engine().run(P, T, d(start, np.int64), d(cnt, np.int32), d(u, np.int64), d(bar, np.int32),
                           d(sipm, np.int32), d(seq, np.int32), d(time, np.float64), d(pe, np.float64),
                           d(status, np.int32))
    return ({k: v.cpu().numpy() for k, v in cl.items()}, {k: v.cpu().numpy() for k, v in mem.items()})


def rows_of(cl, mem, layers_of=None):
    """Cluster dicts in the reference's find_event format from find_events outputs (one event or many)."""
    rows = []
    order = np.argsort(mem["cl"], kind="stable")
    mcl, midx = mem["cl"][order], mem["idx"][order]
    starts = np.searchsorted(mcl, np.arange(len(cl["pe"])))
    ends = np.searchsorted(mcl, np.arange(len(cl["pe"])), side="right")
    for i in range(len(cl["pe"])):
        rows.append(dict(sectortype=int(cl["type"][i]), start=float(cl["start"][i]), end=float(cl["end"][i]),
                         pe=float(cl["pe"][i]), slope=float(cl["slope"][i]), pulses=list(midx[starts[i]:ends[i]]),
                         poscalc=bool(cl["poscalc"][i]), avgtime=float(cl["avgtime"][i]), pos=cl["pos"][i].copy(),
                         sidepe=list(cl["sidepe"][i]), sidetime=list(cl["sidetime"][i]),
                         sidehits=[int(v) for v in cl["sidehits"][i]], nlayers=int(cl["nlayers"][i])))
    return rows


def find_event(pulses, G, status, cfg=FinderConfig(), vectorized=False):
    """pulses: dict of arrays for ONE event in collection order (idx, bar, sipm, time, pe, seq)."""
    n = len(pulses["idx"])
    cl, mem = find_events(np.zeros(n, np.int64), np.arange(n), pulses["bar"], pulses["sipm"], pulses["time"],
                          pulses["pe"], pulses["seq"], G, status, cfg)
    rows = rows_of(cl, mem)
    idx = np.asarray(pulses["idx"])
    for r in rows:
        r["pulses"] = [int(idx[k]) for k in r["pulses"]]
    return rows
