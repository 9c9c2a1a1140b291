"""Resident chain: steps -> coincidence clusters in one C call (crv_chain) per batch, replayed as a CUDA graph.

Modelled on the reference's resident CRV adapter (mixing/device_crv.py:127-573; mixing/DEVICE_CRV.md, "Explicit
capacities" and "Every true error flag rejects the entire batch"):

* capacities are explicit static bounds (ChainCaps: every entry a positive int, no entry missing or unknown), not
  physics cuts;
* a batch is copied into static device buffers sized by them (fewer events: the remaining event rows carry no steps;
  fewer steps: the step count is read on the device), so every batch replays the same captured graph;
* nothing is read back while a batch runs: one read after the replay fetches the stage counts and the status block,
  and any status flag rejects the whole batch (BatchRejected, with the sizes it needed).  With grow=True the engine
  instead enlarges the capacities from those sizes, captures again and re-runs the batch (the reference has no
  automatic retry; here it is opt-in).

The result of a batch is the same, bit for bit, as ChainEngine.run on the same steps and seed: the same kernels run
on the same data, only the sizes come from the device.
"""
from __future__ import annotations

import ctypes
import threading
from dataclasses import dataclass, fields, replace

import numpy as np

from . import _capi
from .response import DeviceSteps, EngineError, _stream, _torch

INT64_MAX = (1 << 63) - 1

# one stream capture at a time in the process: entering a capture synchronises the device, which another thread's
# capture in progress does not permit
_CAPTURE_LOCK = threading.Lock()


@dataclass(frozen=True)
class ChainCaps:
    """Capacities of one resident-chain batch (CrvChainCaps)."""
    events: int                   # rows of the event table
    steps: int                    # rows of the step table
    photons: int                  # photons of a batch
    charges: int                  # SiPM charges
    slots: int                    # digi slots before zero suppression
    digis: int                    # digis (bounds the reco waveforms)
    pulses: int                   # pulses (bounds finder hits, clusters and members)
    max_steps_per_event: int      # largest event of any batch

    def __post_init__(self):
        for f in fields(self):
            v = getattr(self, f.name)
            if type(v) is not int or v < 1:
                raise ValueError(f"chain capacity {f.name} must be a positive int, got {v!r}")
        if self.max_steps_per_event > 32768:
            raise ValueError("chain capacity max_steps_per_event: at most 32768 steps per event")

    @classmethod
    def from_dict(cls, d):
        names = {f.name for f in fields(cls)}
        missing, extra = names - set(d), set(d) - names
        if missing or extra:
            raise ValueError(f"explicit chain capacities required; missing={sorted(missing)}, extra={sorted(extra)}")
        return cls(**d)

    def as_dict(self):
        return {f.name: getattr(self, f.name) for f in fields(self)}

    @classmethod
    def from_counts(cls, counts, events, steps, max_steps_per_event, margin=1.25):
        """Capacities from the stage counts of a trial batch (ResidentChain.last_counts or a dict with the same keys)
        with a margin for batch-to-batch spread."""
        m = lambda k: int(max(1024, np.ceil(margin * int(counts[k]))))  # noqa: E731
        return cls(events=int(events), steps=int(steps), photons=m("photons"), charges=m("charges"),
                   slots=m("slots"), digis=m("digis"), pulses=m("pulses"),
                   max_steps_per_event=int(max_steps_per_event))

    def grown(self, need, margin=1.25):
        """Capacities enlarged to the sizes a rejected batch needed (status need[] slots)."""
        N = _capi.NEED
        up = lambda cur, v: max(cur, int(np.ceil(margin * int(v)))) if v else cur  # noqa: E731
        photons = up(self.photons, need[N["PHOTONS_TOTAL"]])
        if need[N["SLOTS_TOTAL"]] and not need[N["PHOTONS_TOTAL"]]:
            photons = int(np.ceil(photons * margin))          # the SiPM slots scale with the photon capacity
        pulses = max(up(self.pulses, need[N["PULSES_OUT"]]), up(self.pulses, need[N["CLUSTERS"]]),
                     up(self.pulses, need[N["MEMBERS"]]))
        mspe = self.max_steps_per_event
        if need[N["STEPS_PER_EVENT"]]:
            mspe = min(32768, max(mspe, int(need[N["STEPS_PER_EVENT"]])))
        return replace(self, photons=photons, charges=up(self.charges, need[N["CHARGES_OUT"]]),
                       slots=up(self.slots, need[N["DIGIS"]]), digis=up(self.digis, need[N["DIGIS_OUT"]]),
                       pulses=pulses, max_steps_per_event=mspe)

    def c(self):
        return _capi.CrvChainCaps(self.events, self.steps, self.photons, self.charges, self.slots, self.digis,
                                  self.pulses, self.max_steps_per_event, 0)


def caps_for(engine, batches, margin=1.0):
    """Starting capacities for batches of a ChainEngine's workload, from the sizes its stage engines have learned
    (photons per step, charges per photon, digi slots per charge, pulses per digi); a resident chain with grow=True
    corrects them on the first batch."""
    ns = max(int(b.nsteps) for b in batches)
    up = lambda v: int(max(1024, np.ceil(margin * v)))  # noqa: E731
    photons = up(engine.resp.photon_per_step * ns)
    charges = up(engine.resp.out_factor * photons)
    slots = up(engine.dig.slot_factor * charges)
    return ChainCaps(events=max(int(b.nevents) for b in batches), steps=ns, photons=photons, charges=charges,
                     slots=slots, digis=slots, pulses=up(engine.pul.out_factor * slots),
                     max_steps_per_event=max(1, min(32768, max(int(b.max_steps) for b in batches))))


class BatchRejected(EngineError):
    """A batch of the resident chain set a status flag: its outputs are not a result."""

    def __init__(self, flags, need, counts):
        self.flags, self.need, self.counts = int(flags), need, dict(counts)
        named = {k: int(need[v]) for k, v in _capi.NEED.items() if need[v]}
        super().__init__(f"resident chain batch rejected: {_capi.status_string(flags)} (needed {named})")


@dataclass
class ResidentResult:
    n_events: int
    counts: dict                  # stage counts (CHAIN_COUNTS)
    clusters: dict                # device cluster columns (copies, valid after later batches)
    members: dict


class ResidentChain:
    """Steps -> clusters on one device with explicit capacities; graph=True replays one captured CUDA graph per batch
    (crv_chain_graph_*: captured on the first batch, again only after a capacity change or a configuration change
    beyond the serving knobs; seeds and knobs are written into the graph's kernels).  Captures are serialised in the
    process and run in thread-local mode, so other host threads keep launching meanwhile."""

    def __init__(self, engine, caps: ChainCaps, real_dtype=None, graph=True, grow=False, max_grow=4, lookup=None):
        """engine: a ChainEngine (its tables, finder, template and configuration are used).  lookup: a LookupModel
        (crvgpu.lookup) of the engine's geometry: the photons then come from the lookup-table model (crv_chain_lookup,
        as chain.charges with lookup tables), and every batch also needs its steps in the model's form (run(...,
        lookup_steps=LookupModel.upload_steps(steps, pdg)))."""
        torch = _torch()
        self.eng = engine
        self.lookup = lookup
        if lookup is not None and len(lookup.groups) > _capi.LOOKUP_CHAIN_GROUPS:
            raise ValueError(f"the resident chain takes at most {_capi.LOOKUP_CHAIN_GROUPS} lookup groups")
        self.device = engine.device
        self.graph_mode, self.grow, self.max_grow = bool(graph), bool(grow), int(max_grow)
        self.real_dtype = real_dtype if real_dtype is not None else torch.float32
        self.status = _capi.DeviceStatus(self.device)
        self.counts = torch.zeros(10, dtype=torch.int64, device=self.device)
        self.last_counts = None
        self.launches_per_run = 0
        self.replays = 0                # graph replays (kernel launches of a replay: launches_per_run)
        self.captures = 0               # graph captures (a new seed or knob set needs none)
        self._graph, self._graph_key, self._side = None, None, None
        self._warm = False
        self._alloc(caps)

    # -- buffers ----------------------------------------------------------------------------------------------------
    def _alloc(self, caps: ChainCaps):
        torch = _torch()
        L = _capi.load()
        dev, c = self.device, caps
        self.caps = caps
        self._drop_graph()
        # the previous buffers go first (called between batches, nothing in flight): growth does not need both sets
        self.ws = self.st = self.cl = self.mem = self.ev = None
        i32, i64, f64, rd = torch.int32, torch.int64, torch.float64, self.real_dtype
        self.ev = dict(event=torch.zeros(c.events, dtype=i32, device=dev),
                       subrun=torch.zeros(c.events, dtype=i32, device=dev),
                       run=torch.zeros(c.events, dtype=i32, device=dev),
                       first=torch.zeros(c.events, dtype=i64, device=dev),
                       nsteps=torch.zeros(c.events, dtype=i32, device=dev),
                       key=torch.full((c.events,), INT64_MAX, dtype=i64, device=dev))
        self.st = {k: torch.zeros(c.steps, dtype=rd, device=dev) for k in ("x", "y", "z", "t", "edep")}
        self.st["bar"] = torch.zeros(c.steps, dtype=i32, device=dev)
        self.lst = None
        if self.lookup is not None:                     # the steps in the lookup model's form (bar: self.st's)
            self.lst = {k: torch.zeros(c.steps, dtype=f64, device=dev) for k in _capi.LOOKUP_STEP_COLS}
            self.lst["pdg"] = torch.zeros(c.steps, dtype=i64, device=dev)
        self.nsteps_dev = torch.zeros(1, dtype=i64, device=dev)
        cap = c.pulses
        self.cl = dict(event=torch.empty(cap, dtype=i64, device=dev), type=torch.empty(cap, dtype=i32, device=dev),
                       **{k: torch.empty(cap, dtype=f64, device=dev) for k in ("pe", "start", "end", "slope",
                                                                                "avgtime")},
                       poscalc=torch.empty(cap, dtype=torch.uint8, device=dev),
                       pos=torch.empty((cap, 3), dtype=f64, device=dev),
                       sidepe=torch.empty((cap, 2), dtype=f64, device=dev),
                       sidetime=torch.empty((cap, 2), dtype=f64, device=dev),
                       sidehits=torch.empty((cap, 2), dtype=i32, device=dev),
                       nlayers=torch.empty(cap, dtype=i32, device=dev))
        self.mem = dict(cl=torch.empty(cap, dtype=i64, device=dev), idx=torch.empty(cap, dtype=i32, device=dev),
                        event=torch.empty(cap, dtype=i64, device=dev))
        P = self.eng.params(1)
        wsb = self._workspace_bytes(P, caps)
        if wsb < 0:
            raise ValueError("crv_chain_workspace: invalid capacities")
        self.ws = torch.empty(int(wsb) + 1024, dtype=torch.uint8, device=dev)
        self._C = _capi.CrvClusters(*[_capi.ptr(self.cl[k]) for k in ("event", "type", "pe", "start", "end", "slope",
                                                                      "avgtime", "poscalc", "pos", "sidepe",
                                                                      "sidetime", "sidehits", "nlayers")])
        self._M = _capi.CrvMembers(_capi.ptr(self.mem["cl"]), _capi.ptr(self.mem["idx"]), _capi.ptr(self.mem["event"]))
        rb = 4 if self.st["x"].dtype.itemsize == 4 else 8
        self._S = _capi.CrvSteps(*[_capi.ptr(self.st[k]) for k in ("x", "y", "z", "t", "edep", "bar")], rb, 0)
        self._E = _capi.CrvEvents(*[_capi.ptr(self.ev[k]) for k in ("event", "subrun", "run", "first", "nsteps")])
        self._LK = self._lookup_c() if self.lookup is not None else None
        self.nbytes = int(self.ws.numel()) + sum(int(t.numel() * t.element_size()) for d in
                                                 (self.ev, self.st, self.cl, self.mem, self.lst or {})
                                                 for t in d.values())

    def _workspace_bytes(self, P, caps):
        L = _capi.load()
        f = L.crv_chain_lookup_workspace if self.lookup is not None else L.crv_chain_workspace
        return f(ctypes.byref(P), ctypes.byref(caps.c()))

    def _lookup_c(self):
        """CrvLookupChain of the model over the static step buffers."""
        m = self.lookup
        K = _capi.CrvLookupChain()
        K.steps = _capi.CrvLookupSteps(*[_capi.ptr(self.lst[k]) for k in _capi.LOOKUP_STEP_COLS],
                                       _capi.ptr(self.st["bar"]), _capi.ptr(self.lst["pdg"]))
        K.ngroups = len(m.groups)
        for i, g in enumerate(m.groups):
            K.group[i] = m._group_c(g)
            K.table[i] = g["DL"].c(m.precision)
        return K

    def configure(self, cfg):
        """Switch the engine to another design point.  The serving knobs (photon yield, attenuation, threshold, finder
        window) reach a captured graph without a new capture; other changes capture again on the next batch."""
        self.eng.configure(cfg)
        P = self.eng.params(1)
        if self._workspace_bytes(P, self.caps) > self.ws.numel():
            self._alloc(self.caps)

    def load(self, ds: DeviceSteps, lookup_steps=None):
        """Copy a batch into the static buffers (device copies on the current stream).  lookup_steps: the batch's
        steps in the lookup model's form (LookupModel.upload_steps), in the order of ds's rows (lookup model only)."""
        if (self.lookup is not None) != (lookup_steps is not None):
            raise ValueError("the lookup-table chain takes every batch's lookup_steps; the analytic chain none")
        c = self.caps
        over = ds.nevents > c.events or ds.nsteps > c.steps or ds.max_steps > c.max_steps_per_event
        if over and self.grow and ds.max_steps <= 32768:
            up = lambda cur, v: max(cur, int(np.ceil(1.25 * v)))  # noqa: E731
            self._alloc(replace(c, events=up(c.events, ds.nevents), steps=up(c.steps, ds.nsteps),
                                max_steps_per_event=min(32768, up(c.max_steps_per_event, ds.max_steps))))
            c, over = self.caps, False
        if over:
            raise ValueError(f"batch of {ds.nevents} events / {ds.nsteps} steps / {ds.max_steps} steps per event "
                             f"exceeds the chain capacities {c.events} / {c.steps} / {c.max_steps_per_event}")
        if ds.x.dtype != self.real_dtype:
            raise ValueError(f"step table dtype {ds.x.dtype} differs from the chain's {self.real_dtype}")
        n, e = ds.nsteps, ds.nevents
        if self.lookup is not None:
            if ds.order is not None:
                raise ValueError("the lookup-table chain needs steps grouped by event in increasing event key")
            for k in _capi.LOOKUP_STEP_COLS + ("pdg",):
                if int(lookup_steps[k].numel()) != n:
                    raise ValueError(f"lookup step column {k}: {int(lookup_steps[k].numel())} rows, the batch {n}")
                self.lst[k][:n].copy_(lookup_steps[k])
        for k in ("x", "y", "z", "t", "edep", "bar"):
            self.st[k][:n].copy_(getattr(ds, k))
        E = self.ev
        E["event"][:e].copy_(ds.ev_event)
        E["subrun"][:e].copy_(ds.ev_subrun)
        E["run"][:e].copy_(ds.ev_run)
        E["first"][:e].copy_(ds.ev_first)
        E["nsteps"][:e].copy_(ds.ev_nsteps)
        E["key"][:e].copy_(((ds.ev_subrun.to(E["key"].dtype) & 0xFFFFFFFF) << 20)
                           | (ds.ev_event.to(E["key"].dtype) & 0xFFFFFFFF))
        if e < c.events:
            E["nsteps"][e:].zero_()
            E["first"][e:].zero_()
            E["key"][e:].fill_(INT64_MAX)
        self.nsteps_dev.fill_(n)
        self._n_events = e

    # -- the call ---------------------------------------------------------------------------------------------------
    def _args(self, P):
        t = self.eng.tabs
        return (ctypes.byref(P), ctypes.byref(self.caps.c()), ctypes.byref(self._E), _capi.ptr(self.ev["key"]),
                _capi.ptr(self.ev["run"]), ctypes.byref(self._S), _capi.ptr(self.nsteps_dev), ctypes.byref(t.c_bars()),
                ctypes.byref(t.c_channels()), ctypes.byref(t.c_pixels()), _capi.ptr(self.eng.tmpl),
                int(self.eng.tlen), ctypes.byref(self.eng.fin.c_geom()), ctypes.byref(self._C),
                ctypes.byref(self._M), _capi.ptr(self.counts), _capi.ptr(self.ws), self.ws.numel(), _stream(),
                self.status.ptr)

    def _call(self, P):
        L = _capi.load()
        if self.lookup is not None:
            _capi.check(L.crv_chain_lookup(*self._args(P), ctypes.byref(self._LK)), "crv_chain_lookup")
        else:
            _capi.check(L.crv_chain(*self._args(P)), "crv_chain")

    def _drop_graph(self):
        if self._graph is not None:
            _torch().cuda.synchronize()          # a replay may still be in flight
            _capi.load().crv_chain_graph_destroy(self._graph)
            self._graph = None

    def _capture(self, P, key):
        """Capture one crv_chain call (and the status zeroing) as a native CUDA graph on a side stream, in
        thread-local capture mode, so other host threads (serving slots) keep launching meanwhile."""
        torch = _torch()
        L = _capi.load()
        self._drop_graph()
        if self._side is None:
            self._side = torch.cuda.Stream()
        cur = torch.cuda.current_stream()
        self._side.wait_stream(cur)
        with _CAPTURE_LOCK, torch.cuda.stream(self._side):
            if not self._warm:                                  # first capture: one eager call outside it
                self.status.reset()
                self._call(P)
                self._warm = True
            h = ctypes.c_void_p()
            n0 = _capi.launch_count()
            if self.lookup is not None:
                _capi.check(L.crv_chain_graph_create_lookup(*self._args(P), ctypes.byref(self._LK), ctypes.byref(h)),
                            "crv_chain_graph_create_lookup")
            else:
                _capi.check(L.crv_chain_graph_create(*self._args(P), ctypes.byref(h)), "crv_chain_graph_create")
            self.launches_per_run = _capi.launch_count() - n0
        cur.wait_stream(self._side)
        self._graph, self._graph_key = h, key
        self.captures += 1

    def launch(self, seed):
        """Run the loaded batch (asynchronous; read the outcome with finish()).  Graph mode replays the captured
        chain; a new seed or serving knobs go into the graph's kernels without a new capture (crv_chain_graph_
        set_params), other changes (tables, template, capacities, settings that shape the launches) capture again."""
        P = self.eng.params(seed)
        if self.graph_mode:
            L = _capi.load()
            key = (id(self.eng.tabs), id(self.eng.fin), id(self.eng.tmpl), id(self.lookup))
            if (self._graph is None or self._graph_key != key
                    or L.crv_chain_graph_set_params(self._graph, ctypes.byref(P)) != _capi.CRV_OK):
                self._capture(P, key)
            _capi.check(L.crv_chain_graph_launch(self._graph, _stream()), "crv_chain_graph_launch")
            self.replays += 1
        else:
            n0 = _capi.launch_count()
            self.status.reset()
            self._call(P)
            self.launches_per_run = _capi.launch_count() - n0

    def finish(self, copy=True):
        """Read counts and status (one host read); raise BatchRejected on any flag; the batch's clusters."""
        torch = _torch()
        hdr = torch.cat([self.counts, self.status.t]).cpu().numpy()
        counts = {k: int(hdr[i]) for i, k in enumerate(_capi.CHAIN_COUNTS)}
        self.last_counts = counts
        flags = int(np.int64(hdr[10]) & 0xFFFFFFFF)
        if flags:
            raise BatchRejected(flags, hdr[11:27].copy(), counts)
        ncl, nm = counts["clusters"], counts["members"]
        take = (lambda v, n: v[:n].clone()) if copy else (lambda v, n: v[:n])  # noqa: E731
        return ResidentResult(self._n_events, counts, {k: take(v, ncl) for k, v in self.cl.items()},
                              {k: take(v, nm) for k, v in self.mem.items()})

    def run(self, ds: DeviceSteps, seed, copy=True, lookup_steps=None):
        """One batch: load, launch, read.  With grow, a rejected batch for capacity alone is re-run with larger
        capacities (captured again).  lookup_steps: see load."""
        for attempt in range(self.max_grow + 1):
            self.load(ds, lookup_steps)
            self.launch(seed)
            try:
                return self.finish(copy)
            except BatchRejected as rej:
                if not self.grow or rej.flags != _capi.ST_CAPACITY or attempt == self.max_grow:
                    raise
                self._alloc(self.caps.grown(rej.need))
        raise AssertionError("unreachable")
