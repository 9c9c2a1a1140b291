"""Serving loop: design-point jobs through the device-resident chain with continuous batching.

The reference runs one design-point job per process (a knob set over a step sample).  Here jobs arrive as a
stream and are served by slots: a slot is a resident chain (ResidentChain: one crv_chain call per chunk with explicit
capacities, one host read per chunk) with its own CUDA stream, buffers and host thread, and the number of slots
follows from the HBM budget (the footprint of one slot, measured on a chunk).  Jobs are cut into chunks
of events; free slots take the next chunk of the arrived job with the least work left, so a job that arrives while
others run joins the mix at the next chunk boundary and its chunks overlap with theirs on the device.  Step tables
stay resident: a job names a range of events of a device step pool, which it reads through views.

Per-job knobs (the design point): photon yield [PE/MeV], long attenuation length [mm], readout threshold [PE] and
coincidence window [ns].  Every draw is keyed by (job seed, run, subrun, event, SiPM, draw), so a job's result does not
depend on what else runs: alone and in a mix it is the same, bit for bit.  With the lookup-table photon model (the
production call's tables, crv/crvfastsim/chain.py:197-213) the slots run the lookup-table resident chain; the yields
then come from the model's configuration, and a job's threshold and window are its knobs.  That model keys its draws
by the step's row in the batch (the row the stage API's photon ids refer to), so its result depends on how a job is
cut into chunks; a job's chunks are fixed (chunk_events from its first event), so alone and in a mix it is again the
same.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, replace

import numpy as np

from .config import SPE_PEAK_VOLT, WORKLOAD_CUTS, ChainConfig, FinderConfig, ResponseConfig, WaveformConfig
from .response import DeviceSteps, _torch


@dataclass
class Job:
    id: int
    n_events: int
    first: int = 0                   # first event of the job in the step pool
    seed: int = 1
    yield_per_mev: float = 40.0
    lambda_long: float = 5000.0      # mm
    threshold_pe: float = 5.0
    window_ns: float = 10.0
    arrival: float = 0.0             # seconds after the start of the run


@dataclass
class JobResult:
    id: int
    n_events: int
    clusters: dict                   # host cluster columns (event, type, pe, start, end, slope, avgtime, ...)
    n_clusters: int
    arrival: float
    start: float
    finish: float
    slot: int

    @property
    def latency(self):
        return self.finish - self.arrival


def job_config(job: Job, precision="fp32", sector="EX", lookup=None) -> ChainConfig:
    """ChainConfig of a design point (the serving knobs of the workload).  lookup: the lookup-table model's response
    configuration (its yields replace the job's yield and attenuation knobs)."""
    return ChainConfig(response=ResponseConfig(yield_per_mev=job.yield_per_mev, lambda_long=job.lambda_long),
                       waveform=WaveformConfig(min_voltage=job.threshold_pe * SPE_PEAK_VOLT),
                       finder=FinderConfig(cuts={sector: replace(WORKLOAD_CUTS, max_dt=job.window_ns)}),
                       precision=precision, lookup=lookup)


def random_jobs(n, rng, min_events=1000, max_events=1_000_000, pool_events=None, rate=None):
    """Jobs of the serving workload: events log-uniform in [min_events, max_events], knobs uniform (yield 30-50
    PE/MeV, long attenuation 350-650 cm, threshold 3-8 PE, coincidence window 5-20 ns), Poisson arrivals at `rate`
    jobs/s (all at 0 when rate is None)."""
    ev = np.exp(rng.uniform(np.log(min_events), np.log(max_events), n)).astype(np.int64)
    gaps = rng.exponential(1.0 / rate, n) if rate else np.zeros(n)
    arr = np.cumsum(gaps) - (gaps[0] if rate else 0.0)
    jobs = []
    for i in range(n):
        first = int(rng.integers(0, max(1, pool_events - ev[i] + 1))) if pool_events else 0
        jobs.append(Job(id=i, n_events=int(ev[i]), first=first, seed=int(rng.integers(1, 2 ** 31)),
                        yield_per_mev=float(rng.uniform(30, 50)), lambda_long=float(rng.uniform(3500, 6500)),
                        threshold_pe=float(rng.uniform(3, 8)), window_ns=float(rng.uniform(5, 20)),
                        arrival=float(arr[i])))
    return jobs


def slice_events(ds: DeviceSteps, a: int, b: int, lookup_steps=None):
    """Events [a, b) of a device step table as views of its columns (event table rebased to the slice).  With
    lookup_steps (the table's steps in the lookup model's form, row for row): (the slice, views of those columns)."""
    torch = _torch()
    first = ds.ev_first[a:b]
    r0 = int(first[0].item()) if b > a else 0
    cnt = ds.ev_nsteps[a:b]
    n = int(cnt.sum().item()) if b > a else 0
    sl = slice(r0, r0 + n)
    out = DeviceSteps(x=ds.x[sl], y=ds.y[sl], z=ds.z[sl], t=ds.t[sl], edep=ds.edep[sl], bar=ds.bar[sl],
                      ev_event=ds.ev_event[a:b], ev_subrun=ds.ev_subrun[a:b], ev_run=ds.ev_run[a:b],
                      ev_first=(first - r0).to(torch.int64), ev_nsteps=cnt, nsteps=n, nevents=b - a,
                      max_steps=int(cnt.max().item()) if b > a else 0)
    if lookup_steps is None:
        return out
    return out, {k: v[sl] for k, v in lookup_steps.items()}


@dataclass
class _Slot:
    index: int
    engine: object                   # ChainEngine (tables of the design point)
    stream: object
    footprint: int = 0
    job_id: object = None            # design point the engine is configured for
    chain: object = None             # ResidentChain over the engine (resident mode)
    express: bool = False            # serves only jobs of at most one chunk, on a high-priority stream
    busy: bool = False


class ServeEngine:
    """Continuous-batching job server over a resident step pool.

    pool: DeviceSteps with the events jobs refer to.  hbm_budget: bytes the slots may hold (the number of slots is
    min(max_slots, budget // footprint of one slot)).  chunk_events: events per chain call (bounds a slot's
    footprint and the granularity at which jobs interleave)."""

    def __init__(self, geom, cond, pool: DeviceSteps, hbm_budget: int, max_slots=8, chunk_events=4096,
                 precision="fp32", device="cuda", resident=True, graph=True, express=False, lookup=None,
                 lookup_config=None, lookup_steps=None):
        """resident: slots run the resident chain (one host read per chunk) instead of the per-stage engine (a read per
        stage).  graph: every resident slot replays one captured CUDA graph of the chain, captured here, before any
        slot thread runs; a job's seed and knobs are written into the graph's kernels (crv_chain_graph_set_params),
        so serving needs no capture while it runs (a capacity growth would capture that slot again).
        express: one more slot (within the HBM budget) that takes only jobs of at most one chunk, on a stream of the
        highest priority: a small job that arrives while the other slots run chunks of large jobs starts at once, and
        the block scheduler gives its kernels the SMs that free up before those of the other streams.
        lookup: a LookupModel (crvgpu.lookup) of the geometry, with lookup_config its response configuration and
        lookup_steps the pool's steps in its form (LookupModel.upload_steps, row for row): the slots run the
        lookup-table resident chain (resident mode only)."""
        from .chain import ChainEngine
        from .geometry import sector_geom
        from .resident import ChainCaps, ResidentChain, caps_for
        torch = _torch()
        self.resident = bool(resident)
        self.graph = bool(graph) and self.resident
        self.geom, self.cond, self.pool = geom, cond, pool
        self.G = sector_geom(geom)
        self.sector = str(self.G.sector_names[0])
        self.precision = precision
        self.device = device
        self.chunk = int(chunk_events)
        if lookup is not None:
            if not self.resident:
                raise ValueError("the lookup-table model serves through the resident chain (resident=True)")
            if lookup_config is None or lookup_steps is None:
                raise ValueError("the lookup-table model needs its response configuration and the pool's lookup steps")
            if pool.order is not None:
                raise ValueError("the lookup-table chain needs the pool's steps grouped by event in increasing key")
        self.lookup, self.lookup_config, self.lookup_steps = lookup, lookup_config, lookup_steps
        base = self._config(Job(0, 1))
        # The first slot measures its footprint on a full chunk at the most demanding design point of the knob ranges
        # (largest yield and attenuation length, lowest threshold, widest window), with a margin for the event-to-event
        # spread of later chunks.
        heavy = self._config(Job(0, 1, yield_per_mev=50.0, lambda_long=6500.0, threshold_pe=3.0, window_ns=20.0))
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        m0 = torch.cuda.memory_allocated()
        s0 = _Slot(0, ChainEngine(geom, cond, base, G=self.G, device=device), torch.cuda.Stream())
        first, first_lk = self._slice(0, min(self.chunk, pool.nevents))
        with torch.cuda.stream(s0.stream):
            s0.engine.configure(heavy)
            if self.lookup is None:
                s0.engine.run(first, 1)
            if self.resident:
                # capacities of a chunk at the heavy design point (a trial run of the resident chain), with a margin
                # for the event-to-event spread of later chunks; chunks that need more grow them
                trial = ResidentChain(s0.engine, caps_for(s0.engine, [first]), real_dtype=pool.x.dtype, graph=False,
                                      grow=True, max_grow=8, lookup=self.lookup)
                trial.run(first, 1, lookup_steps=first_lk)
                counts = trial.last_counts
                trial = None
                torch.cuda.synchronize()
                torch.cuda.empty_cache()
                self.caps = ChainCaps.from_counts(counts, events=self.chunk, steps=int(1.2 * first.nsteps) + 1024,
                                                  max_steps_per_event=min(32768, 2 * max(1, first.max_steps)),
                                                  margin=1.3)
                s0.engine = ChainEngine(geom, cond, base, G=self.G, device=device)
                s0.chain = ResidentChain(s0.engine, self.caps, real_dtype=pool.x.dtype, graph=self.graph, grow=True,
                                         lookup=self.lookup)
        torch.cuda.synchronize()
        if self.resident:
            s0.footprint = int(s0.chain.nbytes * 1.05)
        else:
            s0.footprint = int(1.25 * max(1, torch.cuda.max_memory_allocated() - m0))
        n = int(max(1, min(max_slots, hbm_budget // s0.footprint)))
        self.express = bool(express) and hbm_budget // s0.footprint > n
        self.slots = [s0]
        for i in range(1, n + int(self.express)):
            eng = ChainEngine(geom, cond, base, G=self.G, device=device)
            ex = i == n
            sl = _Slot(i, eng, torch.cuda.Stream(priority=-8) if ex else torch.cuda.Stream(), s0.footprint,
                       express=ex)
            if self.resident:
                sl.chain = ResidentChain(eng, self.caps, real_dtype=pool.x.dtype, graph=self.graph, grow=True,
                                         lookup=self.lookup)
            self.slots.append(sl)
        self.footprint = s0.footprint
        if self.graph:                               # capture every slot's graph now, one slot at a time
            for sl in self.slots:
                with torch.cuda.stream(sl.stream):
                    sl.chain.run(first, 1, lookup_steps=first_lk)
                sl.stream.synchronize()

    def _config(self, job: Job) -> ChainConfig:
        return job_config(job, self.precision, self.sector, self.lookup_config)

    def _slice(self, a: int, b: int):
        """Events [a, b) of the pool, and their steps in the lookup model's form (None without the model)."""
        if self.lookup is None:
            return slice_events(self.pool, a, b), None
        return slice_events(self.pool, a, b, self.lookup_steps)

    def _run_chunk(self, slot: _Slot, job: Job, a: int, b: int) -> dict:
        torch = _torch()
        with torch.cuda.stream(slot.stream):
            if slot.job_id != job.id:
                cfg = self._config(job)
                if slot.chain is not None:
                    slot.chain.configure(cfg)
                else:
                    slot.engine.configure(cfg)
                slot.job_id = job.id
            if slot.chain is not None:
                ds, lk = self._slice(a, b)
                out = slot.chain.run(ds, job.seed, lookup_steps=lk).clusters
            else:
                r = slot.engine.run(slice_events(self.pool, a, b), job.seed)
                out = {k: v.clone() for k, v in r.clusters.items()}
            slot.stream.synchronize()
        return out

    def run(self, jobs, realtime=True, policy="srpt", iso_rate=None, iso_overhead=0.0, slack=2.0, iso_table=None):
        """Serve `jobs` (arrival times in seconds from now when realtime, else all at once).  Returns JobResults in
        job order.

        Scheduling: a job is split into chunks of chunk_events events; whenever a slot is free it takes the next chunk
        of an arrived job, so jobs that arrive during others join at the next chunk boundary, and an otherwise idle
        device works on one job's chunks on every slot.  Which job:
          "srpt":     the one with the fewest events left (shortest remaining work first: small jobs are not queued
                      behind large ones; large jobs wait longest under load);
          "edf":      the one with the earliest deadline, arrival + slack * its isolated run time;
          "slowdown": the one whose latency / isolated time would be largest if it were served now (time waited plus
                      its remaining isolated time, over its isolated time): it evens out the slowdown of small and
                      large jobs instead of favouring either.
        The isolated run time is iso_table (measured sizes, see measure_isolated) or iso_overhead + events / iso_rate.
        Chunk results are kept per job and joined in event order when its last chunk is done."""
        if policy not in ("srpt", "edf", "slowdown"):
            raise ValueError(f"unknown scheduling policy {policy!r}")
        if policy != "srpt" and not iso_table and not (iso_rate and iso_rate > 0):
            raise ValueError(f"{policy} scheduling needs the isolated run times (iso_table or iso_rate)")

        def iso_of(n):
            return float(isolated_time(iso_table, n)) if iso_table else iso_overhead + n / iso_rate
        if policy == "edf":
            prio = lambda j: (info[j]["job"].arrival + slack * info[j]["iso"], j)  # noqa: E731
        elif policy == "slowdown":
            def prio(j):
                rec = info[j]
                now = time.perf_counter() - t0
                left = rec["iso"] * rec["left"] / max(rec["job"].n_events, 1)
                return (-((now - rec["job"].arrival) + left) / rec["iso"], j)
        else:
            prio = lambda j: (info[j]["left"], info[j]["job"].arrival, j)  # noqa: E731
        torch = _torch()
        t0 = time.perf_counter()
        cv = threading.Condition()
        state = {"pending": sorted(jobs, key=lambda j: j.arrival), "active": [], "done": 0, "stop": False}
        info = {}
        results = {}
        errors = []
        total = len(jobs)

        def admit_arrived(now):
            # caller holds cv
            while state["pending"] and (not realtime or state["pending"][0].arrival <= now):
                job = state["pending"].pop(0)
                bounds = [(a, min(a + self.chunk, job.first + job.n_events))
                          for a in range(job.first, job.first + job.n_events, self.chunk)]
                info[job.id] = {"job": job, "next": 0, "bounds": bounds, "parts": [None] * len(bounds),
                                "left": job.n_events, "ndone": 0, "start": None,
                                "iso": iso_of(job.n_events) if policy != "srpt" else 0.0}
                state["active"].append(job.id)

        def finish(jid):
            rec = info[jid]
            parts = [p for p in rec["parts"] if p is not None]
            cl = {k: torch.cat([p[k] for p in parts]).cpu().numpy() for k in parts[0]} if parts else {}
            job = rec["job"]
            fin = time.perf_counter() - t0
            results[jid] = JobResult(jid, job.n_events, cl, len(cl.get("pe", ())),
                                     job.arrival if realtime else 0.0, rec["start"], fin, rec.get("slot", -1))

        def worker(slot):
            while True:
                with cv:
                    while True:
                        if errors or state["done"] == total:
                            return
                        admit_arrived(time.perf_counter() - t0)
                        cand = [jid for jid in state["active"] if info[jid]["next"] < len(info[jid]["bounds"])]
                        if slot.express:                      # one-chunk jobs only
                            cand = [jid for jid in cand if len(info[jid]["bounds"]) == 1]
                        elif express is not None and not express.busy:
                            # one-chunk jobs go to the idle express slot
                            cand = [jid for jid in cand if len(info[jid]["bounds"]) > 1]
                        if cand:
                            jid = min(cand, key=prio)
                            rec = info[jid]
                            k = rec["next"]
                            rec["next"] += 1
                            a, b = rec["bounds"][k]
                            rec["left"] -= b - a
                            if rec["start"] is None:
                                rec["start"] = time.perf_counter() - t0
                                rec["slot"] = slot.index
                            slot.busy = True
                            break
                        wait = None
                        if realtime and state["pending"]:
                            wait = max(0.0, state["pending"][0].arrival - (time.perf_counter() - t0))
                        cv.wait(timeout=wait if wait is not None else 0.05)
                try:
                    out = self._run_chunk(slot, rec["job"], a, b)
                except Exception as exc:                    # reported to the caller after the run
                    with cv:
                        errors.append(exc)
                        cv.notify_all()
                    return
                with cv:
                    slot.busy = False
                    rec["parts"][k] = out
                    rec["ndone"] += 1
                    if rec["ndone"] == len(rec["bounds"]):
                        state["active"].remove(jid)
                        finish(jid)
                        state["done"] += 1
                    cv.notify_all()

        express = next((s_ for s_ in self.slots if s_.express), None)
        for s_ in self.slots:
            s_.job_id = None
            s_.busy = False
        threads = [threading.Thread(target=worker, args=(s_,), daemon=True) for s_ in self.slots]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
        return [results[j.id] for j in jobs]


def measure_isolated(srv, sizes, seed=3, reps=2):
    """Isolated run time of a job of each size (events): the job alone on an idle device, best of `reps` runs.
    Returns {size: seconds}; isolated_time() interpolates it."""
    out = {}
    for n in sizes:
        best = None
        for r in range(reps):
            t0 = time.perf_counter()
            srv.run([Job(0, int(n), seed=seed + r)], realtime=False)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        out[int(n)] = best
    return out


def isolated_time(table, n):
    """Isolated run time of n events from a measured size table (linear in events between the measured sizes,
    extrapolated with the rate of the largest two)."""
    xs = np.array(sorted(table), float)
    ys = np.array([table[int(x)] for x in xs])
    n = np.asarray(n, float)
    if len(xs) == 1:
        return ys[0] * n / xs[0]
    hi = ys[-1] + (n - xs[-1]) * (ys[-1] - ys[-2]) / (xs[-1] - xs[-2])
    return np.where(n <= xs[-1], np.interp(n, xs, ys), hi)


def latency_stats(results, iso_rate=None, iso_overhead=0.0, iso_table=None):
    """p50 / p99 job latency [s] and p99 of latency / isolated run time.  The isolated time is measured per size
    (iso_table from measure_isolated, interpolated), or modelled as iso_overhead + events / iso_rate."""
    lat = np.array([r.latency for r in results])
    nev = np.array([r.n_events for r in results], float)
    iso = isolated_time(iso_table, nev) if iso_table else iso_overhead + nev / iso_rate
    span = max(r.finish for r in results) - min(r.arrival for r in results) if results else 0.0
    ev = sum(r.n_events for r in results)
    ratio = lat / iso
    out = {"jobs": len(results), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
           "p99_over_isolated": float(np.percentile(ratio, 99)), "p50_over_isolated": float(np.percentile(ratio, 50)),
           "events_per_s": float(ev / span) if span > 0 else None}
    # slowdown per size class (decades of events)
    cls = {}
    for lo in (1e3, 1e4, 1e5, 1e6):
        m = (nev >= lo) & (nev < 10 * lo)
        if m.any():
            cls[f"{int(lo)}-{int(10 * lo)}"] = {"jobs": int(m.sum()), "p50": float(np.percentile(ratio[m], 50)),
                                                "p99": float(np.percentile(ratio[m], 99))}
    out["slowdown_by_size"] = cls
    return out
