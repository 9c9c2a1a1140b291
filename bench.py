"""Benchmark of the GB300 CRV response engine: CRV events/s steps -> coincidence clusters.

Workload (default): 1,048,576 events of the workload's one-module geometry (4 layers x 16 counters of 450 cm),
Poisson(40) synthetic steps per event (~42 M steps, SoA float32 x/y/z/t/edep + int32 bar, resident in HBM), the full
chain (photons, SiPM, waveforms + zero suppression, pulse fit, coincidences) in event batches.  One benchmark step =
one pass over all events.  The FP32-mixed engine is the headline (value); the FP64 plain chain is timed beside it.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Multi-GPU: events are independent, so each rank processes its own event range (weak scaling, no collective on the
data path; a barrier brackets the timed region and the time is the max over ranks).
--impl reference: the reference algorithm on the host cores (the CPU oracle's restatement of the reference NumPy
path: keyed C photons/SiPM + NumPy waveforms/pulse fit + Python coincidence finder), one process per core.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "mu2e-fastsim_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "CRV events/s steps→coincidences, FP32 vs FP64 plain, 1 GB300; p99 job latency"
UNIT = "events/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------------------------------------------------
# CPU reference arm (oracle port of the reference NumPy path)

def _cpu_worker(args):
    n_events, first_event, seed = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path[:0] = [ROOT, os.path.join(ROOT, "mu2e-fastsim_gb300")]
    from oracle import oracle as O
    from crvgpu import config as CF
    from crvgpu import geometry as GM
    from crvgpu import waveform as WV
    geom = GM.module_geometry()
    cond = GM.default_conditions(geom)
    cfg = CF.ChainConfig()
    G = GM.sector_geom(geom)
    steps = GM.synthetic_steps(n_events, geom, seed=seed, first_event=first_event)
    t0 = time.perf_counter()
    Q, _ = O.charges(steps, geom, cond, cfg.response, cfg.sipm, seed, cfg.window[1])
    wc = CF.WaveformConfig()
    run_of = lambda keys: np.ones(len(np.asarray(keys).ravel()), np.int64)  # noqa: E731
    tdc0 = lambda labels: O.tdc0_of_labels(labels, cond, seed, wc.period, "roc_feb", run_of)  # noqa: E731
    D = O.synthesize(Q["chan"], Q["time"], Q["charge"], tdc0, WV.single_pe_template(wc), wc, wc.period, cfg.window,
                     O.keyed_noise(seed, run_of))
    W = O.reco_waveforms(D, cond)
    rc = CF.RecoConfig()
    P = O.pulses_from_waveforms(W, cond, rc, rc.period)
    out = O.clusters_from_pulses(W, P, G, cond.status, CF.workload_finder(G.sector_names))
    return time.perf_counter() - t0, n_events, len(out["cl_event"])


def cpu_reference(n_events_per_proc, procs, seed=7):
    """Events/s of the CPU reference path on `procs` processes (spawned), each on its own event range."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    jobs = [(n_events_per_proc, 1_000_000 + i * n_events_per_proc, seed) for i in range(procs)]
    t0 = time.perf_counter()
    if procs == 1:
        res = [_cpu_worker(jobs[0])]
    else:
        with ctx.Pool(procs) as pool:
            res = pool.map(_cpu_worker, jobs)
    wall = time.perf_counter() - t0
    ev = sum(r[1] for r in res)
    busy = max(r[0] for r in res)
    return ev / busy, ev, busy, wall


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    procs = max(1, min(os.cpu_count() or 1, 64))
    per = args.ref_events
    vals = []
    for _ in range(max(1, args.warmup_ref)):
        cpu_reference(max(8, per // 8), procs)
    for _ in range(args.steps):
        v, ev, busy, wall = cpu_reference(per, procs)
        vals.append(v)
    v = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * per * procs / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"one 4x16 module, Poisson(40) steps/event, full chain; bounded sample of "
                                   f"{per} events per process x {procs} processes", "events_per_step": per * procs},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": procs, "kind": "port",
                             "sample": f"{per} events per process on {procs} processes"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------------------------------------------------
# GPU arm

class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 9]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def uneven_chunk(n_wf, seed, device, period=12.55, area=400.0):
    """Device-generated waveforms of the uneven batched-fit workload: length uniform over {32, 64, 128, 256, 512},
    1-12 Gumbel pulses of log-uniform 5-500 PE and beta U(10, 25) ns at uniform times in the window, pedestal 100
    with N(0, 2) ADC noise, int16 samples clipped to [0, 4095]."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    lens = torch.tensor([32, 64, 128, 256, 512], device=device)[torch.randint(0, 5, (n_wf,), generator=g,
                                                                               device=device)]
    off = torch.cumsum(lens, 0) - lens
    ns = int(lens.sum().item())
    start = torch.randint(0, 200, (n_wf,), generator=g, device=device)
    wf_of = torch.repeat_interleave(torch.arange(n_wf, device=device), lens)
    t = ((start[wf_of] + torch.arange(ns, device=device) - off[wf_of]) * period).float()
    y = torch.full((ns,), 100.0, device=device) + 2.0 * torch.randn(ns, generator=g, device=device)
    npul = torch.randint(1, 13, (n_wf,), generator=g, device=device)
    t0 = (start * period).float()
    span = (lens * period).float()
    for k in range(12):
        u = torch.rand((4, n_wf), generator=g, device=device)
        pe = torch.exp(np.log(5.0) + u[0] * (np.log(500.0) - np.log(5.0)))
        beta = 10.0 + 15.0 * u[1]
        mu = t0 + u[2] * span
        amp = torch.where(npul > k, pe * area / beta, torch.zeros_like(pe))
        z = (t - mu[wf_of]) / beta[wf_of]
        y += amp[wf_of] * torch.exp(-z - torch.exp(-z))
    adc = torch.clamp(torch.round(y), 0, 4095).to(torch.int16)
    return dict(off=off, n=lens.to(torch.int32), start=start.to(torch.int64), adc=adc, ns=ns,
                ped=torch.full((n_wf,), 100.0, dtype=torch.float64, device=device),
                area=torch.full((n_wf,), area, dtype=torch.float64, device=device),
                height=torch.full((n_wf,), area / 15.0, dtype=torch.float64, device=device), true=int(npul.sum()))


def uneven_pulse_fit(total, chunk, device="cuda"):
    """Waveforms/s of the batched pulse fit (reconstruct_full: rounds bounded by the waveform length) over `total`
    device-generated uneven waveforms, FP32-mixed and FP64 plain; device time of the fit calls only."""
    import torch
    from crvgpu import config as CF
    from crvgpu.params import make_params
    from crvgpu.pulsefit import PulseEngine
    out = {"waveforms": total, "chunk": chunk}
    chunks = [uneven_chunk(min(chunk, total - c0), 1000 + c0, device) for c0 in range(0, total, chunk)]
    out["samples"] = sum(c["ns"] for c in chunks)
    out["true_pulses"] = sum(c["true"] for c in chunks)
    from crvgpu.pulsefit import DEFAULT_SHAPE, GraphFitter, ShapeTuner, set_shape
    set_shape(DEFAULT_SHAPE)
    for prec in ("fp32", "fp64"):
        eng = PulseEngine(device)
        eng.out_factor = 16.0
        P = make_params(reco=CF.RecoConfig(), precision=prec)
        P.period = CF.PERIOD

        def run(c):
            return eng.run(P, c["off"], c["n"], c["start"], c["ped"], c["area"], c["height"], adc16=c["adc"],
                           max_pulses=2 ** 31 - 1, nsamples=c["ns"])
        run(chunks[0])                                            # warm-up: workspace and capacities
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        found = 0
        e0.record()
        for c in chunks:
            found += int(run(c)["wf"].numel())
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out[prec] = {"waveforms_per_s": total / (ms / 1000.0), "ms": ms, "pulses": found}
    # FP32-mixed with the launch shape tuned for the batch size and every batch a replay of one captured CUDA graph
    eng = PulseEngine(device)
    eng.out_factor = 16.0
    P = make_params(reco=CF.RecoConfig(), precision="fp32")
    P.period = CF.PERIOD
    kw = lambda c: dict(off=c["off"], n=c["n"], start_tdc=c["start"], ped=c["ped"], area=c["area"],  # noqa: E731
                        height=c["height"], adc16=c["adc"], max_pulses=2 ** 31 - 1, nsamples=c["ns"])
    tuner = ShapeTuner()
    shape = tuner.shape_for(eng, P, kw(chunks[0]))
    set_shape(shape)
    gf = GraphFitter(P, max(int(c["n"].numel()) for c in chunks), max(c["ns"] for c in chunks), 16 * chunk)
    first = gf.fit(chunks[0]["off"], chunks[0]["n"], chunks[0]["start"], chunks[0]["ped"], chunks[0]["area"],
                   chunks[0]["height"], chunks[0]["adc"])
    plain = eng.run(P, **kw(chunks[0]))
    same = all(torch.equal(first[k], plain[k]) for k in plain)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    found = 0
    e0.record()
    for c in chunks:
        found += int(gf.fit(c["off"], c["n"], c["start"], c["ped"], c["area"], c["height"], c["adc"])["wf"].numel())
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    out["fp32_tuned_graph"] = {"waveforms_per_s": total / (ms / 1000.0), "ms": ms, "pulses": found,
                               "shape": {"threads": shape[0], "blocks_per_sm": shape[1], "rounds": shape[2]},
                               "tuning_ms": {f"{a}/{b}/{c}": round(v, 3) for (a, b, c), v in
                                             next(iter(tuner.best.values()))[1].items()},
                               "matches_plain": bool(same)}
    set_shape(DEFAULT_SHAPE)
    gf = None
    if out["fp64"]["waveforms_per_s"]:
        out["fp32_over_fp64"] = out["fp32"]["waveforms_per_s"] / out["fp64"]["waveforms_per_s"]
    return out


def serving(geom, cond, n_jobs, pool_events, loads, seed=5, max_slots=2, chunk=2048, resident=True, graph=True,
            express=True, capacity_jobs=None, policies=("srpt", "slowdown")):
    """Serving loop over a resident step pool: isolated run time measured per job size (each size alone on the idle
    device), saturated capacity (a burst of every job at once), then Poisson arrivals at each of `loads` x capacity
    (jobs log-uniform 1e3 .. pool_events events, knobs drawn per job).  Wall-clock latencies."""
    import torch
    from crvgpu import geometry as GM
    from crvgpu.response import upload_steps
    from crvgpu.serve import ServeEngine, latency_stats, measure_isolated, random_jobs
    pool = upload_steps(GM.synthetic_steps(pool_events, geom, seed=77), nbars=geom.nbars)
    free, _ = torch.cuda.mem_get_info()
    srv = ServeEngine(geom, cond, pool, hbm_budget=int(0.6 * free), max_slots=max_slots, chunk_events=chunk,
                      resident=resident, graph=graph, express=express)
    sizes = sorted({int(v) for v in np.geomspace(1000, pool_events, 7)})
    iso = measure_isolated(srv, sizes)
    rng = np.random.default_rng(seed)
    # saturated capacity: a burst of capacity_jobs jobs (default n_jobs) of the same distribution, all at once
    burst = random_jobs(capacity_jobs or n_jobs, rng, max_events=pool_events, pool_events=pool_events)
    t0 = time.perf_counter()
    srv.run(burst, realtime=False)
    cap = sum(j.n_events for j in burst) / (time.perf_counter() - t0)
    mean_ev = np.mean([j.n_events for j in random_jobs(4096, np.random.default_rng(seed), max_events=pool_events)])
    out = {"jobs": n_jobs, "slots": len(srv.slots), "express_slot": srv.express, "slot_footprint_gb": srv.footprint / 1e9,
           "slot_engine": ("resident chain, one captured graph per slot re-parameterised per job" if srv.graph else
                           "resident chain, eager") if resident else "per-stage chain",
           "chunk_events": srv.chunk, "pool_events": pool_events, "job_events": f"log-uniform 1e3..{pool_events}",
           "isolated_s_by_size": {str(k): round(v, 5) for k, v in iso.items()}, "capacity_events_per_s": cap,
           "captures_while_serving": 0, "policy": "srpt (and the slowdown-balancing policy)", "loads": {}}
    c0 = sum(sl.chain.captures for sl in srv.slots if sl.chain is not None)
    for k, load in enumerate(loads):
        jobs = random_jobs(n_jobs, np.random.default_rng(seed + 1 + k), max_events=pool_events,
                           pool_events=pool_events, rate=load * cap / mean_ev)
        st = latency_stats(srv.run(jobs, realtime=True), iso_table=iso)
        out["loads"][str(load)] = {k2: v for k2, v in st.items() if k2 != "jobs"}
        if "slowdown" in policies:          # the same arrivals, scheduled to even out the slowdown of small and large jobs
            sl = latency_stats(srv.run(jobs, realtime=True, policy="slowdown", iso_table=iso), iso_table=iso)
            out["loads"][str(load)]["slowdown_policy"] = {k2: v for k2, v in sl.items() if k2 != "jobs"}
    out["captures_while_serving"] = sum(sl.chain.captures for sl in srv.slots if sl.chain is not None) - c0
    srv = pool = None
    return out


def lookup_inputs(n_rows, seed=41, prob=0.0015, yield_per_mev=28610.0, edep=3.4, length=20.0):
    """Synthetic inputs of the lookup-table photon model with the shape of a 3200 mm table (10 x 41 x 56 position
    bins, 5 beta bins, 150 delay bins of random weights, 8 emission bins, arrival probability `prob`, no fibre decay)
    and rows of muon crossings: 20 mm through the thickness at random width and length positions (200 substeps),
    photons per substep from yield x edep and the Cherenkov rate of beta 0.999."""
    from types import SimpleNamespace
    rng = np.random.default_rng(seed)
    edges = {"x": np.linspace(0, 9.89, 11), "y": np.linspace(-25.67, 25.67, 42), "z": np.linspace(-1600, 1600, 57),
             "beta": np.linspace(0.455, 1.0, 6), "theta": np.linspace(0, np.pi, 12), "phi": np.linspace(0, np.pi, 6),
             "r": np.linspace(0, 0.616, 6)}
    nb = {k: len(v) - 1 for k, v in edges.items()}

    def table(n):
        d = rng.integers(0, 4, (n, 150)).astype(np.uint8)
        e = rng.integers(0, 40, (n, 8)).astype(np.uint8)
        return SimpleNamespace(prob=np.full(n, prob, np.float32), delays=d, delay_sum=d.sum(1, dtype=np.int32),
                               emis=e, emis_sum=e.sum(1, dtype=np.int32))

    ns = nb["x"] * nb["y"] * nb["z"]
    L = SimpleNamespace(name="synthetic_3200", half_thickness=9.64, half_width=25.42, half_length=1600.0,
                        fiber_separation=26.0, hole_radius_x=2.0, hole_radius_y=1.0, fiber_radius=0.7,
                        corner_radius=1.75, fiber_decay_time=0.0, edges=edges,
                        tables={"scint": table(ns), "ckscint": table(ns * nb["beta"]),
                                "ckfiber": table(nb["beta"] * nb["theta"] * nb["phi"] * nb["r"] * nb["z"])})
    a = np.c_[np.full(n_rows, -length / 2), rng.uniform(-24, 24, n_rows), rng.uniform(-1500, 1500, n_rows)]
    d = np.c_[np.full(n_rows, length), rng.normal(0, 2, n_rows), rng.normal(0, 2, n_rows)]
    dl = np.linalg.norm(d, axis=1)
    nsub = np.maximum((dl / 0.1).astype(np.int64), 1)
    t0 = rng.uniform(0, 1e5, n_rows)

    def per_substep(avg):
        x = np.where(avg > 10, rng.normal(avg, np.sqrt(avg)), rng.poisson(avg))
        return np.maximum(np.rint(x / nsub), 0).astype(np.int64)

    ck = 266.0 * (0.999 - 0.474) / (1.0 - 0.474) * length      # Cherenkov photons of the crossing (linear map)
    rows = {"s": a, "d": d, "t0": t0, "t1": t0 + 0.07, "nsub": nsub, "beta": np.full(n_rows, 0.999),
            "theta": np.arccos(np.clip(d[:, 2] / dl, -1, 1)), "dev": np.full(n_rows, 0.94),
            "step": np.arange(n_rows, dtype=np.int64), "chan": (np.arange(n_rows, dtype=np.int64) % 8192) * 4,
            "n_scint": per_substep(np.full(n_rows, yield_per_mev * edep)), "n_ck_s": per_substep(np.full(n_rows, ck)),
            "n_ck_f": per_substep(np.full(n_rows, ck))}
    return L, rows


def lookup_substeps(n_rows, reps=3, cpu_rows=20000, precision="fp64"):
    """Lookup-table photon model: (step, SiPM) rows/s of crv_substep_photons on device-resident rows (device time of
    the launches, CUDA events), and the oracle's rate on one core over a bounded sample of the same rows."""
    import torch
    from crvgpu import lookup as LK
    L, rows = lookup_inputs(n_rows)
    DL, R = LK.DeviceLookup(L), LK.DeviceRows(rows)
    eng = LK.SubstepEngine()
    st, _, _ = eng.run(DL, R, 1, precision=precision)     # warm-up, output capacity
    n_ph = int(st.numel())
    st = None
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for r in range(reps):
        eng.run(DL, R, 2 + r, precision=precision)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    out = {"rows": n_rows, "rows_per_s": n_rows / (ms / 1000.0), "ms_per_call": ms, "photons_per_row": n_ph / n_rows,
           "substeps_per_row": float(np.mean(rows["nsub"])), "table": "synthetic 3200 mm: 10x41x56 position bins, "
           "5 beta, 150 delay bins, prob 0.0015",
           "precision": "fp64 (bit-exact with the oracle)" if precision == "fp64" else "fp32-mixed (FP64 times)",
           "published_context": "reference JAX substep kernel ~300k rows/s on A100 (its own bench)"}
    if precision != "fp64":
        cpu_rows = 0
    try:
        if not cpu_rows:
            raise RuntimeError("CPU sample with the FP64 leg")
        from oracle import oracle as O
        sub = {k: v[:cpu_rows] for k, v in rows.items()}
        t0 = time.perf_counter()
        O.substep_photons(L, sub, 2)
        out["cpu_oracle_rows_per_s"] = cpu_rows / (time.perf_counter() - t0)
        out["cpu_oracle_sample"] = f"{cpu_rows} rows on 1 core"
    except Exception as exc:                              # reported baseline only
        out["cpu_oracle_error"] = str(exc)[:200]
    DL = R = eng = None
    return out


def fullscale(n_events, batch, seed=13, resident_batch=2048, stage_events=4096):
    """Full-scale detector (86 modules of 4 x 16 counters, bar lengths over {230, 300, 450, 560, 660} cm, Poisson(60)
    steps plus 0.5 noise steps per counter per event): events/s of the chain on a resident subset, device time over
    the batches.  FP32-mixed through the resident engine (one CUDA graph replay per `resident_batch`-event batch) and
    per stage, FP64 plain per stage (`batch`-event batches: the per-stage workspaces of this geometry take ~150 GB
    per 1,024 events).  The per-stage legs run on the first `stage_events` events, the resident FP32 leg on all."""
    import torch
    from crvgpu import chain as CH, config as CF, geometry as GM
    from crvgpu.resident import ChainCaps, ResidentChain, caps_for
    from crvgpu.response import upload_steps
    from crvgpu.serve import slice_events
    geom = GM.module_geometry(86)
    cond = GM.default_conditions(geom)

    def make(bsize):
        out, n = [], 0
        for b0 in range(0, n_events, bsize):
            st = GM.synthetic_steps(min(bsize, n_events - b0), geom, seed=seed, mean_steps=60.0,
                                    noise_per_counter=0.5, first_event=b0)
            n += len(st)
            out.append(upload_steps(st, nbars=geom.nbars))
        return out, n

    def device_ms(fn, bs):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ncl = sum(fn(ds) for ds in bs)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), ncl

    rb, nsteps = make(resident_batch)                  # the events, generated once; per-stage batches are views
    stage_events = min(stage_events, n_events)
    batches = [slice_events(r, a, min(a + batch, r.nevents)) for r in rb for a in range(0, r.nevents, batch)]
    batches = batches[:max(1, stage_events // batch)]
    out = {"events": n_events, "stage_events": sum(b.nevents for b in batches), "batch": batch,
           "resident_batch": resident_batch, "resident_batches": len(rb), "steps": nsteps, "counters": geom.nbars}
    for prec in ("fp32", "fp64"):
        eng = CH.ChainEngine(geom, cond, CF.ChainConfig(precision=prec))
        eng.run(batches[0], 3)
        ms, ncl = device_ms(lambda ds: eng.run(ds, 3).n_clusters, batches)
        ne = sum(b.nevents for b in batches)
        out[prec if prec == "fp64" else "fp32_stage"] = {"events_per_s": ne / (ms / 1000.0), "ms": ms,
                                                         "clusters": ncl, "events": ne}
        if prec == "fp32":
            try:
                eng.release()                          # the per-stage workspaces of this geometry are large
                torch.cuda.empty_cache()
                sample = slice_events(rb[0], 0, min(128, rb[0].nevents))
                trial = ResidentChain(eng, caps_for(eng, [sample]), graph=False, grow=True, max_grow=8)
                trial.run(sample, 3)
                scale = max(b.nevents for b in rb) / sample.nevents
                caps = ChainCaps.from_counts({k: v * scale for k, v in trial.last_counts.items()},
                                             events=max(b.nevents for b in rb), steps=max(b.nsteps for b in rb),
                                             max_steps_per_event=max(b.max_steps for b in rb), margin=1.15)
                trial = None
                torch.cuda.empty_cache()
                rc = ResidentChain(eng, caps, graph=True, grow=True)
                rc.run(rb[0], 3)
                ms, ncl = device_ms(lambda ds: rc.run(ds, 3).counts["clusters"], rb)
                out["fp32"] = {"events_per_s": n_events / (ms / 1000.0), "ms": ms, "clusters": ncl,
                               "engine": f"resident (graph replay per {resident_batch}-event batch)"}
                rc = None
            except Exception as exc:                   # the per-stage figure stands, and says why
                out["fp32"] = dict(out["fp32_stage"], engine=f"per-stage (resident failed: {str(exc)[:160]})")
        eng = None
        torch.cuda.empty_cache()
    out["fp32_over_fp64"] = out["fp32"]["events_per_s"] / out["fp64"]["events_per_s"]
    try:                                                 # the oracle chain on a bounded full-scale sample, one core
        dt, ne, ncl = _cpu_full_worker((6, seed))
        out["cpu_baseline"] = {"value": ne / dt, "unit": "events/s", "cores": 1, "kind": "port",
                               "sample": f"{ne} full-scale events through the oracle chain on 1 core ({dt:.1f} s)"}
    except Exception as exc:                             # reported baseline only
        out["cpu_baseline"] = {"error": str(exc)[:200]}
    out["projected_s_16777216_events_fp32"] = 16777216 / out["fp32"]["events_per_s"]
    return out


def lookup_chain(n_events, precision="fp32", seed=4, reps=3):
    """The lookup-table photon model inside the resident chain (crv_chain_lookup, one graph replay per batch) on the
    workload's module with a synthetic lookup table of its bars (crvgpu.lookup.synthetic_module_lookup: muons crossing
    the thickness), against the stage path on the same events and seed: chain.charges with the lookup tables (host
    tables in and out), then the per-stage engine from those charges.  Wall-clock per batch after warm-up; the two give
    the same clusters."""
    import torch
    from crvgpu import chain as CH
    from crvgpu.config import ChainConfig
    from crvgpu.lookup import LookupModel, synthetic_module_lookup
    from crvgpu.resident import ChainCaps, ResidentChain
    from crvgpu.response import upload_steps
    geom, cond, tables, lcfg, steps, pdg = synthetic_module_lookup(n_events, seed=seed)
    cfg = ChainConfig(lookup=lcfg, precision=precision)
    ds = upload_steps(steps, nbars=geom.nbars)
    model = LookupModel(geom, lcfg, tables, cond.deviation, precision=precision)
    cols = model.upload_steps(steps, pdg)
    eng = CH.ChainEngine(geom, cond, cfg)
    caps = ChainCaps(events=ds.nevents, steps=ds.nsteps, photons=1024, charges=1024, slots=1024, digis=1024,
                     pulses=1024, max_steps_per_event=max(1, ds.max_steps))
    rc = ResidentChain(eng, caps, real_dtype=torch.float64, graph=True, grow=True, max_grow=8, lookup=model)
    rc.run(ds, seed, lookup_steps=cols)
    rc.run(ds, seed + 1, lookup_steps=cols)
    torch.cuda.synchronize()
    best = None
    for k in range(reps):
        t0 = time.perf_counter()
        r = rc.run(ds, seed + 2 + k, lookup_steps=cols)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)

    def stage(sd):
        Q = CH.charges(steps, None, geom, cond, cfg, None, key=sd, tabs=tables, pdg=pdg)
        dq = {"label": torch.from_numpy(np.asarray(Q["chan"], np.int64)).cuda(),
              **{k: torch.from_numpy(np.ascontiguousarray(Q[k])).cuda() for k in ("time", "charge", "pe", "photon")}}
        return eng.run(ds, sd, charges=dq)
    stage(seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref = stage(seed + 2 + reps - 1)
    torch.cuda.synchronize()
    t_st = time.perf_counter() - t0
    same = ref.n_clusters == r.counts["clusters"] and all(torch.equal(r.clusters[k], v) for k, v in ref.clusters.items())
    return {"events": ds.nevents, "steps": ds.nsteps, "precision": precision, "tables": "synthetic, one 450 cm table",
            "resident_events_per_s": ds.nevents / best, "stage_path_events_per_s": ds.nevents / t_st,
            "resident_over_stage": t_st / best, "same_clusters": bool(same), "counts": r.counts,
            "launches_per_batch": rc.launches_per_run}


def e2e_dropin(geom, cond, n_events, seed=11, first_event=7_000_000, precision="fp32", reps=3):
    """The reference-facing call sequence on host tables, as a reference user makes it through the drop-in entry
    points (chain.charges -> chain.digis -> chain.reco_waveforms -> chain.clusters: host step table in, host arrays
    between the stages, host cluster table out).  Wall-clock events/s, median of `reps` passes after a warm-up."""
    import torch
    from crvgpu import chain as CH, config as CF, geometry as GM
    steps = GM.synthetic_steps(n_events, geom, seed=seed, first_event=first_event)
    cfg = CF.ChainConfig(precision=precision)
    G = GM.sector_geom(geom)
    h2d = sum(np.asarray(steps[k]).nbytes for k in ("x", "y", "z", "t", "edep", "bar", "event", "subrun", "run"))

    def once():
        Q = CH.charges(steps, None, geom, cond, cfg, None, key=5)
        D = CH.digis(Q, cond, cfg, None, key=5, geom=geom)
        W = CH.reco_waveforms(D, cond)
        cl, _ = CH.clusters(W, cond, geom, G, cfg)
        return len(cl[0]["cl_event"]), sum(v.nbytes for v in cl[0].values())
    once()
    times = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ncl, d2h = once()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    dt = float(np.median(times))
    return {"events": n_events, "events_per_s": n_events / dt, "s_per_pass": dt, "clusters": ncl,
            "precision": precision, "h2d_bytes_per_pass": int(h2d), "d2h_bytes_per_pass": int(d2h),
            "calls": "chain.charges -> chain.digis -> chain.reco_waveforms -> chain.clusters (host tables)"}


def dumper_steps(steps, seed=3):
    """A synthetic step table in the CrvStepTableDumper layout (run/subrun/event unsigned, nstep/bar/sp int, t0/t1
    double, start/end positions and the rest float), whose midpoints are the workload's steps."""
    rng = np.random.default_rng(seed)
    n = len(steps["bar"])
    ev = np.asarray(steps["event"])
    first = np.r_[True, ev[1:] != ev[:-1]] if n else np.zeros(0, bool)
    cnt = np.diff(np.r_[np.flatnonzero(first), n])
    d = {"run": np.asarray(steps["run"]).astype(np.uint32), "subrun": np.asarray(steps["subrun"]).astype(np.uint32),
         "event": ev.astype(np.uint32), "nstep": np.repeat(cnt, cnt).astype(np.int32),
         "bar": np.asarray(steps["bar"], np.int32), "sp": np.ones(n, np.int32), "sp_product_id": np.ones(n, np.uint32),
         "t0": np.asarray(steps["t"], np.float64) - 0.25, "t1": np.asarray(steps["t"], np.float64) + 0.25,
         "edep": np.asarray(steps["edep"], np.float32)}
    for a in "xyz":
        h = rng.uniform(-3, 3, n).astype(np.float32)
        d[f"{a}0"] = np.asarray(steps[a], np.float32) - h
        d[f"{a}1"] = np.asarray(steps[a], np.float32) + h
    for k in ("px0", "py0", "pz0", "p1"):
        d[k] = rng.normal(0, 300, n).astype(np.float32)
    d["len"] = np.asarray(steps["len"], np.float32)
    return d


def step_tables(geom, cond, n_events, seed=11, first_event=9_000_000, precision="fp32", reps=3):
    """Step-table files (tables.write / tables.read: the dumper layout as a ROOT TTree, zlib level 1): write and read
    throughput on the host, and the file -> clusters sequence (tables.read, then the drop-in chain calls)."""
    import shutil
    import tempfile
    import torch
    from crvgpu import chain as CH, config as CF, geometry as GM, tables as TB
    steps = dumper_steps(GM.synthetic_steps(n_events, geom, seed=seed, first_event=first_event))
    rows = len(steps["bar"])
    raw = sum(v.nbytes for v in steps.values())
    tmp = tempfile.mkdtemp(prefix="crvsteps")
    path = os.path.join(tmp, "crvsteps.bench.root")
    try:
        tw = []
        for _ in range(2):
            t0 = time.perf_counter()
            TB.write(path, steps, None)
            tw.append(time.perf_counter() - t0)
        size = os.path.getsize(path)
        tr = []
        for _ in range(reps):
            t0 = time.perf_counter()
            s = TB.read(path, "steps")
            tr.append(time.perf_counter() - t0)
        same = all(np.array_equal(s[k], v) for k, v in steps.items())
        cfg = CF.ChainConfig(precision=precision)
        G = GM.sector_geom(geom)

        def once():
            st = TB.read(path, "steps")
            Q = CH.charges(st, None, geom, cond, cfg, None, key=5)
            D = CH.digis(Q, cond, cfg, None, key=5, geom=geom)
            W = CH.reco_waveforms(D, cond)
            cl, _ = CH.clusters(W, cond, geom, G, cfg)
            return len(cl[0]["cl_event"])
        once()
        te = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ncl = once()
            torch.cuda.synchronize()
            te.append(time.perf_counter() - t0)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    w, r, e = min(tw), float(np.median(tr)), float(np.median(te))
    return {"events": n_events, "rows": rows, "columns": len(steps), "column_bytes": int(raw), "file_bytes": int(size),
            "compression": "zlib level 1 (ROOT setting 101)", "write_s": w, "read_s": r,
            "read_rows_per_s": rows / r, "read_mb_per_s": raw / r / 1e6, "write_mb_per_s": raw / w / 1e6,
            "read_identical": bool(same), "file_to_clusters_events_per_s": n_events / e, "clusters": ncl,
            "host_threads": min(16, os.cpu_count() or 1),
            "calls": "tables.read -> chain.charges -> chain.digis -> chain.reco_waveforms -> chain.clusters"}


def _cpu_fit_worker(args):
    """Oracle reconstruct_full (the reference's pulse fit restated) on one length bucket of the uneven workload."""
    length, n_wf, seed = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path[:0] = [ROOT, os.path.join(ROOT, "mu2e-fastsim_gb300")]
    import torch
    from oracle import oracle as O
    from crvgpu import config as CF
    c = uneven_chunk(4 * n_wf, seed, "cpu")
    n = c["n"].numpy()
    sel = np.flatnonzero(n == length)[:n_wf]
    off = c["off"].numpy()[sel]
    adc = np.stack([c["adc"].numpy()[o:o + length].astype(np.int64) for o in off]) if len(sel) else \
        np.zeros((0, length), np.int64)
    rc = CF.RecoConfig()
    t0 = time.perf_counter()
    r = O.reconstruct_full(adc, n[sel], c["start"].numpy()[sel], c["ped"].numpy()[sel], c["area"].numpy()[sel],
                           c["height"].numpy()[sel], rc, CF.PERIOD)
    return length, len(sel), time.perf_counter() - t0, len(r["pe"])


def cpu_fit_baseline(per_bucket=(400, 300, 200, 120, 80)):
    """Waveforms/s of the oracle's reconstruct_full on one core per length bucket of the uneven batched-fit workload
    (a bounded subset each), and the rate of the equal mix the workload draws (harmonic mean over the buckets)."""
    lengths = (32, 64, 128, 256, 512)
    out = {}
    for L, nw in zip(lengths, per_bucket):
        _, got, dt, npu = _cpu_fit_worker((L, nw, 77 + L))
        out[str(L)] = {"waveforms": got, "s": dt, "waveforms_per_s": got / dt, "pulses": npu}
    mix = len(lengths) / sum(1.0 / out[str(L)]["waveforms_per_s"] for L in lengths)
    return {"value": mix, "unit": "waveforms/s", "cores": 1, "kind": "port",
            "sample": "oracle reconstruct_full, " + ", ".join(f"{out[str(L)]['waveforms']} waveforms of {L}"
                                                              for L in lengths) + " samples; equal mix",
            "per_length": out}


def _cpu_full_worker(args):
    n_events, seed = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path[:0] = [ROOT, os.path.join(ROOT, "mu2e-fastsim_gb300")]
    from oracle import oracle as O
    from crvgpu import config as CF
    from crvgpu import geometry as GM
    from crvgpu import waveform as WV
    geom = GM.module_geometry(86)
    cond = GM.default_conditions(geom)
    cfg = CF.ChainConfig()
    G = GM.sector_geom(geom)
    steps = GM.synthetic_steps(n_events, geom, seed=seed, mean_steps=60.0, noise_per_counter=0.5)
    t0 = time.perf_counter()
    Q, _ = O.charges(steps, geom, cond, cfg.response, cfg.sipm, seed, cfg.window[1])
    wc = CF.WaveformConfig()
    run_of = lambda keys: np.ones(len(np.asarray(keys).ravel()), np.int64)  # noqa: E731
    tdc0 = lambda labels: O.tdc0_of_labels(labels, cond, seed, wc.period, "roc_feb", run_of)  # noqa: E731
    D = O.synthesize(Q["chan"], Q["time"], Q["charge"], tdc0, WV.single_pe_template(wc), wc, wc.period, cfg.window,
                     O.keyed_noise(seed, run_of))
    W = O.reco_waveforms(D, cond)
    rc = CF.RecoConfig()
    P = O.pulses_from_waveforms(W, cond, rc, rc.period)
    out = O.clusters_from_pulses(W, P, G, cond.status, CF.workload_finder(G.sector_names))
    return time.perf_counter() - t0, n_events, len(out["cl_event"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--events", type=int, default=1 << 20)
    ap.add_argument("--batch", type=int, default=1 << 16)
    ap.add_argument("--ref-events", type=int, default=96)
    ap.add_argument("--warmup-ref", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--serve-jobs", type=int, default=100, help="jobs per load level of the serving measurement (0: skip)")
    ap.add_argument("--fullscale-events", type=int, default=32768,
                    help="events of the full-scale measurement, resident FP32 leg (0: skip)")
    ap.add_argument("--fullscale-stage-events", type=int, default=4096,
                    help="events of the full-scale per-stage FP32 and FP64 legs")
    ap.add_argument("--dropin-events", type=int, default=16384,
                    help="events of the drop-in (host tables through the stage entry points) end-to-end leg (0: skip)")
    ap.add_argument("--step-table-events", type=int, default=65536,
                    help="events of the step-table file leg (tables.write / tables.read, file -> clusters; 0: skip)")
    ap.add_argument("--serve-pool", type=int, default=1 << 18, help="events of the resident step pool")
    ap.add_argument("--lookup-chain-events", type=int, default=16384,
                    help="events of the resident chain with the lookup-table model (0: skip)")
    ap.add_argument("--serve-loads", default="0.5,0.8,0.95", help="offered loads (fractions of the measured capacity)")
    ap.add_argument("--serve-capacity-jobs", type=int, default=0,
                    help="jobs of the saturated burst that measures the capacity (0: as many as --serve-jobs)")
    ap.add_argument("--serve-policies", default="srpt,slowdown", help="scheduling policies run at every load")
    ap.add_argument("--lookup-rows", type=int, default=1 << 20,
                    help="(step, SiPM) rows of the lookup-table photon model measurement (0: skip)")
    ap.add_argument("--lookup-precision", default="both", choices=["both", "fp64", "fp32"],
                    help="precision of the lookup-table measurement")
    ap.add_argument("--uneven-waveforms", type=int, default=1 << 22,
                    help="waveforms of the uneven batched pulse-fit measurement (0: skip)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))

    def barrier():
        if dist is not None:
            dist.barrier()

    from crvgpu import _capi, chain as CH, config as CF, geometry as GM
    from crvgpu.response import upload_steps

    geom = GM.module_geometry()
    cond = GM.default_conditions(geom)
    # this rank's events (weak scaling: every rank its own event range)
    first = rank * args.events
    t_gen = time.perf_counter()
    batches = []
    host_batches = []
    nsteps_total = 0
    for b0 in range(0, args.events, args.batch):
        nb = min(args.batch, args.events - b0)
        st = GM.synthetic_steps(nb, geom, seed=11, first_event=first + b0)
        host_batches.append(st)
        batches.append(upload_steps(st, nbars=geom.nbars))
        nsteps_total += len(st)
    t_gen = time.perf_counter() - t_gen
    step_bytes = sum(b.x.numel() * 4 * 5 + b.bar.numel() * 4 for b in batches)

    cfg32 = CF.ChainConfig(precision="fp32")
    cfg64 = CF.ChainConfig(precision="fp64")
    eng32 = CH.ChainEngine(geom, cond, cfg32)
    eng64 = CH.ChainEngine(geom, cond, cfg64)

    def one_pass(eng, seed, diagnostics=False):
        tot = dict(clusters=0, pulses=0, charges=0, digis=0, waveforms=0, groups=0, hits=0, members=0, events=0,
                   photons=0, sipms=0)
        for ds in batches:
            r = eng.run(ds, seed, diagnostics=diagnostics)
            tot["clusters"] += r.n_clusters
            tot["pulses"] += r.n_pulses
            tot["charges"] += r.n_charges
            tot["digis"] += r.n_digis
            tot["waveforms"] += r.n_waveforms
            tot["hits"] += r.n_hits
            tot["members"] += r.n_members
            tot["events"] += r.n_events
            tot["photons"] += r.n_photons
            tot["sipms"] += r.n_sipms
        return tot

    def resident_pass(rc, seed):
        tot = dict(clusters=0, pulses=0, charges=0, digis=0, events=0)
        for ds in batches:
            r = rc.run(ds, seed)
            tot["clusters"] += r.counts["clusters"]
            tot["pulses"] += r.counts["pulses"]
            tot["charges"] += r.counts["charges"]
            tot["digis"] += r.counts["digis"]
            tot["events"] += r.n_events
        return tot

    def timed(eng, k, w, pass_fn=None):
        pass_fn = pass_fn or one_pass
        for _ in range(w):
            pass_fn(eng, 5)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        clocks = Clocks(local)
        clocks.start()
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = _capi.launch_count()
        r0 = getattr(eng, "replays", 0)
        e0.record(st)
        tot = None
        for _ in range(k):
            tot = pass_fn(eng, 5)
        e1.record(st)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        # library launches outside graphs, plus the kernels of every graph replay
        launches = _capi.launch_count() - n0 + (getattr(eng, "replays", 0) - r0) * getattr(eng, "launches_per_run", 0)
        ck = clocks.stop()
        ms = e0.elapsed_time(e1)
        if dist is not None:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, tot, ck, launches

    # per-stage engine (every stage reads its sizes back to the host)
    ms_st, tot_st, clk_st, launches_st = timed(eng32, args.steps, args.warmup)
    ev_total = args.events * world * args.steps
    stage_value = ev_total / (ms_st / 1000.0)
    # resident engine: one crv_chain call per batch, replayed as a CUDA graph, explicit capacities sized by a trial
    # batch (batches that need more grow them during the warm-up)
    from crvgpu.resident import ChainCaps, ResidentChain, caps_for
    from crvgpu.serve import slice_events
    try:
        sample = slice_events(batches[0], 0, min(8192, batches[0].nevents))
        trial = ResidentChain(eng32, caps_for(eng32, [sample]), graph=False, grow=True, max_grow=8)
        trial.run(sample, 5)
        scale = max(b.nevents for b in batches) / sample.nevents
        res_caps = ChainCaps.from_counts({k: v * scale for k, v in trial.last_counts.items()},
                                         events=max(b.nevents for b in batches), steps=max(b.nsteps for b in batches),
                                         max_steps_per_event=max(b.max_steps for b in batches), margin=1.1)
        trial = None
        torch.cuda.empty_cache()
        rchain = ResidentChain(eng32, res_caps, graph=True, grow=True)
        ms32, tot32, clk, launches = timed(rchain, args.steps, args.warmup, pass_fn=resident_pass)
        resident = {"engine": "resident (graph replay per batch)", "caps": rchain.caps.as_dict(),
                    "launches_per_batch": rchain.launches_per_run, "device_bytes": rchain.nbytes,
                    "clusters_per_pass": tot32["clusters"], "stage_engine_clusters_per_pass": tot_st["clusters"]}
    except Exception as exc:          # the line then carries the per-stage engine's figures, and says so
        trial = rchain = None
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        ms32, tot32, clk, launches = ms_st, tot_st, clk_st, launches_st
        resident = {"engine": "per-stage (the resident engine failed)", "error": str(exc)[:300]}
    value = ev_total / (ms32 / 1000.0)

    # e2e: step tables in pinned host memory -> device (asynchronous copies on a second stream, the next batch while
    # the current one computes) -> chain -> cluster table back to the host, one pass
    from crvgpu.response import pin_steps
    pinned = [pin_steps(st, nbars=geom.nbars) for st in host_batches]
    copy_stream = torch.cuda.Stream()
    ready = [torch.cuda.Event() for _ in pinned]

    def prefetch(i):
        with torch.cuda.stream(copy_stream):
            d = pinned[i].to_device()
            ready[i].record(copy_stream)
        return d

    def e2e_pass():
        h2d = d2h = 0
        nxt = prefetch(0)
        for i in range(len(pinned)):
            cur = nxt
            torch.cuda.current_stream().wait_event(ready[i])
            h2d += pinned[i].nbytes
            if i + 1 < len(pinned):
                nxt = prefetch(i + 1)
            r_ = rchain.run(cur, 5, copy=False) if rchain is not None else eng32.run(cur, 5)
            host_cl = {k: v.cpu().numpy() for k, v in r_.clusters.items()}
            d2h += sum(a.nbytes for a in host_cl.values())
        return h2d, d2h

    e2e_pass()                                            # warm-up (pinned buffers, allocator)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    h2d, d2h = e2e_pass()
    e1.record()
    torch.cuda.synchronize()
    e2e = args.events / (e0.elapsed_time(e1) / 1000.0)
    r = None
    pinned = None
    rchain = None
    torch.cuda.synchronize()
    torch.cuda.empty_cache()

    fp64 = None
    if not args.no_fp64:
        ms64, tot64, clk64, _ = timed(eng64, max(1, args.steps // 2), 1)
        fp64 = args.events * world * max(1, args.steps // 2) / (ms64 / 1000.0)

    # per-kernel device time of one FP32 pass (profiling events; not the timed number)
    torch.cuda.synchronize()
    _capi.profile(True)
    counts = one_pass(eng32, 5, diagnostics=True)
    torch.cuda.synchronize()
    prof = _capi.profile_read()
    _capi.profile(False)
    per_kernel = {}
    for name, t in prof:
        a = per_kernel.setdefault(name, [0, 0.0])
        a[0] += 1
        a[1] += t
    tot_ms = sum(v[1] for v in per_kernel.values())
    hbm, peak_kind = peaks()
    nb = len(batches)

    # Algorithmic bytes per event batch, from the stage counts of the pass.  The pulse fit is one group of launches
    # per batch (k_pf_begin + the round launches k_pf_round), timed together:
    #   pulse fit:  int16 samples in (12 per digi) + per waveform 44 B in (sample row 8, length 4, start TDC 8,
    #               pedestal / area / height 24) + per pulse 104 B out (11 FP64 columns, wf, seq, 3 flags)
    #   k_wf_synth: per charge 16 B in (time, charge) + per digi 152 B out (label, start, TDC0, start TDC, 12 volts,
    #               12 ADC)
    #   k_sipm_sim: per photon 8 B in (FP32 time, key) + per SiPM 32 B in (first photon, count, label, run, slots)
    #               + per charge 24 B out (time, voltage, photon id)
    #   k_coinc:    per hit 28 B in (bar, SiPM, sequence, time, PE) + per event 20 B in (first hit, count, key)
    #               + per cluster 120 B out (event, type, PE, start, end, slope, average time, position, flags) + 4 B
    #               per member index
    groups = {"pulse fit": ("k_pf_begin", "k_pf_round", "k_pf_persist"), "k_wf_synth": ("k_wf_synth", "k_wf_synth32"), "k_coinc": ("k_coinc", "k_coinc_global"),
              "k_sipm_sim": ("k_sipm_sim",)}

    def alg_bytes(group):
        if group == "pulse fit":
            return (counts["digis"] * 12 * 2 + counts["waveforms"] * 44 + counts["pulses"] * 104) / nb
        if group == "k_wf_synth":
            return (counts["charges"] * 16 + counts["digis"] * 152) / nb
        if group == "k_sipm_sim":
            return (counts["photons"] * 8 + counts["sipms"] * 32 + counts["charges"] * 24) / nb
        if group == "k_coinc":
            return (counts["hits"] * 28 + counts["events"] * 20 + counts["clusters"] * 120
                    + counts["members"] * 4) / nb
        return None

    def group_of(name):
        return next((g for g, ks in groups.items() if name in ks), name)

    by_group = {}
    for name, (_, ms_k) in per_kernel.items():
        by_group[group_of(name)] = by_group.get(group_of(name), 0.0) + ms_k
    top_group = max(by_group.items(), key=lambda kv: kv[1])[0]

    # DRAM bytes (read + write) over algorithmic bytes of one 16,384-event chain batch, from single-kernel ncu captures
    # of every launch of the stage in that batch (k_sipm_sim, 3 launches: 3.419 GB over 2.978 GB; k_wf_synth32,
    # 3 launches: 1.823 GB over 1.405 GB; k_pf_persist, 1 launch: 0.757 GB over 0.396 GB); the traffic of a stage grows
    # with the events processed, so the ratio scales it to this run's batch
    traffic_ratio = {"k_sipm_sim": 1.148, "k_wf_synth": 1.298, "pulse fit": 1.910}

    def roofline_of(group):
        ks = groups.get(group, (group,))
        if not any(k in per_kernel for k in ks):
            return None
        ms = sum(per_kernel[k][1] for k in ks if k in per_kernel)
        per_batch_ms = ms / nb
        b = alg_bytes(group)
        if b is None or per_batch_ms <= 0:
            return None
        ach = b / (per_batch_ms / 1000.0) / 1e9
        tr = traffic_ratio.get(group)
        return {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": (tr * b) if tr else None,
                "kernel": "+".join(ks), "algorithmic_bytes_per_launch": b, "ms_per_launch": per_batch_ms,
                "launch": "one event batch", "peak_kind": f"{peak_kind} (copy bandwidth)"}

    # FP32-mixed error report against the FP64-plain run of the same events and keys (first batch): counts need not
    # agree; digis, pulses, hits and clusters are matched (crvgpu.accuracy)
    acc = {}
    try:
        from crvgpu.accuracy import error_table
        r64 = eng64.run(batches[0], 5, keep=True)
        r32 = eng32.run(batches[0], 5, keep=True)
        acc = error_table(r64, r32, eng32.wcfg.adc_conversion, eng32.wcfg.pedestal)
        acc["sample"] = f"first batch: {batches[0].nevents} events, seed 5"
        r32 = None
        eng64.release()
        torch.cuda.empty_cache()
        try:                                              # the waveform stage alone, on the FP64 run's charges
            from crvgpu.accuracy import waveform_only_table
            acc["waveform_stage_alone"] = waveform_only_table(eng32, r64, eng32.wcfg.adc_conversion,
                                                              eng32.wcfg.pedestal)
        except Exception as exc:
            acc["waveform_stage_alone"] = {"error": str(exc)[:200]}
    except Exception as exc:  # the report is informative; its failure is shown, not hidden
        acc["error"] = str(exc)[:300]

    cpu = None
    if rank == 0 and not args.no_cpu:
        procs = 1
        v, ev, busy, wall = cpu_reference(960, procs)
        cpu = {"value": v, "unit": UNIT, "cores": procs, "kind": "port",
               "sample": f"{ev} events of the same workload through the oracle chain on 1 core ({busy:.1f} s)"}

    # the extra measurements below start from a device without the benchmark's own chain engines and batches
    eng32 = eng64 = batches = r = ds = r64 = r32 = pe64 = pe32 = None
    torch.cuda.synchronize()
    torch.cuda.empty_cache()

    dropin = None
    if rank == 0 and args.dropin_events > 0:
        try:
            dropin = e2e_dropin(geom, cond, args.dropin_events)
        except Exception as exc:                          # shown, not hidden
            dropin = {"error": str(exc)[:300]}
        torch.cuda.empty_cache()

    tables_io = None
    if rank == 0 and args.step_table_events > 0:
        try:
            tables_io = step_tables(geom, cond, args.step_table_events)
        except Exception as exc:                          # shown, not hidden
            tables_io = {"error": str(exc)[:300]}
        torch.cuda.empty_cache()

    lkchain = None
    if rank == 0 and args.lookup_chain_events > 0:
        try:
            lkchain = lookup_chain(args.lookup_chain_events)
        except Exception as exc:                          # shown, not hidden
            lkchain = {"error": str(exc)[:300]}
        torch.cuda.empty_cache()

    uneven = None
    if rank == 0 and args.uneven_waveforms > 0:
        uneven = uneven_pulse_fit(args.uneven_waveforms, 1 << 19)
        if not args.no_cpu:
            try:
                uneven["cpu_baseline"] = cpu_fit_baseline()
            except Exception as exc:                      # reported baseline only
                uneven["cpu_baseline"] = {"error": str(exc)[:200]}
        torch.cuda.empty_cache()

    lookup = None
    if rank == 0 and args.lookup_rows > 0:
        if args.lookup_precision == "fp32":
            lookup = lookup_substeps(args.lookup_rows, precision="fp32")
        else:
            lookup = lookup_substeps(args.lookup_rows)
            torch.cuda.empty_cache()
            if args.lookup_precision == "both":
                lookup["fp32_mixed"] = {k: v for k, v in lookup_substeps(args.lookup_rows, precision="fp32").items()
                                        if k in ("rows_per_s", "ms_per_call", "photons_per_row", "precision")}
        torch.cuda.empty_cache()

    full = None
    if rank == 0 and args.fullscale_events > 0:
        full = fullscale(args.fullscale_events, 1024, stage_events=args.fullscale_stage_events)
        torch.cuda.empty_cache()

    serve = None
    if rank == 0 and args.serve_jobs > 0:
        serve = serving(geom, cond, args.serve_jobs, args.serve_pool, [float(v) for v in args.serve_loads.split(",")],
                        capacity_jobs=args.serve_capacity_jobs or None,
                        policies=tuple(args.serve_policies.split(",")))

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms32 / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32-mixed", "data": "synthetic",
                "config": {"workload": f"{args.events} events/GPU, one 4x16 module of 450 cm counters, Poisson(40) "
                                       f"steps/event ({nsteps_total} steps, SoA f32 resident), full chain "
                                       f"steps->coincidences in batches of {args.batch} events, resident engine "
                                       f"(one CUDA graph replay per batch)",
                           "precision": "fp32-mixed (float-float LM solve, FP64 absolute times)",
                           "l2": f"inputs larger than L2 ({step_bytes / 1e9:.2f} GB of steps)"},
                "stage_engine_events_per_s": stage_value,
                "resident": resident,
                "fp64_plain_events_per_s": fp64,
                "fp32_over_fp64": (value / fp64) if fp64 else None,
                "fp32_vs_fp64": acc,
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
                "e2e_dropin": dropin, "step_tables": tables_io, "lookup_chain": lkchain,
                "gpu_launches": int(launches),
                "clocks": clk,
                "kernels": {k: {"launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / tot_ms, 4)}
                            for k, v in sorted(per_kernel.items(), key=lambda kv: -kv[1][1])[:12]},
                "dominant_kernel": top_group,
                "roofline": roofline_of(top_group),
                "roofline_waveform": roofline_of("k_wf_synth"),
                "roofline_pulse_fit": roofline_of("pulse fit"),
                "peak_hbm_gbs": hbm, "peak_kind": peak_kind,
                "uneven_pulse_fit": uneven,
                "lookup_photons": lookup,
                "serving": serve,
                "fullscale": full,
                "cpu_baseline": cpu}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
