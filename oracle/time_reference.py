"""Time the reference's own NumPy stages beside this repository's CPU port of them (the oracle), on the same inputs.

Test and measurement tooling, not part of the engine.  The reference is pure Python: it is importable where its
checkout is readable, but does not travel with this repository, so the CPU baseline that bench.py times on the GPU
host is the oracle port.  This script relates the two speeds on one machine: the deterministic stages the port
restates one to one, each called on identical inputs and checked to give identical outputs, timed best of `reps`:

  waveform synthesis   crvfastsim.reco.waveform._synthesize       vs oracle.synthesize
  pulse fit            crvfastsim.reco.pulsefit.reconstruct_full  vs oracle.reconstruct_full
  coincidence finder   crvfastsim.reco.coinc.find_event per event vs oracle.find_event per event

  python oracle/time_reference.py REFERENCE_CRV_DIR [N_EVENTS]     (or CRV_REFERENCE_DIR in the environment)

The inputs are the workload's (one 4 x 16 module, Poisson(40) steps per event, 12.55 ns sampling) through the port's
keyed photon and SiPM stages.  One process, one thread per library (OPENBLAS_NUM_THREADS=1).
"""
import json
import os
import sys
import tempfile
import time
from dataclasses import replace

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
os.environ.setdefault("OMP_NUM_THREADS", "1")
os.environ["CRVFS_CPU_ATTACHMENT"] = "numpy"

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, os.path.join(ROOT, "mu2e-fastsim_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def best(fn, reps):
    out, ts = None, []
    for _ in range(reps):
        t0 = time.perf_counter()
        out = fn()
        ts.append(time.perf_counter() - t0)
    return out, min(ts)


def main(ref_dir, n_events=128, reps=3):
    sys.path.insert(0, os.path.join(ROOT, "tests", "refshim"))
    sys.path.insert(0, ref_dir)
    from crvfastsim.reco import coinc as RC
    from crvfastsim.reco import pulsefit as RPF
    from crvfastsim.reco import synth as RSY
    from crvfastsim.reco import waveform as RWF
    from crvgpu import config as CF
    from crvgpu import geometry as GM
    from crvgpu import waveform as WV
    from oracle import oracle as O
    period = 12.55
    RPF.PERIOD = RWF.PERIOD = RSY.PERIOD = period
    geom = GM.module_geometry()
    cond = GM.default_conditions(geom)
    cfg = CF.ChainConfig()
    steps = GM.synthetic_steps(n_events, geom, seed=11)
    Q, _ = O.charges(steps, geom, cond, cfg.response, cfg.sipm, 7, cfg.window[1])
    res = {"events": n_events, "charges": int(len(Q["time"]))}
    # ---- waveform synthesis (no noise: the reference draws sequential normals, the port keyed ones)
    wc = CF.WaveformConfig()
    tmpl = WV.single_pe_template(wc)
    path = os.path.join(tempfile.mkdtemp(), "gumbel_spe.txt")
    t, v = WV.gumbel_raw(wc.gumbel_peak, wc.gumbel_mu, wc.gumbel_beta, wc.single_pe_precision, wc.single_pe_max_time)
    np.savetxt(path, np.c_[t, v], fmt="%.17g")
    rcfg = RWF.WaveformConfig(single_pe_file=path, single_pe_stretch=1.0, min_voltage=wc.min_voltage)
    labels = np.unique(Q["chan"])
    tab = np.random.default_rng(3).uniform(0, period, len(labels))
    lut = lambda lab: tab[np.searchsorted(labels, lab)]  # noqa: E731
    window = tuple(cfg.window)
    ref, t_ref = best(lambda: RWF._synthesize(Q["chan"], Q["time"], Q["charge"], lut, rcfg, window, None), reps)
    got, t_port = best(lambda: O.synthesize(Q["chan"], Q["time"], Q["charge"], lut, tmpl, wc, period, window, None),
                       reps)
    same = all(np.array_equal(ref[k], got[k]) for k in ("chan", "start", "starttdc", "volt", "adc"))
    res["waveform"] = {"reference_s": t_ref, "port_s": t_port, "port_over_reference_speed": t_ref / t_port,
                       "identical": bool(same), "digis": int(len(ref["chan"]))}
    # ---- pulse fit on the reco waveforms of these digis
    W = O.reco_waveforms(got, cond)
    pc = CF.RecoConfig()
    rpc = RPF.RecoConfig(**{k: getattr(pc, k) for k in RPF.RecoConfig.__dataclass_fields__ if hasattr(pc, k)})
    args = (W["adc"], W["n"], W["start"], W["ped"], W["area"], W["height"])
    ref, t_ref = best(lambda: RPF.reconstruct_full(*args, rpc), reps)
    got_p, t_port = best(lambda: O.reconstruct_full(*args, pc, period), reps)
    same = all(np.array_equal(np.asarray(ref[k]), np.asarray(got_p[k])) for k in ("wf", "seq", "failed")) and \
        np.allclose(ref["pe"], got_p["pe"], rtol=0, atol=0)
    res["pulse_fit"] = {"reference_s": t_ref, "port_s": t_port, "port_over_reference_speed": t_ref / t_port,
                        "identical": bool(same), "waveforms": int(len(W["n"])), "pulses": int(len(ref["pe"]))}
    # ---- coincidence finder, event by event, on the first pulses of these waveforms
    P = O.pulses_from_waveforms(W, cond, pc, period)
    G = GM.sector_geom(geom)
    fcfg = CF.workload_finder(G.sector_names)
    rG = RC.SectorGeom(sector=np.asarray(G.sector), layer=np.asarray(G.layer),
                       counter_in_type=np.asarray(G.counter_in_type), x=np.asarray(G.x), y=np.asarray(G.y),
                       pos=np.asarray(G.pos), length_dir=np.asarray(G.length_dir),
                       sector_type=np.asarray(G.sector_type), sector_names=list(G.sector_names),
                       pos_side0=np.asarray(G.pos_side0), pos_side1=np.asarray(G.pos_side1),
                       sipms_side0=np.asarray(G.sipms_side0), sipms_side1=np.asarray(G.sipms_side1))
    base = fcfg.cuts[G.sector_names[0]]
    rcut = replace(RC.EXTRACTED_V04["EX"], **{k: getattr(base, k) for k in RC.SectorCuts.__dataclass_fields__})
    rcfg_f = RC.FinderConfig(cuts={G.sector_names[0]: rcut})
    wf = P["wf"]
    ev = W["ev"][wf]
    o = np.lexsort((P["seq"], wf, ev))
    ev, wf = ev[o], wf[o]
    idx = np.arange(len(ev)) - np.searchsorted(ev, ev)
    cols = {"idx": idx, "bar": W["bar"][wf], "sipm": W["sipm"][wf], "time": P["time"][o], "pe": P["pe"][o],
            "seq": P["seq"][o]}
    bounds = np.flatnonzero(np.r_[True, ev[1:] != ev[:-1], True])
    events = [{k: v[a:b] for k, v in cols.items()} for a, b in zip(bounds[:-1], bounds[1:])]
    status = np.asarray(cond.status)
    ref, t_ref = best(lambda: [RC.find_event(p, rG, status, rcfg_f, vectorized=False) for p in events], reps)
    got_c, t_port = best(lambda: [O.find_event(p, G, status, fcfg) for p in events], reps)
    nref = sum(len(r) for r in ref)
    nport = sum(len(r) for r in got_c)
    res["coinc"] = {"reference_s": t_ref, "port_s": t_port, "port_over_reference_speed": t_ref / t_port,
                    "events_with_pulses": len(events), "clusters_reference": nref, "clusters_port": nport}
    return res


if __name__ == "__main__":
    a = sys.argv[1:]
    ref_dir = a.pop(0) if a and os.path.isdir(a[0]) else os.environ.get("CRV_REFERENCE_DIR")
    if not ref_dir:
        sys.exit("time_reference.py: give the reference's CRV directory (the one holding crvfastsim)")
    print(json.dumps(main(ref_dir, int(a[0]) if a else 128), indent=1))
