"""Generate the golden fixtures of the CRV response chain by running the reference NumPy stages.

Run here (where the reference checkout is readable):  python tests/golden/make_golden.py [REFERENCE_CRV_DIR] [NAME ...]
(NAME: pulsefit, concat, waveform, waveform_gate, coinc, stats, pixelid, lookup, lookup_file, lookup_fuzz, lookup_chain,
attach, chaintests, readout, wiring, propagation, pulsecache, pulsetests; default all)
The reference is imported from REFERENCE_CRV_DIR (or the CRV_REFERENCE_DIR environment variable; one of them is
required: the directory that holds the reference's crvfastsim package) with the small stand-ins in
tests/refshim for pandas and the core library.  The sampling period is patched to 12.55 ns in every reference
module that binds it (pulsefit, waveform, synth), as the workload specifies; one pulse-fit set keeps 12.5 ns.

Fixtures (compressed .npz, a few hundred kB in total):
  pulsefit.npz   reconstruct / reconstruct_full outputs for single-pulse, KPP-like, uneven multi-pulse and edge-case
                 waveforms (crv/crvfastsim/reco/pulsefit.py:222-316)
  concat.npz     concat_waveforms grouping (pulsefit.py:319-345)
  waveform.npz   _synthesize digis with and without injected noise (crv/crvfastsim/reco/waveform.py:96-172) and the
                 resampled Gumbel single-PE template (waveform.py:46-62)
  waveform_gate.npz  _synthesize digis under eight digitisation windows cut from the ungated starts (exact and
                 one-ulp-inside edges, single-start windows, lower edges inside long pulse trains)
  coinc.npz      find_event clusters on three geometries, scalar and vectorised combination checks
                 (crv/crvfastsim/reco/coinc.py:289-392, coinc_cpu.py:11-51)
  stats.npz      statistics of the reference SiPM stage (sipm.py:102-198) and photon-count rule (photons.py:102-112)
  pixelid.npz    SiPM pixel ids by rule (sipm.py:80-91): pixel histograms of "truncate" and "lrint", PE per SiPM on
                 crowded SiPMs, and charge statistics with cross-talk and afterpulses under "lrint"
  lookup.npz     a synthetic lookup table and (step, SiPM) rows with the statistics of the reference substep kernel
                 (crv/crvfastsim/response/photons.py:163-224) over 16 generator seeds: mean photons per row, arrival
                 delay histogram; for the first 120 rows, the table bins the reference reads (its probability
                 lookups recorded in substep order); the delay / emission index search on random thresholds
  lookup_file.npz  two version-6 lookup-table files (one from the reference's own test double, one with edge cases:
                 reflector 1, minor version, a table without bins, empty and 255-long weight vectors) and the
                 reference's decoded arrays of each (lookup.py:149-192)
  lookup_fuzz.json  600 mutated images of the two lookup_file.npz files (byte flips, corrupted 8-byte fields,
                 truncations, inserted / deleted bytes) as recipes, with the reference's verdict on each: the hash of its
                 decoded arrays, or the exception its load raised
  pulsecache.npz the distinct reconstruct_full calls of the reference's normal-equation-cache tests
                 (crv/tests/test_pulsefit_normal_cache.py: an edge batch and a synthetic batch; 12.5 ns) with outputs
  pulsetests.npz every reconstruct call of the reference's own pulse-fit tests (crv/tests/test_reco_pulsefit.py:
                 injected-parameter recovery, below threshold, pedestal undershoot; at its stock 12.5 ns period), with
                 the reference's outputs
  chaintests.npz every chain.reco_waveforms and chain.tdc0_per_feb call of the reference's own chain-glue tests
                 (crv/tests/test_chain.py), and both on a multi-event digi sample (chain.py:219-231, 273-286)
  readout_calls.json  every readout.sensor_mask / apply / effective_status call of the reference's own readout-mask
                 tests (crv/tests/test_readout_mask.py; crv/crvfastsim/readout.py:9-72): tagged-JSON arguments and
                 the output or the exception raised
  wiring.npz     every chain.clusters call of the reference's pulse-configuration wiring and chain-contract tests
                 (crv/tests/test_chain_config_wiring.py, test_chain_reco_contract.py; NumPy backend): waveforms,
                 status and time offsets, the pulse configuration and the flat pulse table (chain.py:296-362; 12.5 ns)
  propagation.npz  every photons.table_propagation and photons.bar_ratios call of the reference's propagation tests
                 (crv/tests/test_propagation.py): the known-value table and its fit, geometries, ratio maps and the
                 per-bar ratios or the KeyError raised (photons.py:229-289)
  attach.npz     every find_event call of the reference's own attachment boundary tests
                 (crv/tests/test_coinc_attachment_cpu.py: strict windows, ties, order, configuration flags), run under
                 pytest with find_event recorded: inputs, geometry, cuts, finder flags and the reference's clusters
  lookup_chain.npz  make_photons with two synthetic tables (reflector 0 and 1) on a two-sector geometry
                 (photons.py:292-371): table propagation fits, per-bar speed / attenuation ratios, the rows of
                 iter_rows (every field but the drawn photon counts), and over 16 seeds the mean photons per (step,
                 channel) and the arrival-delay histogram
"""
import os
import sys
import tempfile
from dataclasses import replace
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ARGS = sys.argv[1:]
if ARGS and os.path.isdir(ARGS[0]):
    REF = Path(ARGS.pop(0))
elif os.environ.get("CRV_REFERENCE_DIR"):
    REF = Path(os.environ["CRV_REFERENCE_DIR"])
else:
    sys.exit("make_golden.py: give the reference's CRV directory (the one holding crvfastsim) as the first argument "
             "or in CRV_REFERENCE_DIR")
ONLY = set(ARGS)
sys.path.insert(0, str(HERE.parent / "refshim"))
sys.path.insert(0, str(REF))
os.environ["CRVFS_CPU_ATTACHMENT"] = "numpy"

from crvfastsim.reco import coinc as C          # noqa: E402
from crvfastsim.reco import pulsefit as PF      # noqa: E402
from crvfastsim.reco import synth as SY         # noqa: E402
from crvfastsim.reco import waveform as WF      # noqa: E402
from crvfastsim.response import photons as PH   # noqa: E402
from crvfastsim.response import sipm as SI      # noqa: E402

PERIOD = 12.55


def set_period(p):
    PF.PERIOD = p
    WF.PERIOD = p
    SY.PERIOD = p


# ---------------------------------------------------------------------------------------------------------------------
# pulse fit

def gumbel(t, A, mu, b):
    z = (t - mu) / b
    return A * np.exp(-z - np.exp(-z))


def single_pulses(rng, W=160, n=24, start=10):
    t = (start + np.arange(n)) * PERIOD
    A = rng.uniform(300, 2000, W)
    mu = (start + 6) * PERIOD + rng.uniform(-6, 6, W)
    b = rng.uniform(14, 24, W)
    y = gumbel(t[None, :], A[:, None], mu[:, None], b[:, None])
    adc = np.round(y + 100.0 + rng.normal(0, 2.0, (W, n))).astype(np.int64)
    return adc, np.full(W, n), np.full(W, start), np.full(W, 100.0), np.full(W, 400.0), np.full(W, 30.0)


def uneven(rng, W=120):
    """Uneven multi-pulse waveforms: lengths over {32, 64, 128, 256, 512}, 1-12 pulses, log-uniform 5-500 PE."""
    lens = rng.choice([32, 64, 128, 256, 512], W)
    L = int(lens.max())
    area = 400.0
    adc = np.zeros((W, L), np.int64)
    start = rng.integers(0, 200, W)
    for w in range(W):
        n = lens[w]
        t = (start[w] + np.arange(n)) * PERIOD
        y = np.zeros(n)
        for _ in range(rng.integers(1, 13)):
            pe = np.exp(rng.uniform(np.log(5), np.log(500)))
            b = rng.uniform(10, 25)
            mu = t[0] + rng.uniform(0, n * PERIOD)
            y += gumbel(t, pe * area / b, mu, b)
        adc[w, :n] = np.clip(np.round(y + 100.0 + rng.normal(0, 2.0, n)), 0, 4095)
    return adc, lens, start, np.full(W, 100.0), np.full(W, area), np.full(W, area / 15.0)


def edge_cases():
    rows = []
    n = 24
    t = (10 + np.arange(n)) * PERIOD
    rows.append(np.full(n, 100))                                        # flat
    rows.append(np.full(n, 4095))                                       # saturated flat
    sat = np.clip(np.round(gumbel(t, 30000.0, 16 * PERIOD, 19.0) + 100), 0, 4095)
    rows.append(sat)                                                     # saturated pulse (plateau)
    rows.append(np.round(gumbel(t, 800.0, 16 * PERIOD, 19.0) + 90.0))  # pedestal undershoot
    rows.append(np.round(gumbel(t, 30.0, 16 * PERIOD, 19.0) + 100.0))  # below threshold
    rows.append(np.round(gumbel(t, 800.0, 11 * PERIOD, 19.0) + 100.0))  # peak at the start
    rows.append(np.round(gumbel(t, 800.0, 33 * PERIOD, 19.0) + 100.0))  # peak at the end
    p2 = gumbel(t, 900.0, 14 * PERIOD, 15.0) + gumbel(t, 600.0, 19 * PERIOD, 15.0)
    rows.append(np.round(p2 + 100.0))                                   # two overlapping pulses
    pl = np.full(n, 100.0); pl[8:12] = 400; pl[12:14] = 200            # plateau then fall
    rows.append(pl)
    adc = np.stack(rows).astype(np.int64)
    W = len(adc)
    nn = np.full(W, n)
    extra = np.stack([np.round(gumbel(t, 800.0, 16 * PERIOD, 19.0) + 100.0)] * 4).astype(np.int64)
    adc = np.concatenate([adc, extra])
    nn = np.concatenate([nn, [1, 2, 3, 7]])                              # short valid lengths
    W = len(adc)
    return adc, nn, np.full(W, 10), np.full(W, 100.0), np.full(W, 400.0), np.full(W, 30.0)


def run_pulsefit(tag, args, out, full=False):
    adc, n, st, ped, area, height = args
    f = PF.reconstruct_full if full else PF.reconstruct
    r = f(adc, n, st, ped, area, height, PF.RecoConfig())
    out[f"{tag}_adc"], out[f"{tag}_n"], out[f"{tag}_start"] = adc, n, st
    out[f"{tag}_ped"], out[f"{tag}_area"], out[f"{tag}_height"] = ped, area, height
    for k, v in r.items():
        out[f"{tag}_out_{k}"] = v


def make_pulsefit():
    rng = np.random.default_rng(101)
    out = {}
    set_period(PERIOD)
    run_pulsefit("single", single_pulses(rng), out)
    adc, n, st, ped, area, height = SY.waveforms(40, seed=3, L=12)
    run_pulsefit("kpp", (adc, n, st, ped, area, height), out)
    run_pulsefit("uneven", uneven(rng), out, full=True)
    run_pulsefit("edge", edge_cases(), out, full=True)
    set_period(12.5)
    run_pulsefit("p125", single_pulses(np.random.default_rng(7), W=40), out)
    set_period(PERIOD)
    out["period"] = np.array([PERIOD])
    np.savez_compressed(HERE / "pulsefit.npz", **out)


def make_concat():
    rng = np.random.default_rng(5)
    nd = 400
    key = np.sort(rng.integers(0, 20, nd))
    bar = rng.integers(0, 3, nd)
    sipm = rng.integers(0, 2, nd)
    o = np.lexsort((bar, key))
    key, bar, sipm = key[o], bar[o], sipm[o]
    lens = np.full(nd, 12)
    tdc = np.zeros(nd, np.int64)
    for i in range(1, nd):
        same = key[i] == key[i - 1] and bar[i] == bar[i - 1] and sipm[i] == sipm[i - 1]
        tdc[i] = tdc[i - 1] + (12 if (same and rng.random() < 0.5) else int(rng.integers(13, 40)))
    flat = rng.integers(0, 4096, nd * 12)
    gid, mat, n, start, first = PF.concat_waveforms(key, bar, sipm, tdc, flat, lens)
    np.savez_compressed(HERE / "concat.npz", key=key, bar=bar, sipm=sipm, tdc=tdc, flat=flat, lens=lens, gid=gid,
                        mat=mat, n=n, start=start, first=first)


# ---------------------------------------------------------------------------------------------------------------------
# waveform synthesis

class InjectedNormal:
    """rng stand-in: normal(loc, scale, size) = loc + scale * Z[:size] from a fixed standard-normal matrix."""

    def __init__(self, Z):
        self.Z = Z
        self.calls = []

    def normal(self, loc, scale, size):
        C_, L_ = size
        self.calls.append(size)
        return loc + scale * self.Z[:C_, :L_]


def gumbel_template_file(path, peak=0.0055, mu=15.0, beta=10.0, precision=0.5, max_time=100.0):
    t = np.arange(0.0, max_time + precision / 2, precision)
    v = peak * np.e * np.exp(-(t - mu) / beta - np.exp(-(t - mu) / beta))
    np.savetxt(path, np.c_[t, v], fmt="%.17g")
    return t, v


def charges_sample(rng, nchan=150):
    chans, times, qs = [], [], []
    qref = 2.652e-13
    for c in range(nchan):
        lab = 40000 + 3 * c                                              # arbitrary labels, increasing
        ncl = rng.integers(1, 4)
        t0s = np.sort(rng.uniform(-40.0, 1700.0, ncl))
        tt = []
        for t0 in t0s:
            k = rng.integers(1, 60)
            tt.append(t0 + np.sort(rng.exponential(8.0, k)))
        tt = np.sort(np.concatenate(tt))
        q = qref * rng.choice([1.0, 0.93, 0.5, 0.07, 1.0], len(tt))
        chans.append(np.full(len(tt), lab)); times.append(tt); qs.append(q)
    return np.concatenate(chans), np.concatenate(times), np.concatenate(qs)


def make_waveform():
    set_period(PERIOD)
    rng = np.random.default_rng(11)
    tmpdir = tempfile.mkdtemp()
    path = os.path.join(tmpdir, "gumbel_spe.txt")
    traw, vraw = gumbel_template_file(path)
    cfg = WF.WaveformConfig(single_pe_file=path, single_pe_stretch=1.0, min_voltage=5 * 0.0055)
    tmpl = WF.single_pe_template(cfg.single_pe_file, cfg.single_pe_precision, cfg.single_pe_stretch,
                                 cfg.single_pe_max_time)
    chan, time, charge = charges_sample(rng)
    uch = np.unique(chan)
    tdc0_tab = rng.uniform(0, PERIOD, len(uch))
    lut = lambda lab: tdc0_tab[np.searchsorted(uch, lab)]              # noqa: E731
    window = (0.0, 128 * PERIOD)
    out = dict(template=tmpl, traw=traw, vraw=vraw, chan=chan, time=time, charge=charge, uch=uch,
               tdc0_tab=tdc0_tab, window=np.array(window), min_voltage=np.array([cfg.min_voltage]),
               stretch=np.array([cfg.single_pe_stretch]))
    a = WF._synthesize(chan, time, charge, lut, cfg, window, None)
    for k, v in a.items():
        out[f"clean_{k}"] = v
    Z = np.random.default_rng(12).standard_normal((4000, 600))
    inj = InjectedNormal(Z)
    b = WF._synthesize(chan, time, charge, lut, cfg, window, inj)
    assert len(inj.calls) == 1
    out["noise_shape"] = np.array(inj.calls[0])
    out["noise_Z"] = Z[:inj.calls[0][0], :inj.calls[0][1]]
    for k, v in b.items():
        out[f"noisy_{k}"] = v
    np.savez_compressed(HERE / "waveform.npz", **out)


def make_waveform_gate():
    """The digitisation window gate of the ZS scan (waveform.py:150-160): a start outside the window neither makes a
    digi nor moves the scan on, so a trigger before the gate does not hide an in-gate continuation, and both bounds
    are inclusive.  Windows are cut from the ungated starts themselves (exact edges, one ulp inside, one-start
    windows, mid-train lower edges) on a sample with long pulse trains (many consecutive 12-sample digis)."""
    set_period(PERIOD)
    rng = np.random.default_rng(21)
    tmpdir = tempfile.mkdtemp()
    path = os.path.join(tmpdir, "gumbel_spe.txt")
    gumbel_template_file(path)
    cfg = WF.WaveformConfig(single_pe_file=path, single_pe_stretch=1.0, min_voltage=5 * 0.0055)
    tmpl = WF.single_pe_template(cfg.single_pe_file, cfg.single_pe_precision, cfg.single_pe_stretch,
                                 cfg.single_pe_max_time)
    chan, time, charge = charges_sample(rng, nchan=60)
    qref = 2.652e-13
    trains = []
    for c in range(12):                                                  # steady trains of 20-90 samples
        t0 = rng.uniform(-60.0, 1200.0)
        tt = t0 + np.arange(0.0, rng.uniform(250.0, 1100.0), rng.uniform(1.0, 2.5))
        trains.append((np.full(len(tt), 50000 + 3 * c), tt, np.full(len(tt), 1.5 * qref)))
    chan = np.concatenate([chan] + [t[0] for t in trains])
    time = np.concatenate([time] + [t[1] for t in trains])
    charge = np.concatenate([charge] + [t[2] for t in trains])
    uch = np.unique(chan)
    tdc0_tab = rng.uniform(0, PERIOD, len(uch))
    lut = lambda lab: tdc0_tab[np.searchsorted(uch, lab)]              # noqa: E731
    base = WF._synthesize(chan, time, charge, lut, cfg, (-1e5, 1e5), None)
    S = np.unique(base["start"])
    up, dn = np.inf, -np.inf
    tr = base["chan"] >= 50000
    first_train = np.array([base["start"][tr & (base["chan"] == c)].min() for c in np.unique(base["chan"][tr])])
    q = lambda f: S[int(f * (len(S) - 1))]                               # noqa: E731
    windows = [
        (q(0.2), q(0.8)),                                                # exact inclusive edges
        (np.nextafter(q(0.2), up), np.nextafter(q(0.8), dn)),            # one ulp inside: both edge starts drop
        (q(0.5), np.nextafter(q(0.5), up)),                              # a single start
        (np.nextafter(q(0.5), dn), q(0.5)),
        (float(np.median(first_train)) + 5.5 * PERIOD, 1500.0),          # lower edge inside the trains
        (float(first_train.min()) + 13.0 * PERIOD, float(first_train.max()) + 30.25 * PERIOD),
        (200.0, 1500.0),
        (-1e5, 1e5),
    ]
    out = dict(template=tmpl, chan=chan, time=time, charge=charge, uch=uch, tdc0_tab=tdc0_tab,
               windows=np.array(windows), min_voltage=np.array([cfg.min_voltage]),
               stretch=np.array([cfg.single_pe_stretch]))
    for i, w in enumerate(windows):
        r = WF._synthesize(chan, time, charge, lut, cfg, w, None)
        for k in ("chan", "start", "tdc0", "starttdc", "volt", "adc"):
            out[f"w{i}_{k}"] = r[k]
    np.savez_compressed(HERE / "waveform_gate.npz", **out)


# ---------------------------------------------------------------------------------------------------------------------
# coincidences

def module_geom(n_layers=4, n_counters=16, pitch=51.3, layer_pitch=21.1, stagger=12.8, half_length=2250.0):
    """One module of 4 x 16 counters, lengths along z, widths along x, thickness along y (one sector EX)."""
    layer = np.repeat(np.arange(n_layers), n_counters)
    counter = np.tile(np.arange(n_counters), n_layers)
    x = (counter - (n_counters - 1) / 2) * pitch + stagger * (layer % 2)
    y = (layer - (n_layers - 1) / 2) * layer_pitch
    nb = len(layer)
    return C.SectorGeom(sector=np.zeros(nb, int), layer=layer, counter_in_type=counter, x=x, y=y,
                        pos=np.column_stack([x, y, np.zeros(nb)]), length_dir=np.array([2]),
                        sector_type=np.array([1]), sector_names=["EX"], pos_side0=np.array([-half_length]),
                        pos_side1=np.array([half_length]), sipms_side0=np.array([True]),
                        sipms_side1=np.array([True]))


def two_sector_geom():
    """Two sectors of different types and lengths, the second read out on side 0 only."""
    a = module_geom()
    b = module_geom(half_length=1150.0)
    nb = len(a.layer)
    return C.SectorGeom(sector=np.r_[np.zeros(nb, int), np.ones(nb, int)], layer=np.r_[a.layer, b.layer],
                        counter_in_type=np.r_[a.counter_in_type, b.counter_in_type], x=np.r_[a.x, b.x + 2000.0],
                        y=np.r_[a.y, b.y], pos=np.r_[a.pos, b.pos + [2000.0, 0, 300.0]], length_dir=np.array([2, 2]),
                        sector_type=np.array([1, 2]), sector_names=["EX", "T1"],
                        pos_side0=np.array([-2250.0, -850.0]), pos_side1=np.array([2250.0, 1450.0]),
                        sipms_side0=np.array([True, True]), sipms_side1=np.array([True, False]))


def test_geom8():
    """The eight-bar, one-sector geometry of the reference attachment tests (two counters x four layers)."""
    layer = np.tile(np.arange(4), 2)
    x = np.repeat([0., 400.], 4)
    y = layer * 10.
    return C.SectorGeom(sector=np.zeros(8, dtype=int), layer=layer, counter_in_type=np.repeat([0, 1], 4), x=x, y=y,
                        pos=np.column_stack([x, y, np.zeros(8)]), length_dir=np.array([2]),
                        sector_type=np.array([1]), sector_names=["EX"], pos_side0=np.array([-700.]),
                        pos_side1=np.array([700.]), sipms_side0=np.array([True]), sipms_side1=np.array([True]))


def flatten_clusters(rows_per_event):
    """Flatten per-event cluster rows into arrays (event, fields) and a member table."""
    out = {k: [] for k in ("ev", "type", "pe", "start", "end", "slope", "avgtime", "poscalc", "pos", "sidepe",
                           "sidetime", "sidehits", "nlayers")}
    mem_cl, mem_idx = [], []
    for e, rows in rows_per_event:
        for r in rows:
            n = len(out["ev"])
            out["ev"].append(e); out["type"].append(r["sectortype"]); out["pe"].append(r["pe"])
            out["start"].append(r["start"]); out["end"].append(r["end"]); out["slope"].append(r["slope"])
            out["avgtime"].append(r["avgtime"]); out["poscalc"].append(r["poscalc"])
            out["pos"].append(np.asarray(r["pos"], float)); out["sidepe"].append(r["sidepe"])
            out["sidetime"].append(r["sidetime"]); out["sidehits"].append(r["sidehits"])
            out["nlayers"].append(len(r["layers"]))
            mem_cl += [n] * len(r["pulses"]); mem_idx += list(r["pulses"])
    res = {k: np.asarray(v) for k, v in out.items()}
    res["pos"] = np.asarray(out["pos"], float).reshape(-1, 3)
    res["mem_cl"] = np.asarray(mem_cl, np.int64)
    res["mem_idx"] = np.asarray(mem_idx, np.int64)
    return res


def random_small_events(rng, n_events):
    """Small events on the eight-bar geometry with quantised times and PEs (ties, attachment, secondary pulses)."""
    ev, idx, bar, sipm, time, pe, seq = [], [], [], [], [], [], []
    for e in range(n_events):
        k = rng.integers(3, 14)
        for i in range(k):
            ev.append(e); idx.append(i); bar.append(rng.integers(0, 8)); sipm.append(rng.integers(0, 4))
            time.append(100.0 + 2.5 * rng.integers(0, 8)); pe.append(float(rng.choice([3.0, 5.0, 10.0, 20.0])))
            seq.append(int(rng.random() < 0.1))
    return dict(ev=np.array(ev), idx=np.array(idx), bar=np.array(bar), sipm=np.array(sipm), time=np.array(time),
                pe=np.array(pe), seq=np.array(seq))


def run_coinc(tag, P, G, cfg, status, out):
    for vec in (False, True):
        rows = []
        ue = np.unique(P["ev"])
        for e in ue:
            m = P["ev"] == e
            p = {k: P[k][m] for k in ("idx", "bar", "sipm", "time", "pe", "seq")}
            rows.append((e, C.find_event(p, G, status, cfg, vectorized=vec)))
        fl = flatten_clusters(rows)
        for k, v in fl.items():
            out[f"{tag}_{'vec' if vec else 'scalar'}_{k}"] = v
    for k in ("ev", "idx", "bar", "sipm", "time", "pe", "seq"):
        out[f"{tag}_in_{k}"] = P[k]
    out[f"{tag}_status"] = status
    for k in ("sector", "layer", "counter_in_type", "x", "y", "pos", "length_dir", "sector_type", "pos_side0",
              "pos_side1", "sipms_side0", "sipms_side1"):
        out[f"{tag}_G_{k}"] = np.asarray(getattr(G, k))
    out[f"{tag}_G_sector_names"] = np.array(G.sector_names)


def cuts_array(cfg, names):
    return np.array([[getattr(cfg.cuts[n], f) for f in ("pe_threshold", "max_dt_adjacent", "max_dt", "min_slope",
                                                          "max_slope", "max_slope_diff", "coincidence_layers",
                                                          "min_cluster_pes", "initial_max_distance",
                                                          "final_max_distance")] for n in names])


def make_coinc():
    out = {}
    base = replace(C.EXTRACTED_V04["EX"], max_dt=10.0, coincidence_layers=3)
    # module: synthetic track + noise events from the reference generator
    G = module_geom()
    cfg = C.FinderConfig(cuts={"EX": base})
    P = SY.coinc_events(300, G, seed=4, noise_mean=10.0, shower_frac=0.1, shower_mean=30.0)
    status = np.zeros(4 * len(G.layer), np.int64)
    status[[5, 9, 130]] = [1, 4, 2]                                     # compensated partners
    run_coinc("module", P, G, cfg, status, out)
    out["module_cuts"] = cuts_array(cfg, ["EX"])
    # two sector types, one single-sided
    G2 = two_sector_geom()
    cfg2 = C.FinderConfig(cuts={"EX": base, "T1": replace(base, max_dt=8.0, coincidence_layers=4)})
    P2 = SY.coinc_events(200, G2, seed=9, noise_mean=6.0, shower_frac=0.1, shower_mean=30.0)
    run_coinc("two", P2, G2, cfg2, np.zeros(4 * len(G2.layer), np.int64), out)
    out["two_cuts"] = cuts_array(cfg2, ["EX", "T1"])
    # eight bars: ties and attachment
    G3 = test_geom8()
    cfg3 = C.FinderConfig(cuts={"EX": replace(C.EXTRACTED_V04["EX"], max_dt=10.0)})
    P3 = random_small_events(np.random.default_rng(21), 400)
    run_coinc("eight", P3, G3, cfg3, np.zeros(32, np.int64), out)
    out["eight_cuts"] = cuts_array(cfg3, ["EX"])
    fc = C.FinderConfig()
    out["finder"] = np.array([fc.fiber_signal_speed, fc.max_time_interval, fc.time_offset])
    np.savez_compressed(HERE / "coinc.npz", **out)


# ---------------------------------------------------------------------------------------------------------------------
# statistics of the stochastic reference stages

def make_stats():
    out = {}
    rng = np.random.default_rng(31)
    cfg = replace(SI.SiPMConfig(pixel_id="truncate"), cross_talk=0.05, trap0_prob=0.02)
    S = 4000
    n = rng.poisson(80, S)
    chan = np.repeat(np.arange(S), n)
    t = np.repeat(rng.uniform(0, 1500, S), n) + rng.exponential(7.4, len(chan))
    r = SI.simulate(chan, t, np.arange(len(chan)), np.ones((40, 40)), cfg, np.random.default_rng(32), t_end=1606.4)
    out["sipm_nphot"] = np.array([len(chan)])
    out["sipm_charges"] = np.array([len(r["pe"])])
    out["sipm_pe_sum"] = np.array([r["pe"].sum()])
    out["sipm_frac_low"] = np.array([(r["pe"] < 0.99).mean()])
    out["sipm_S"], out["sipm_n"] = np.array([S]), n
    out["sipm_tspread_seed"] = np.array([31])
    for m in (0.5, 3.0, 9.9, 10.1, 40.0, 200.0):
        c = PH._per_substep(np.full(200_000, m), np.ones(200_000, np.int64), np.random.default_rng(int(m * 10)))
        out[f"count_{m}"] = np.array([c.mean(), c.var()])
    np.savez_compressed(HERE / "stats.npz", **out)


def make_pixelid():
    """SiPM pixel ids (sipm.py:80-91): the reference's pixel histograms over the 41 x 41 ids for both rules on a map with
    content in bins 6-33 and in the last bin (39, 39) (lrint reaches pixel 40 only from there); PE per SiPM on crowded
    SiPMs (saturation differs between the rules, no cross-talk); and charge statistics with cross-talk and afterpulses
    under lrint."""
    rng = np.random.default_rng(41)
    pmap = np.zeros((40, 40))
    pmap[6:34, 6:34] = rng.uniform(0.0, 1.0, (28, 28))
    pmap[39, 39] = 20.0
    out = {"pmap": pmap}
    for pid in SI.PIXEL_IDS:
        x, y = SI.draw_pixels(pmap, 400_000, np.random.default_rng(42), pid)
        out[f"hist_{pid}"] = np.bincount(x * 41 + y, minlength=41 * 41)
        cfg = replace(SI.SiPMConfig(pixel_id=pid), cross_talk=0.0, trap0_prob=0.0)
        chan = np.repeat(np.arange(400), 400)
        r = SI.simulate(chan, np.zeros(len(chan)), np.arange(len(chan)), pmap, cfg, np.random.default_rng(43))
        out[f"crowded_pe_{pid}"] = np.array([r["pe"].sum() / 400])
    cfg = replace(SI.SiPMConfig(pixel_id="lrint"), cross_talk=0.05, trap0_prob=0.02)
    S = 4000
    trng = np.random.default_rng(45)                                     # photon counts and times: from the seed
    n = trng.poisson(80, S)
    chan = np.repeat(np.arange(S), n)
    t = np.repeat(trng.uniform(0, 1500, S), n) + trng.exponential(7.4, len(chan))
    r = SI.simulate(chan, t, np.arange(len(chan)), pmap, cfg, np.random.default_rng(44), t_end=1606.4)
    out["lrint_seed"], out["lrint_S"] = np.array([45]), np.array([S])
    out["lrint_charges"] = np.array([len(r["pe"])])
    out["lrint_pe_sum"] = np.array([r["pe"].sum()])
    out["lrint_frac_low"] = np.array([(r["pe"] < 0.99).mean()])
    np.savez_compressed(HERE / "pixelid.npz", **out)


def write_v6(rng, reflector=1, minor=2, theta_edges=1):
    """A version-6 lookup-table image in the documented layout (crv/crvfastsim/response/lookup.py:3-11) with the edge
    cases: reflector 1, a minor version, a table without bins (one theta edge), empty and 255-long weight vectors."""
    import struct
    edges = {"x": np.linspace(0, 8, 4), "y": np.linspace(-20, 20, 3), "z": np.linspace(-500, 500, 5),
             "beta": np.linspace(0.5, 1, 3), "theta": np.linspace(0, np.pi, theta_edges), "phi": np.linspace(0, 1, 3),
             "r": np.linspace(0, 0.7, 2)}
    b = bytearray(struct.pack("<3i4x", 6, minor, reflector))
    b += rng.uniform(0.1, 30.0, 10).astype("<f8").tobytes()
    for n in (3, 0):
        cm = np.c_[np.linspace(0.5, 1.0, n), rng.uniform(0, 200, n)]
        b += struct.pack("<Q", n) + cm.astype("<f8").tobytes()
    for k in ("x", "y", "z", "beta", "theta", "phi", "r"):
        b += struct.pack("<Q", len(edges[k])) + edges[k].astype("<f8").tobytes()
    nb = {k: len(v) - 1 for k, v in edges.items()}
    ns = nb["x"] * nb["y"] * nb["z"]
    for n in (ns, ns * nb["beta"], nb["beta"] * nb["theta"] * nb["phi"] * nb["r"] * nb["z"]):
        for i in range(n):
            nd = int(rng.choice([0, 1, 5, 30, 255]))
            ne = int(rng.choice([0, 2, 7]))
            d = rng.integers(0, 256, nd).astype(np.uint8)
            e = rng.integers(0, 256, ne).astype(np.uint8)
            b += struct.pack("<If", i, float(rng.uniform(0, 0.05)))
            b += struct.pack("<Q", nd) + d.tobytes() + struct.pack("<Q", ne) + e.tobytes()
    return bytes(b)


def make_lookup_file():
    """Version-6 lookup-table files decoded by the reference's load (lookup.py:149-179): one written by the
    reference's own test double (crv/tests/test_lookup_library.py _write_table), one by write_v6 (edge cases)."""
    import importlib.util
    from crvfastsim.response import lookup as LK
    spec = importlib.util.spec_from_file_location("ref_lookup_tests", REF / "tests" / "test_lookup_library.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = {}
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        mod._write_table(d / "LookupTable_6000_0", np.random.default_rng(1))
        (d / "LookupTable_2370_1").write_bytes(write_v6(np.random.default_rng(2)))
        for tag, name in (("a", "6000_0"), ("b", "2370_1")):
            out[f"{tag}_image"] = np.frombuffer((d / f"LookupTable_{name}").read_bytes(), np.uint8)
            for k, v in LK.arrays(LK.load(name, str(d))).items():
                out[f"{tag}_{k}"] = np.asarray(v)
    np.savez_compressed(HERE / "lookup_file.npz", **out)


def mutate(image, recipe):
    """Apply a mutation recipe to a file image: ("set", offset, bytes), ("cut", length), ("ins", offset, bytes),
    ("del", offset, count).  tests/test_lookup_file.py applies the same recipes."""
    b = bytearray(image)
    for op in recipe:
        if op[0] == "set":
            b[op[1]:op[1] + len(op[2])] = bytes(op[2])
        elif op[0] == "cut":
            b = b[:op[1]]
        elif op[0] == "ins":
            b = b[:op[1]] + bytes(op[2]) + b[op[1]:]
        else:
            b = b[:op[1]] + b[op[1] + op[2]:]
    return bytes(b)


def decoded_hash(arrays):
    import hashlib
    h = hashlib.sha256()
    for k in sorted(arrays):
        a = np.ascontiguousarray(arrays[k])
        h.update(f"{k}|{a.dtype.str}|{a.shape}|".encode())
        h.update(a.tobytes())
    return h.hexdigest()


def make_lookup_fuzz():
    """Mutated version-6 images (byte flips, corrupted 8-byte fields, truncations, inserted / deleted bytes) of the two
    lookup_file.npz images, each decoded by the reference's load: the recipe, whether it loaded, and the hash of its
    decoded arrays (lookup.py:149-192).  Requires lookup_file.npz."""
    import json
    import struct
    from crvfastsim.response import lookup as LK
    g = np.load(HERE / "lookup_file.npz")
    rng = np.random.default_rng(6)
    cases = []
    with tempfile.TemporaryDirectory() as d:
        for tag in ("a", "b"):
            img = g[f"{tag}_image"].tobytes()
            for it in range(300):
                kind = it % 4
                if kind == 0:
                    rec = [("set", int(rng.integers(0, len(img))), [int(rng.integers(0, 256))])
                           for _ in range(int(rng.integers(1, 8)))]
                elif kind == 1:
                    vals = [2 ** 63 - 1, 2 ** 64 - 1, 2 ** 40, 1 << 20, 255, 0]
                    rec = [("set", int(rng.integers(0, len(img) - 8)),
                            list(struct.pack("<Q", vals[int(rng.integers(0, 6))])))]
                elif kind == 2:
                    rec = [("cut", int(rng.integers(0, len(img))))]
                elif rng.random() < 0.5:
                    rec = [("ins", int(rng.integers(0, len(img))),
                            [int(x) for x in rng.integers(0, 256, int(rng.integers(1, 5)))])]
                else:
                    rec = [("del", int(rng.integers(0, len(img))), int(rng.integers(1, 5)))]
                p = os.path.join(d, "LookupTable_9_9")
                with open(p, "wb") as f:
                    f.write(mutate(img, rec))
                try:
                    verdict = decoded_hash(LK.arrays(LK.load("9_9", d)))
                except Exception as e:                           # noqa: BLE001 (the reference's failure, recorded)
                    verdict = "error:" + type(e).__name__
                cases.append({"image": tag, "recipe": rec, "verdict": verdict})
    (HERE / "lookup_fuzz.json").write_text(json.dumps(cases, separators=(",", ":")))


def synthetic_lookup(rng, decay_time=7.4):
    """A small lookup table with the reference's layout (lookup.py:70-98): bin edges, arrival probabilities, delay and
    emission weights; geometry of a 2 cm x 5 cm counter with two fibre holes."""
    edges = {"x": np.linspace(0.0, 10.0, 6), "y": np.linspace(-26.0, 26.0, 11), "z": np.linspace(-1000.0, 1000.0, 9),
             "beta": np.linspace(0.4, 1.0, 4), "theta": np.linspace(0.0, np.pi, 5), "phi": np.linspace(0.0, np.pi, 4),
             "r": np.linspace(0.0, 0.7, 4)}
    nb = {k: len(v) - 1 for k, v in edges.items()}

    def table(n, D=24, E=4, pmax=0.02):
        d = rng.integers(0, 30, (n, D)).astype(np.uint8)
        e = rng.integers(0, 30, (n, E)).astype(np.uint8)
        return dict(prob=rng.uniform(0.0, pmax, n).astype(np.float32), delays=d, delay_sum=d.sum(1, dtype=np.int32),
                    emis=e, emis_sum=e.sum(1, dtype=np.int32))

    ns = nb["x"] * nb["y"] * nb["z"]
    tabs = {"scint": table(ns), "ckscint": table(ns * nb["beta"]),
            "ckfiber": table(nb["beta"] * nb["theta"] * nb["phi"] * nb["r"] * nb["z"], pmax=0.2)}
    geo = dict(half_thickness=9.64, half_width=25.42, half_length=1000.0, fiber_separation=26.0, hole_radius_x=2.0,
               hole_radius_y=1.0, fiber_radius=0.7, corner_radius=1.75, fiber_decay_time=decay_time)
    return edges, tabs, geo


def shaped_lookup(rng, decay_time=3.0):
    """synthetic_lookup with light propagation built in: arrival probabilities fall off as exp(-d / 1500 mm) and the
    delay weights peak 6 ns/m later with the distance d to the SiPM end (so the reference's propagation fits apply)."""
    edges, tabs, geo = synthetic_lookup(rng, decay_time)
    zc = 0.5 * (edges["z"][1:] + edges["z"][:-1]) + geo["half_length"]
    for name, T in tabs.items():
        n, D = T["delays"].shape
        nz = len(zc)
        zi = np.arange(n) % nz if name != "ckfiber" else np.arange(n) % nz
        T["prob"] = (T["prob"] * np.exp(-zc[zi] / 1500.0)).astype(np.float32)
        peak = np.clip(np.rint(2 + 0.006 * zc[zi]).astype(np.int64), 0, D - 1)
        w = rng.integers(0, 4, (n, D))
        w[np.arange(n), peak] += 60
        T["delays"] = w.astype(np.uint8)
        T["delay_sum"] = T["delays"].sum(1, dtype=np.int32)
    return edges, tabs, geo


def synthetic_rows(rng, R=1500):
    """(step, SiPM) rows of tracks through the counter: local start, step vector, times, photons per substep."""
    a = np.c_[rng.uniform(-9.5, 9.5, R), rng.uniform(-25, 25, R), rng.uniform(-950, 950, R)]
    d = np.c_[rng.normal(0, 4, R), rng.normal(0, 4, R), rng.normal(0, 20, R)]
    # a fifth of the rows cross the fibre holes' neighbourhood, so the fibre table is exercised
    f = rng.random(R) < 0.2
    a[f, 0] = rng.uniform(-0.6, 0.6, f.sum())
    a[f, 1] = np.where(rng.random(f.sum()) < 0.5, -13.0, 13.0) + rng.uniform(-0.5, 0.5, f.sum())
    d[f, 0] = rng.normal(0, 0.3, f.sum())
    d[f, 1] = rng.normal(0, 0.3, f.sum())
    t0 = rng.uniform(0, 1e3, R)
    dl = np.linalg.norm(d, axis=1)
    return {"s": a, "d": d, "t0": t0, "t1": t0 + rng.uniform(0.0, 0.2, R),
            "nsub": np.maximum((dl / 0.1).astype(np.int64), 1), "beta": rng.uniform(0.5, 1.0, R),
            "theta": np.arccos(np.clip(d[:, 2] / np.where(dl > 0, dl, 1.0), -1, 1)), "dev": rng.uniform(0.8, 1.2, R),
            "mu": rng.uniform(0.0, 2e-4, R), "step": np.arange(R, dtype=np.int64) * 7 + 3,
            "chan": (np.arange(R, dtype=np.int64) % 5000) * 4 + 1, "n_scint": rng.integers(0, 40, R),
            "n_ck_s": rng.integers(0, 4, R), "n_ck_f": rng.integers(0, 30, R)}


class _RecordingTable(np.ndarray):
    """A probability column that logs the index arrays it is read with (the bins a substep kernel selects)."""

    def __getitem__(self, idx):
        if isinstance(idx, np.ndarray) and idx.dtype.kind in "iu":
            _RecordingTable.log.append(np.asarray(idx).copy())
        return np.asarray(self).__getitem__(idx)


def reference_bins(L, rows):
    """Per table, the bins the reference's substep kernel reads for these rows, in its substep order."""
    from types import SimpleNamespace
    out = {}
    for name in ("scint", "ckscint", "ckfiber"):
        tabs = {k: SimpleNamespace(**vars(t)) for k, t in L.tables.items()}
        tabs[name].prob = np.asarray(L.tables[name].prob).view(_RecordingTable)
        _RecordingTable.log = []
        Lr = SimpleNamespace(**{**vars(L), "tables": tabs})
        PH._substep_photons(Lr, rows, np.random.default_rng(0))
        out[name] = np.concatenate(_RecordingTable.log) if _RecordingTable.log else np.zeros(0, np.int64)
    return out


def make_lookup(seeds=16):
    from types import SimpleNamespace
    rng = np.random.default_rng(73)
    edges, tabs, geo = synthetic_lookup(rng)
    rows = synthetic_rows(rng)
    L = SimpleNamespace(edges=edges, tables={k: SimpleNamespace(**v) for k, v in tabs.items()}, **geo)
    R = len(rows["nsub"])
    counts = np.zeros(R)
    H = 64
    hist = np.zeros(H)
    total = 0
    for s in range(seeds):
        st, ch, tm = PH._substep_photons(L, rows, np.random.default_rng(1000 + s))
        ri = (st - 3) // 7
        counts += np.bincount(ri, minlength=R)
        dt = tm - rows["t0"][ri]
        hist += np.bincount(np.clip(dt.astype(np.int64), 0, H - 1), minlength=H)
        total += len(st)
    out = {f"edge_{k}": v for k, v in edges.items()}
    for k, T in tabs.items():
        out.update({f"{k}_{f}": v for f, v in T.items()})
    out.update({f"geo_{k}": np.float64(v) for k, v in geo.items()})
    out.update({f"row_{k}": v for k, v in rows.items()})
    out.update(ref_seeds=np.int64(seeds), ref_counts=counts / seeds, ref_delay_hist=hist / seeds,
               ref_total=np.int64(total))
    sub = {k: v[:120] for k, v in rows.items()}
    for name, b in reference_bins(L, sub).items():
        out[f"ref_bins_{name}"] = b.astype(np.int32)
    # the delay / emission index search on random bins and thresholds (u x the bin's sum, u in [0, 1))
    qrng = np.random.default_rng(17)
    T = L.tables["scint"]
    qb = qrng.integers(0, len(T.prob), 4000)
    qd = qrng.random(4000) * T.delay_sum[qb]
    qe = qrng.random(4000) * T.emis_sum[qb]
    out.update(ref_search_bins=qb, ref_search_dthr=qd, ref_search_ethr=qe,
               ref_search_delay=PH._first_above(T.delays, qb, qd).astype(np.int32),
               ref_search_emis=PH._first_above(T.emis, qb, qe).astype(np.int32))
    np.savez_compressed(HERE / "lookup.npz", **out)


class _Col(np.ndarray):
    """A step-table column with pandas' to_numpy (the reference reads columns that way)."""

    def to_numpy(self):
        return np.asarray(self)


class _Steps:
    def __init__(self, cols):
        self.cols = {k: np.asarray(v).view(_Col) for k, v in cols.items()}

    def __getattr__(self, k):
        try:
            return self.__dict__["cols"][k]
        except KeyError:
            raise AttributeError(k)

    def __getitem__(self, k):
        return self.cols[k]


def lookup_chain_inputs(rng, n_steps=400):
    """Two tables (reflector 0 and 1), a geometry of two sectors (EX: 2 modules x 4 bars, reflector 0; T1: 4 bars,
    reflector -1), muon / electron / proton / photon / ion steps inside the bars."""
    from types import SimpleNamespace
    tabs = {}
    for name, refl, seed in (("tabA", 0, 5), ("tabB", 1, 6)):
        e, t, g = shaped_lookup(np.random.default_rng(seed), decay_time=3.0)
        tabs[name] = (e, t, g, refl)
    nb = 12
    sector = np.r_[np.zeros(8, np.int64), np.ones(4, np.int64)]
    module = np.r_[np.repeat([0, 1], 4), np.zeros(4, np.int64)]
    l2w = np.array([[0, 1, 2]] * 8 + [[1, 0, 2]] * 4, np.int8)
    center = np.c_[np.arange(nb) * 30.0, np.arange(nb) * 55.0 - 300.0, np.full(nb, 100.0)]
    geom = SimpleNamespace(nbars=nb, sector=sector, module=module, local_to_world=l2w, center=center,
                           sector_names=["EX", "T1"])
    bar = rng.integers(0, nb, n_steps)
    loc0 = np.c_[rng.uniform(-9, 9, n_steps), rng.uniform(-24, 24, n_steps), rng.uniform(-900, 900, n_steps)]
    dirn = rng.normal(0, 1, (n_steps, 3))
    dirn /= np.linalg.norm(dirn, axis=1)[:, None]
    length = rng.uniform(2.0, 25.0, n_steps)
    loc1 = loc0 + dirn * length[:, None]
    w0, w1 = np.zeros((n_steps, 3)), np.zeros((n_steps, 3))
    for k in range(3):
        ax = l2w[bar, k]
        w0[np.arange(n_steps), ax] = center[bar, ax] + loc0[:, k]
        w1[np.arange(n_steps), ax] = center[bar, ax] + loc1[:, k]
    p0 = rng.uniform(50, 2000, n_steps)
    t0 = rng.uniform(0, 1000, n_steps)
    t1 = t0 + length / 299.8
    t0[::37] = np.nan                                  # skipped, as CrvPhotonGenerator skips them
    cols = dict(bar=bar, x0=w0[:, 0], y0=w0[:, 1], z0=w0[:, 2], x1=w1[:, 0], y1=w1[:, 1], z1=w1[:, 2],
                px0=dirn[:, 0] * p0, py0=dirn[:, 1] * p0, pz0=dirn[:, 2] * p0, p1=p0 * 0.99, t0=t0, t1=t1,
                edep=rng.uniform(0.2, 3.0, n_steps), len=length)
    pdg = rng.choice(np.array([13, -13, 11, 2212, 22, 211, 1000060120], np.int64), n_steps)
    deviation = rng.normal(0, 0.05, 4 * nb)
    return tabs, geom, cols, pdg, deviation


def make_lookup_chain(seeds=16):
    from types import SimpleNamespace
    rng = np.random.default_rng(91)
    tabs, geom, cols, pdg, deviation = lookup_chain_inputs(rng)
    ck = np.array([[0.474, 0.0], [1.0, 2.6]])
    tables = {}
    for name, (e, t, g, refl) in tabs.items():
        tables[name] = SimpleNamespace(name=name, reflector=refl, edges=e, ck_scint=ck, ck_fiber=ck * 0.5,
                                       tables={k: SimpleNamespace(**v) for k, v in t.items()}, **g)
    cfg = PH.ResponseConfig(sectors={"EX": PH.SectorConfig("tabA", 0, 1500.0),
                                     "T1": PH.SectorConfig("tabB", -1, 1200.0)},
                            photon_yield_scale=0.94, photon_yield_variation_scale=1.0, speed_ratio={"EX": 1.1},
                            atten_ratio={"T1": 0.9, "EX1": 1.2})
    steps = _Steps(cols)
    rows = list(PH.iter_rows(steps, pdg, geom, cfg, tables, deviation, np.random.default_rng(1)))
    row_keys = ("s", "d", "t0", "t1", "nsub", "beta", "theta", "dev", "mu", "step", "chan")
    sums, hist, total = {}, np.zeros(96), 0
    for s in range(seeds):
        st, ch, tm = PH.make_photons(steps, pdg, geom, cfg, tables, deviation, np.random.default_rng(2000 + s))
        for a, b in zip(st, ch):
            sums[(a, b)] = sums.get((a, b), 0) + 1
        hist += np.bincount(np.clip((tm - cols["t0"][st]).astype(np.int64), 0, 95), minlength=96)
        total += len(st)
    pairs = np.array(sorted(sums), np.int64).reshape(-1, 2)
    out = {f"step_{k}": np.asarray(v) for k, v in cols.items()}
    out["pdg"] = pdg
    out["deviation"] = deviation
    for name, (e, t, g, refl) in tabs.items():
        out.update({f"{name}_edge_{k}": v for k, v in e.items()})
        for tk, T in t.items():
            out.update({f"{name}_{tk}_{f}": v for f, v in T.items()})
        out.update({f"{name}_geo_{k}": np.float64(v) for k, v in g.items()})
        out[f"{name}_reflector"] = np.int64(refl)
        out[f"{name}_propagation"] = np.array(PH.table_propagation(tables[name]))
    out.update(ck=ck, speed_ratio=PH.bar_ratios(cfg.speed_ratio, geom), atten_ratio=PH.bar_ratios(cfg.atten_ratio, geom),
               ref_pairs=pairs, ref_pair_mean=np.array([sums[tuple(p)] for p in pairs], float) / seeds,
               ref_delay_hist=hist / seeds, ref_total=np.int64(total), ref_seeds=np.int64(seeds))
    out["rows_groups"] = np.array([[L.name == "tabB", len(r["nsub"])] for L, r in rows], np.int64)
    for k in row_keys:
        out[f"rows_{k}"] = np.concatenate([np.asarray(r[k]) for _, r in rows])
    np.savez_compressed(HERE / "lookup_chain.npz", **out)


def make_pulsetests():
    import pytest
    records = []
    orig = PF.reconstruct

    def recorded(adc, n, start_tdc, pedestal_db, calib_area, calib_height, cfg=None, *a, **k):
        out = orig(adc, n, start_tdc, pedestal_db, calib_area, calib_height,
                   cfg if cfg is not None else PF.RecoConfig(), *a, **k)
        records.append(((adc, n, start_tdc, pedestal_db, calib_area, calib_height), out))
        return out

    set_period(12.5)                                # the tests are written for the stock period
    PF.reconstruct = recorded
    try:
        # the two waveform tests need the Mu2e single-PE template file (absent); the rest run
        rc = pytest.main(["-q", "-p", "no:cacheprovider", "-k", "not waveform_linear and not roundtrip",
                          str(REF / "tests" / "test_reco_pulsefit.py")])
    finally:
        PF.reconstruct = orig
        set_period(PERIOD)
    assert rc == 0, f"the reference's pulse-fit tests failed here ({rc})"
    out = {"n": np.int64(len(records)), "period": np.array([12.5])}
    for i, (args, r) in enumerate(records):
        tag = f"r{i}"
        for k, v in zip(("adc", "n", "start", "ped", "area", "height"), args):
            out[f"{tag}_{k}"] = np.asarray(v)
        for k, v in r.items():
            out[f"{tag}_out_{k}"] = np.asarray(v)
    np.savez_compressed(HERE / "pulsetests.npz", **out)


def make_chaintests():
    """The reference's chain-glue tests (crv/tests/test_chain.py: one TDC0 per (event, FEB), digi concatenation into
    reco waveforms) run under pytest with chain.reco_waveforms and chain.tdc0_per_feb recorded; then both on a
    multi-event sample (chain.py:219-231, 273-286)."""
    import pytest
    from crvfastsim import chain as CH
    rec_w, rec_t = [], []
    orig_w, orig_t = CH.reco_waveforms, CH.tdc0_per_feb

    def rw(D, cond):
        out = orig_w(D, cond)
        rec_w.append(({k: np.asarray(v).copy() for k, v in D.items()}, cond, out))
        return out

    def rt(labels, cond, rng, width=CH.PERIOD, key="roc_feb"):
        out = orig_t(labels, cond, rng, width, key)
        rec_t.append((np.asarray(labels).copy(), cond, width, key, out))
        return out

    CH.reco_waveforms, CH.tdc0_per_feb = rw, rt
    try:
        # the channel-label test needs JAX (skipped); the other two run
        rc = pytest.main(["-q", "-p", "no:cacheprovider", str(REF / "tests" / "test_chain.py")])
        rng = np.random.default_rng(61)
        nch = 512
        z = np.zeros(nch)
        cond = CH.Conditions(rng.uniform(90, 110, nch), rng.uniform(300, 500, nch), rng.uniform(20, 40, nch),
                             rng.uniform(-2, 2, nch), np.zeros(nch, np.int64), np.arange(nch) // 256,
                             (np.arange(nch) % 256) // 64, z)
        chan, st = [], []
        for ev in (1, 2, 7, (3 << 20) | 4):
            for c in rng.choice(nch, 40, replace=False):
                t = int(rng.integers(0, 50))
                for _ in range(int(rng.integers(1, 6))):
                    chan.append(ev * CH.CHAN_MULT + c)
                    st.append(t)
                    t += 12 if rng.random() < 0.6 else int(rng.integers(13, 40))   # continuation or a gap
        perm = rng.permutation(len(chan))
        D = {"chan": np.array(chan, np.int64)[perm], "starttdc": np.array(st, np.int64)[perm],
             "adc": rng.integers(80, 4000, (len(chan), 12))}
        CH.reco_waveforms(D, cond)
        for key in CH.FEB_PHASE_KEYS:
            CH.tdc0_per_feb(np.unique(D["chan"]), cond, np.random.default_rng(62), CH.PERIOD, key)
    finally:
        CH.reco_waveforms, CH.tdc0_per_feb = orig_w, orig_t
    assert rc == 0, f"the reference's chain tests failed here ({rc})"
    out = {"nw": np.int64(len(rec_w)), "nt": np.int64(len(rec_t))}
    cf = ("pedestal", "pulsearea", "pulseheight", "timeoffset", "roc", "feb")
    for i, (D, cond, W) in enumerate(rec_w):
        for k in ("chan", "starttdc", "adc"):
            out[f"w{i}_{k}"] = D[k]
        for k in cf:
            out[f"w{i}_cond_{k}"] = np.asarray(getattr(cond, k))
        for k, v in W.items():
            out[f"w{i}_out_{k}"] = np.asarray(v)
    for i, (labels, cond, width, key, t) in enumerate(rec_t):
        out[f"t{i}_labels"], out[f"t{i}_out"] = labels, np.asarray(t)
        out[f"t{i}_width"], out[f"t{i}_key"] = np.array([float(width)]), np.array(key)
        for k in ("roc", "feb"):
            out[f"t{i}_cond_{k}"] = np.asarray(getattr(cond, k))
    np.savez_compressed(HERE / "chaintests.npz", **out)


def encode(v):
    """Tagged JSON of a recorded argument: arrays keep dtype and shape, objects their readout attributes (a property
    that raises keeps its exception), mappings their items, NumPy scalars their type; decoded by tests/test_readout.py."""
    if isinstance(v, np.ndarray):
        return {"nd": v.dtype.str, "shape": list(v.shape), "data": v.ravel().tolist()}
    if isinstance(v, np.bool_):
        return {"npbool": bool(v)}
    if isinstance(v, np.integer):
        return {"npint": int(v)}
    if isinstance(v, float) and v != v:
        return {"nan": True}
    if v is None or isinstance(v, (bool, int, float, str)):
        return v
    if isinstance(v, (list, tuple)):
        return {"list" if isinstance(v, list) else "tuple": [encode(x) for x in v]}
    if isinstance(v, dict):
        return {"map": [[k, encode(x)] for k, x in v.items()]}
    attrs = ("sector_names", "sector", "nbars", "status", "readout_mask", "pedestal", "pulsearea", "pulseheight",
             "timeoffset", "roc", "feb", "deviation")
    out = {}
    for a in attrs:
        try:
            out[a] = encode(getattr(v, a))
        except AttributeError:
            continue
        except Exception as e:                                       # noqa: BLE001 (a property that raises)
            out[a] = {"raises": [type(e).__name__, str(e)]}
    return {"obj": out}


def make_readout():
    """The reference's readout-mask tests (crv/tests/test_readout_mask.py) run under pytest with readout.sensor_mask,
    readout.apply and readout.effective_status recorded (crv/crvfastsim/readout.py:9-72): arguments, and the output
    or the exception type and message of every call."""
    import json
    import pytest
    from crvfastsim import readout as RO
    calls = []
    orig = {n: getattr(RO, n) for n in ("sensor_mask", "apply", "effective_status")}

    def recorder(name):
        def f(*args):
            enc = [encode(a) for a in args]
            try:
                out = orig[name](*args)
            except Exception as e:                                   # noqa: BLE001 (recorded, then re-raised)
                calls.append({"fn": name, "args": enc, "error": [type(e).__name__, str(e)]})
                raise
            calls.append({"fn": name, "args": enc,
                          "out": encode(out if name != "apply" else out.readout_mask)})
            return out
        return f

    for n in orig:
        setattr(RO, n, recorder(n))
    try:
        # the CSV-loading and charge-boundary tests need pandas / JAX (absent here); the rest run
        rc = pytest.main(["-q", "-p", "no:cacheprovider", "-k", "not csv_loading and not charge_boundary",
                          str(REF / "tests" / "test_readout_mask.py")])
    finally:
        for n, f in orig.items():
            setattr(RO, n, f)
    assert rc == 0, f"the reference's readout tests failed here ({rc})"
    (HERE / "readout_calls.json").write_text(json.dumps(calls, allow_nan=False, separators=(",", ":")))


def make_wiring():
    """The reference's pulse-configuration wiring tests (crv/tests/test_chain_config_wiring.py, NumPy backend: default,
    custom and no-offset RecoConfig, 12- and 36-sample waveforms) and chain contracts (crv/tests/
    test_chain_reco_contract.py: status masking before the finder, explicit offsets, more than eight pulses in a
    waveform, no waveforms) run under pytest at the stock 12.5 ns with chain.clusters recorded: reco waveforms,
    conditions, the pulse configuration and the flat pulse table (chain.py:296-362)."""
    import dataclasses
    import json
    import pytest
    from crvfastsim import chain as CH
    rec = []
    orig = CH.clusters

    def recorded(W, cond, geom, counters_cfg, cfg, *a, **k):
        outs, timers = orig(W, cond, geom, counters_cfg, cfg, *a, **k)
        rcfg = cfg.pulse_reco if cfg.pulse_reco is not None else PF.RecoConfig()
        rec.append(({kk: np.asarray(v).copy() for kk, v in W.items()}, cond, dataclasses.asdict(rcfg),
                    {kk: np.asarray(v) for kk, v in outs[0]["pulses"].items()}))
        return outs, timers

    set_period(12.5)
    CH.clusters = recorded
    try:
        # NumPy-backend cases of both files (the JAX ones skip; the table-reco ones need the DQM tools, absent)
        rc = pytest.main(["-q", "-p", "no:cacheprovider", "-k",
                          "pulse_config or chain_conditions or cap_at_eight or empty_chain",
                          str(REF / "tests" / "test_chain_config_wiring.py"),
                          str(REF / "tests" / "test_chain_reco_contract.py")])
    finally:
        CH.clusters = orig
        set_period(PERIOD)
    assert rc == 0, f"the reference's wiring tests failed here ({rc})"
    out = {"n": np.int64(len(rec)), "period": np.array([12.5])}
    for i, (W, cond, rcfg, P) in enumerate(rec):
        for k, v in W.items():
            out[f"r{i}_W_{k}"] = v
        for k in ("status", "timeoffset"):
            out[f"r{i}_cond_{k}"] = np.asarray(getattr(cond, k))
        out[f"r{i}_reco"] = np.array(json.dumps(rcfg))
        for k, v in P.items():
            out[f"r{i}_P_{k}"] = v
    np.savez_compressed(HERE / "wiring.npz", **out)


def make_propagation():
    """The reference's light-propagation tests (crv/tests/test_propagation.py: the known-value table fit, bar keys and
    ratios) run under pytest with photons.table_propagation, bar_keys and bar_ratios recorded (photons.py:229-289): the
    table's decoded arrays and the fitted (inverse speed, attenuation length); the geometry and its per-bar sector and
    module keys; the ratio map and the per-bar ratios or the KeyError raised."""
    import json
    import pytest
    from crvfastsim.response import lookup as LK
    tp, br, bk = [], [], []
    o_tp, o_br, o_bk = PH.table_propagation, PH.bar_ratios, PH.bar_keys

    def rec_bk(geom):
        sk, mk = o_bk(geom)
        G = {k: np.asarray(getattr(geom, k)) for k in ("sector", "module")}
        G["nbars"], G["sector_names"] = np.int64(geom.nbars), np.array(list(geom.sector_names))
        bk.append((G, np.asarray(sk).astype(str), np.asarray(mk).astype(str)))
        return sk, mk

    def rec_tp(L):
        out = o_tp(L)
        tp.append((L.name, {k: np.asarray(v) for k, v in LK.arrays(L).items()}, out))
        return out

    def rec_br(values, geom):
        G = {k: np.asarray(getattr(geom, k)) for k in ("sector", "module")}
        G["nbars"], G["sector_names"] = np.int64(geom.nbars), np.array(list(geom.sector_names))
        try:
            out = o_br(values, geom)
        except KeyError as e:
            br.append((dict(values), G, None, str(e.args[0])))
            raise
        br.append((dict(values), G, np.asarray(out), None))
        return out

    PH.table_propagation, PH.bar_ratios, PH.bar_keys = rec_tp, rec_br, rec_bk
    try:
        rc = pytest.main(["-q", "-p", "no:cacheprovider", "-k", "recovers_known_values or bar_keys_and_ratios",
                          str(REF / "tests" / "test_propagation.py")])
    finally:
        PH.table_propagation, PH.bar_ratios, PH.bar_keys = o_tp, o_br, o_bk
    assert rc == 0, f"the reference's propagation tests failed here ({rc})"
    out = {"n_tp": np.int64(len(tp)), "n_br": np.int64(len(br)), "n_bk": np.int64(len(bk))}
    for i, (G, sk, mk) in enumerate(bk):
        for k, v in G.items():
            out[f"bk{i}_G_{k}"] = v
        out[f"bk{i}_sector_keys"], out[f"bk{i}_module_keys"] = sk, mk
    for i, (name, arrs, fit) in enumerate(tp):
        out[f"tp{i}_name"] = np.array(name)
        out[f"tp{i}_fit"] = np.array(fit)
        for k, v in arrs.items():
            out[f"tp{i}_{k}"] = v
    for i, (values, G, ratios, err) in enumerate(br):
        out[f"br{i}_values"] = np.array(json.dumps(values))
        for k, v in G.items():
            out[f"br{i}_G_{k}"] = v
        if ratios is not None:
            out[f"br{i}_out"] = ratios
        else:
            out[f"br{i}_error"] = np.array(err)
    np.savez_compressed(HERE / "propagation.npz", **out)


def make_pulsecache():
    """The reference's normal-equation-cache tests (crv/tests/test_pulsefit_normal_cache.py: an edge batch with a flat
    waveform, an 11-sample saturated prefix, a pedestal undershoot and a 12-of-36 valid length, and a synthetic batch;
    stock 12.5 ns) run under pytest with reconstruct_full recorded; identical calls (cache on and off) kept once."""
    import hashlib
    import pytest
    records, seen = [], set()
    orig = PF.reconstruct_full

    def recorded(adc, n, start_tdc, pedestal_db, calib_area, calib_height, cfg=None, *a, **k):
        out = orig(adc, n, start_tdc, pedestal_db, calib_area, calib_height,
                   cfg if cfg is not None else PF.RecoConfig(), *a, **k)
        args = tuple(np.asarray(x).copy() for x in (adc, n, start_tdc, pedestal_db, calib_area, calib_height))
        h = hashlib.sha256(b"".join(x.tobytes() for x in args)).hexdigest()
        if h not in seen and cfg is None:
            seen.add(h)
            records.append((args, out))
        return out

    set_period(12.5)
    PF.reconstruct_full = recorded
    try:
        rc = pytest.main(["-q", "-p", "no:cacheprovider", str(REF / "tests" / "test_pulsefit_normal_cache.py")])
    finally:
        PF.reconstruct_full = orig
        set_period(PERIOD)
    assert rc == 0, f"the reference's normal-cache tests failed here ({rc})"
    out = {"n": np.int64(len(records)), "period": np.array([12.5])}
    for i, (args, r) in enumerate(records):
        for k, v in zip(("adc", "n", "start", "ped", "area", "height"), args):
            out[f"r{i}_{k}"] = v
        for k, v in r.items():
            out[f"r{i}_out_{k}"] = np.asarray(v)
    np.savez_compressed(HERE / "pulsecache.npz", **out)


def make_attach():
    import json
    import pytest
    records = []
    orig = C.find_event

    def recorded(p, G, status, cfg=None, vectorized=False):
        out = orig(p, G, status, cfg if cfg is not None else C.FinderConfig(), vectorized=vectorized)
        if not vectorized:
            records.append(({k: np.asarray(v).copy() for k, v in p.items()}, G, np.asarray(status).copy(),
                            cfg if cfg is not None else C.FinderConfig(), out))
        return out

    C.find_event = recorded
    try:
        # the config-schema test needs the reference's core library (not part of the finder); the rest run
        rc = pytest.main(["-q", "-p", "no:cacheprovider", "-k", "not test_config_schema",
                          str(REF / "tests" / "test_coinc_attachment_cpu.py")])
    finally:
        C.find_event = orig
    assert rc == 0, f"the reference's attachment tests failed here ({rc})"
    out = {"n": np.int64(len(records))}
    for i, (p, G, status, cfg, rows) in enumerate(records):
        tag = f"a{i}"
        n = len(p["idx"])
        P = {"ev": np.zeros(n, np.int64), **{k: np.asarray(p[k]) for k in ("idx", "bar", "sipm", "time", "pe", "seq")}}
        fl = flatten_clusters([(0, rows)])
        for k, v in fl.items():
            out[f"{tag}_scalar_{k}"] = v
        for k in ("ev", "idx", "bar", "sipm", "time", "pe", "seq"):
            out[f"{tag}_in_{k}"] = P[k]
        out[f"{tag}_status"] = status
        for k in ("sector", "layer", "counter_in_type", "x", "y", "pos", "length_dir", "sector_type", "pos_side0",
                  "pos_side1", "sipms_side0", "sipms_side1"):
            out[f"{tag}_G_{k}"] = np.asarray(getattr(G, k))
        out[f"{tag}_G_sector_names"] = np.array(G.sector_names)
        names = [n_ for n_ in G.sector_names if n_ in cfg.cuts]
        out[f"{tag}_cut_names"] = np.array(names)
        out[f"{tag}_cuts"] = cuts_array(cfg, names)
        flags = {k: getattr(cfg, k) for k in ("fiber_signal_speed", "max_time_interval", "time_offset",
                                             "compensate_status_bits", "ignore_secondary_pulses",
                                             "big_cluster_threshold", "add_opposite_side_pulses")}
        flags["compensate_status_bits"] = list(flags["compensate_status_bits"])
        out[f"{tag}_flags"] = np.array(json.dumps(flags))
    np.savez_compressed(HERE / "attach.npz", **out)


if __name__ == "__main__":
    for name, fn in (("pulsefit", make_pulsefit), ("concat", make_concat), ("waveform", make_waveform),
                     ("waveform_gate", make_waveform_gate),
                     ("coinc", make_coinc), ("stats", make_stats), ("pixelid", make_pixelid), ("lookup", make_lookup), ("lookup_file", make_lookup_file), ("lookup_fuzz", make_lookup_fuzz),
                     ("lookup_chain", make_lookup_chain), ("attach", make_attach), ("chaintests", make_chaintests), ("readout", make_readout), ("wiring", make_wiring), ("propagation", make_propagation), ("pulsecache", make_pulsecache), ("pulsetests", make_pulsetests)):
        if not ONLY or name in ONLY:
            fn()
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)
