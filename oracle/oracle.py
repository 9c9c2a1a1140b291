"""CPU oracle of the CRV response chain: TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module, and only as the checker.
It restates the reference algorithm stage by stage:

  * stochastic stages (photons, SiPM, TDC0, electronics noise): the C library built from oracle/crv_oracle.c, with
    the keyed Philox draws the engine uses (crv/crvfastsim/response/photons.py:102-112, :305-356;
    crv/crvfastsim/response/sipm.py:80-198; crv/crvfastsim/chain.py:219-231);
  * waveform synthesis and zero suppression (crv/crvfastsim/reco/waveform.py:65-172), vectorised NumPy;
  * digi grouping into reco waveforms (crv/crvfastsim/reco/pulsefit.py:319-345, crv/crvfastsim/chain.py:273-286);
  * pulse reconstruction with the bounded Levenberg-Marquardt Gumbel fit (pulsefit.py:49-316), vectorised NumPy;
  * the coincidence finder (crv/crvfastsim/reco/coinc.py:112-392, crv/crvfastsim/reco/coinc_cpu.py:11-51);
  * the chain glue (crv/crvfastsim/chain.py:151-362);
  * the lookup-table photon model: row preparation and substeps in the C library with keyed draws
    (crv/crvfastsim/response/photons.py:163-224, :292-356), its host setup here (table propagation fits and per-bar
    ratios, photons.py:230-289) and make_photons over the (table, reflector) groups (photons.py:305-371).

The deterministic NumPy stages are pinned bit for bit against fixtures generated from the reference itself
(tests/golden/make_golden.py); the stochastic stages, the lookup-table model included, against the reference's
known-answer tests and statistics of its own outputs.
Configuration objects are duck-typed: any object with the reference's field names works.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from itertools import combinations

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
CHAN_MULT = 32768
NPX = 1600                      # photon-map bins (x * 40 + y)
NPS = 41 * 41                   # SiPM pixel ids x * 41 + y (sipm.py:22 NPIX = 41)


def build(force=False):
    """Compile the C part of the oracle (gcc, no contraction)."""
    src = os.path.join(HERE, "crv_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".{os.getpid()}.tmp"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-o", tmp, src,
                           "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.orc_exp.restype = ctypes.c_double
        _lib.orc_exp.argtypes = [ctypes.c_double]
        _lib.orc_log.restype = ctypes.c_double
        _lib.orc_log.argtypes = [ctypes.c_double]
        _lib.orc_sipm_groups.restype = ctypes.c_int
    return _lib


def _p(a):
    """Pointer of an array the caller keeps alive."""
    return ctypes.c_void_p(a.ctypes.data)


class _Keep:
    """Pointer factory that keeps every converted array alive until the holder is dropped (a pointer taken from a
    temporary array would dangle as soon as the temporary is freed)."""

    def __init__(self):
        self.arrays = []

    def __call__(self, a, dtype=None):
        a = np.ascontiguousarray(a, dtype)
        self.arrays.append(a)
        return ctypes.c_void_p(a.ctypes.data)


class OrcParams(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint32), ("pad0", ctypes.c_uint32),
                ("yield_per_mev", ctypes.c_double), ("frac_short", ctypes.c_double), ("frac_long", ctypes.c_double),
                ("lambda_short", ctypes.c_double), ("lambda_long", ctypes.c_double),
                ("signal_speed", ctypes.c_double), ("decay_time", ctypes.c_double),
                ("overvoltage", ctypes.c_double), ("time_constant", ctypes.c_double),
                ("capacitance", ctypes.c_double), ("p1", ctypes.c_double), ("p2", ctypes.c_double),
                ("q_ct", ctypes.c_double), ("q_t0", ctypes.c_double), ("q_t1", ctypes.c_double),
                ("trap0_lifetime", ctypes.c_double), ("trap1_lifetime", ctypes.c_double), ("t_end", ctypes.c_double),
                ("n_pixels_x", ctypes.c_int32), ("n_pixels_y", ctypes.c_int32),
                ("pixel_lrint", ctypes.c_int32), ("pad1", ctypes.c_int32)]


def p_fire(sc, v):
    """Host-side p_fire for derived constants (NumPy exp, as the reference's SiPMConfig.p_fire)."""
    return sc.p1 * (1.0 - np.exp(-v / sc.p2))


def params(rc, sc, seed, t_end):
    """OrcParams from a response config (analytic model) and a SiPM config (reference field names)."""
    P = OrcParams()
    P.seed = int(seed) & 0xFFFFFFFF
    P.yield_per_mev = rc.yield_per_mev
    P.frac_short = rc.frac_short
    P.frac_long = 1.0 - rc.frac_short
    P.lambda_short = rc.lambda_short
    P.lambda_long = rc.lambda_long
    P.signal_speed = rc.signal_speed
    P.decay_time = rc.decay_time
    P.overvoltage, P.time_constant, P.capacitance = sc.overvoltage, sc.time_constant, sc.capacitance
    P.p1, P.p2 = sc.p1, sc.p2
    pf = float(p_fire(sc, sc.overvoltage))
    P.q_ct = (1.0 - (1.0 - sc.cross_talk) ** 0.25) / pf
    P.q_t0 = sc.trap0_prob / pf
    P.q_t1 = sc.trap1_prob / pf
    P.trap0_lifetime, P.trap1_lifetime = sc.trap0_lifetime, sc.trap1_lifetime
    P.t_end = float(t_end)
    P.n_pixels_x, P.n_pixels_y = sc.n_pixels_x, sc.n_pixels_y
    P.pixel_lrint = 1 if getattr(sc, "pixel_id", "truncate") == "lrint" else 0
    return P


def photon_map_cdf(pmap=None):
    """Running sums of the photon map over bins x * 40 + y (uniform map if None), and the dead-pixel table."""
    pm = np.ones((40, 40)) if pmap is None else np.asarray(pmap, float)
    return np.cumsum(pm.ravel())


def dead_table(sc):
    """Dead pixels over the pixel ids x * 41 + y of the 41 x 41 state (sipm.py:125-127, NPIX = 41 at sipm.py:22)."""
    d = np.zeros(NPS, np.uint8)
    for x, y in sc.inactive:
        d[x * 41 + y] = 1
    return d


# ---------------------------------------------------------------------------------------------------------------------
# keyed helpers

def tdc0_uniform(seed, run, event, subrun, febkey):
    n = len(event)
    u = np.empty(n)
    k = _Keep()
    lib().orc_tdc0_uniform(ctypes.c_uint32(seed), ctypes.c_int64(n), *[k(x, np.uint32) for x in (run, event, subrun,
                                                                                             febkey)], k(u))
    return u


def noise_normal(seed, run, event, subrun, chan, tick):
    n = len(event)
    z = np.empty(n)
    k = _Keep()
    lib().orc_noise_normal(ctypes.c_uint32(seed), ctypes.c_int64(n), *[k(x, np.uint32) for x in (run, event, subrun)],
                           k(chan, np.int32), k(tick, np.int64), k(z))
    return z


# ---------------------------------------------------------------------------------------------------------------------
# steps -> photons -> charges

def step_frame(steps, geom):
    """Per step: bar, length coordinate relative to the bar centre, time, edep, half length (step midpoints)."""
    bar = np.asarray(steps["bar"], np.int64)
    ax = np.asarray(geom.local_to_world)[bar, 2]
    pos = np.stack([0.5 * (np.asarray(steps[f"{a}0"], float) + np.asarray(steps[f"{a}1"], float)) for a in "xyz"], 1)
    c = np.asarray(geom.center, float)[bar]
    r = np.arange(len(bar))
    z = pos[r, ax] - c[r, ax]
    half = np.asarray(geom.halflen, float)[bar, ax]
    t = 0.5 * (np.asarray(steps["t0"], float) + np.asarray(steps["t1"], float))
    return bar, z, t, np.asarray(steps["edep"], float), half


def event_ids(steps):
    """(run, subrun, event, step index inside its event); steps of one event must be contiguous."""
    n = len(np.asarray(steps["event"]))
    run = np.asarray(steps["run"], np.int64) if "run" in steps else np.zeros(n, np.int64)
    sub = np.asarray(steps["subrun"], np.int64)
    ev = np.asarray(steps["event"], np.int64)
    new = np.ones(n, bool)
    if n > 1:
        new[1:] = (run[1:] != run[:-1]) | (sub[1:] != sub[:-1]) | (ev[1:] != ev[:-1])
    first = np.flatnonzero(new)
    gid = np.cumsum(new) - 1
    sie = np.arange(n) - first[gid]
    return run, sub, ev, sie


def yield_factor(deviation, rc):
    return (np.asarray(deviation, float) * rc.photon_yield_variation_scale + 1.0) * rc.photon_yield_scale


def photon_counts(steps, geom, rc, deviation, seed):
    """[nsteps, 4] photon counts per (step, SiPM)."""
    bar, z, t, edep, half = step_frame(steps, geom)
    run, sub, ev, sie = event_ids(steps)
    dev = np.ascontiguousarray(yield_factor(deviation, rc))
    n = len(bar)
    cnt = np.zeros(4 * n, np.int64)
    P = params(rc, _NullSiPM, seed, 1e5)
    k = _Keep()
    lib().orc_photon_counts(ctypes.byref(P), ctypes.c_int64(n), k(bar, np.int32), k(z, np.float64), k(t, np.float64),
                            k(edep, np.float64), k(half, np.float64), k(dev, np.float64), k(ev, np.uint32),
                            k(sub, np.uint32), k(run, np.uint32), k(sie, np.int32), k(cnt))
    return cnt.reshape(n, 4)


class _NullSiPM:
    overvoltage, time_constant, capacitance, p1, p2 = 3.0, 13.3, 8.84e-14, 0.607, 2.7
    cross_talk, trap0_prob, trap1_prob, trap0_lifetime, trap1_lifetime = 0.0, 0.0, 0.0, 5.0, 50.0
    n_pixels_x = n_pixels_y = 40


def make_photons(steps, geom, rc, deviation, seed):
    """Photons at the SiPMs, in the reference's block order (SiPM 0..3, then step, then photon):
    (step row, channel, time, key = step-in-event << 16 | photon)."""
    cnt = photon_counts(steps, geom, rc, deviation, seed)
    bar, z, t, edep, half = step_frame(steps, geom)
    run, sub, ev, sie = event_ids(steps)
    n = len(bar)
    rows_step = np.tile(np.arange(n), 4)
    rows_s = np.repeat(np.arange(4), n)
    rc_ = cnt[rows_step, rows_s]
    off = np.r_[0, np.cumsum(rc_)[:-1]].astype(np.int64)
    tot = int(rc_.sum())
    o = [np.empty(tot, np.int64), np.empty(tot, np.int64), np.empty(tot), np.empty(tot, np.int64)]
    P = params(rc, _NullSiPM, seed, 1e5)
    k = _Keep()
    lib().orc_photon_emit(ctypes.byref(P), ctypes.c_int64(4 * n), k(rows_step, np.int64), k(rows_s, np.int32),
                          k(rc_, np.int64), k(off, np.int64), k(bar, np.int32), k(z, np.float64), k(t, np.float64),
                          k(half, np.float64), k(ev, np.uint32), k(sub, np.uint32), k(run, np.uint32),
                          k(sie, np.int32), *[k(x) for x in o])
    return o[0], o[1], o[2], o[3]


def sipm_pixels(keys, sc, seed, pmap=None, chan=0, event=1, subrun=0, run=0):
    """Pixel ids (x * 41 + y; -1 dead) that the SiPM stage draws for photons with these draw keys on one SiPM."""
    P = params(_NullResponse, sc, seed, 0.0)
    keys = np.ascontiguousarray(np.asarray(keys, np.int64))
    out = np.empty(len(keys), np.int32)
    k = _Keep()
    lib().orc_sipm_pixels(ctypes.byref(P), k(np.ascontiguousarray(photon_map_cdf(pmap))), k(dead_table(sc)),
                          ctypes.c_uint32(run), ctypes.c_uint32(event), ctypes.c_uint32(subrun), ctypes.c_int(chan),
                          k(keys, np.int64), ctypes.c_int64(len(keys)), out.ctypes.data_as(ctypes.c_void_p))
    return out


def sipm_groups(label, time, photon, key, run_of_label, sc, seed, t_end, pmap=None):
    """SiPM stage for photons given per photon: SiPM label (event key * CHAN_MULT + channel), time, photon id and draw
    key; run_of_label(labels) -> run numbers.  Returns (charge dict sorted by (label, time), per-SiPM labels,
    per-SiPM charge counts, per-SiPM fired-pixel counts, status)."""
    label = np.asarray(label, np.int64)
    o = np.argsort(label, kind="stable")
    lab_s = label[o]
    u, start, cnt = np.unique(lab_s, return_index=True, return_counts=True)
    evkey, chan = u // CHAN_MULT, u % CHAN_MULT
    sub, ev = evkey >> 20, evkey & ((1 << 20) - 1)
    run = np.asarray(run_of_label(u), np.int64)
    P = params(_NullResponse, sc, seed, t_end)
    cum = np.ascontiguousarray(photon_map_cdf(pmap))
    dead = dead_table(sc)
    G = len(u)
    nq = np.zeros(G, np.int64)
    nfp = np.zeros(G, np.int64)
    nout = ctypes.c_int64(0)
    pt, pv, pp = ctypes.POINTER(ctypes.c_double)(), ctypes.POINTER(ctypes.c_double)(), ctypes.POINTER(ctypes.c_int64)()
    tm = np.ascontiguousarray(np.asarray(time, float)[o])
    ky = np.ascontiguousarray(np.asarray(key, np.int64)[o])
    ph = np.ascontiguousarray(np.asarray(photon, np.int64)[o])
    k = _Keep()
    st = lib().orc_sipm_groups(ctypes.byref(P), k(cum), k(dead), ctypes.c_int64(G), k(start, np.int64),
                               k(cnt, np.int64), k(chan, np.int32), k(ev, np.uint32), k(sub, np.uint32),
                               k(run, np.uint32), k(tm), k(ky), k(ph), k(nq), k(nfp), ctypes.byref(nout),
                               ctypes.byref(pt), ctypes.byref(pv), ctypes.byref(pp))
    n = nout.value
    if n:
        t = np.ctypeslib.as_array(pt, (n,)).copy()
        v = np.ctypeslib.as_array(pv, (n,)).copy()
        phot = np.ctypeslib.as_array(pp, (n,)).copy()
    else:
        t, v, phot = np.zeros(0), np.zeros(0), np.zeros(0, np.int64)
    for q in (pt, pv, pp):
        lib().orc_free(q)
    Q = {"chan": np.repeat(u, nq), "time": t, "charge": sc.capacitance * v, "pe": v / sc.overvoltage,
         "photon": phot}
    return Q, u, nq, nfp, st


class _NullResponse:
    yield_per_mev, frac_short, lambda_short, lambda_long, signal_speed, decay_time = 0.0, 0.3, 1e3, 5e3, 140.0, 0.0


def effective_status(cond):
    st = np.asarray(cond.status)
    mask = getattr(cond, "readout_mask", None)
    if mask is None:
        return st
    st = st.copy()
    st[~np.asarray(mask, bool)] |= 1
    return st


def charges(steps, geom, cond, rc, sc, seed, t_end, pmap=None):
    """chain.charges (crv/crvfastsim/chain.py:151-213) with the analytic photon model and keyed draws.
    Returns (Q, diagnostics) with Q sorted by (label, time)."""
    s, c, t, key = make_photons(steps, geom, rc, cond.deviation, seed)
    status = effective_status(cond)
    keep = (status[c] & 0b101) == 0
    s, c, t, key = s[keep], c[keep], t[keep], key[keep]
    run, sub, ev, _ = event_ids(steps)
    evkey = (sub << 20) | ev
    label = evkey[s] * CHAN_MULT + c
    run_tab = dict(zip(evkey.tolist(), run.tolist()))
    Q, u, nq, nfp, st = sipm_groups(label, t, s, key, lambda L: [run_tab[int(x)] for x in L // CHAN_MULT], sc, seed,
                                    t_end, pmap)
    return Q, dict(photons=len(s), sipm_labels=u, sipm_charges=nq, sipm_fired_pixels=nfp, status=st,
                   photon_label=label)


# ---------------------------------------------------------------------------------------------------------------------
# TDC0 and waveform synthesis

def feb_key(ch, cond, key="roc_feb"):
    return cond.feb[ch] if key == "feb" else cond.roc[ch] * 1000 + cond.feb[ch]


def tdc0_of_labels(labels, cond, seed, width, key, run_of_evkey):
    """One keyed uniform x width per (event, FEB) (crv/crvfastsim/chain.py:219-231)."""
    labels = np.asarray(labels, np.int64)
    evk, ch = labels // CHAN_MULT, labels % CHAN_MULT
    fk = feb_key(ch, cond, key)
    run = np.asarray(run_of_evkey(evk), np.int64)
    return tdc0_uniform(seed, run, evk & ((1 << 20) - 1), evk >> 20, fk) * width


def gumbel_template_raw(peak, mu, beta, precision=0.5, max_time=100.0):
    t = np.arange(0.0, max_time + precision / 2, precision)
    v = peak * np.e * np.exp(-(t - mu) / beta - np.exp(-(t - mu) / beta))
    return t, v


def resample_template(t_raw, v_raw, precision, stretch, max_time):
    """The single-PE template resampled to `precision` ns (crv/crvfastsim/reco/waveform.py:46-62)."""
    t = np.asarray(t_raw, float) * stretch
    v = np.asarray(v_raw, float)
    out = [v[0]]
    k = 1
    for i in range(1, len(t)):
        while t[i] >= k * precision and k * precision < max_time:
            frac = (k * precision - t[i - 1]) / (t[i] - t[i - 1])
            out.append((v[i] - v[i - 1]) * frac + v[i - 1])
            k += 1
        if k * precision >= max_time:
            break
    return np.asarray(out)


def cluster_ids(chan, time, gap):
    new = np.ones(len(time), bool)
    if len(time) > 1:
        new[1:] = (chan[1:] != chan[:-1]) | (time[1:] - time[:-1] > gap)
    return np.cumsum(new) - 1


def synthesize(chan, time, charge, tdc0_of_chan, tmpl, cfg, period, window, noise=None):
    """Zero-suppressed digis of one batch (crv/crvfastsim/reco/waveform.py:96-172).

    noise: None, or callable(cluster labels, cluster first ticks, (C, L)) -> standard normals [C, L]; the waveform
    gets 0 + cfg.noise * z on its valid samples."""
    chan = np.asarray(chan)
    time = np.asarray(time, float)
    charge = np.asarray(charge, float)
    tmpl = np.asarray(tmpl, float)
    zs = cfg.samples_zs
    vmax = tmpl.max()
    cid = cluster_ids(chan, time, cfg.single_pe_max_time + 4 * period)
    C = int(cid[-1]) + 1 if len(cid) else 0
    if C == 0:
        e = np.zeros(0)
        return {"chan": np.zeros(0, np.int64), "start": e, "tdc0": e, "starttdc": np.zeros(0, np.int64),
                "volt": np.zeros((0, zs)), "adc": np.zeros((0, zs), np.int16), "cluster_chan": np.zeros(0, np.int64),
                "cluster_tstart": e, "cluster_keep": np.zeros(0, bool)}
    head = np.flatnonzero(np.r_[True, cid[1:] != cid[:-1]])
    tail = np.r_[head[1:] - 1, len(cid) - 1]
    keep = np.bincount(cid, minlength=C) * vmax >= cfg.min_voltage
    cchan = chan[head]
    tdc0 = tdc0_of_chan(cchan) if callable(tdc0_of_chan) else np.asarray(tdc0_of_chan)[cchan]
    tick0 = np.ceil((time[head] - period - tdc0) / period)
    t_start = tick0 * period + tdc0
    est = np.floor((time[tail] - time[head] + cfg.single_pe_max_time) / period).astype(np.int64)
    reach = int(np.ceil(cfg.single_pe_max_time / period)) + 2
    ts_q = t_start[cid]
    j = np.maximum(np.ceil((time - ts_q) / period), 0).astype(np.int64)[:, None] + np.arange(reach)[None, :]
    dt = j * period + ts_q[:, None] - time[:, None]
    ti = np.rint(dt / cfg.single_pe_precision).astype(np.int64)
    hit = (dt >= 0) & (ti < len(tmpl)) & keep[cid][:, None]
    rows = np.broadcast_to(cid[:, None], j.shape)[hit]
    cols = j[hit]
    need = np.zeros(C, np.int64)
    np.maximum.at(need, rows, cols + 1)
    length = np.maximum(est, need)
    L = int(length.max()) + zs
    wave = np.zeros((C, L))
    contrib = tmpl[np.clip(ti, 0, len(tmpl) - 1)] * (charge / cfg.single_pe_reference_charge)[:, None]
    np.add.at(wave, (rows, cols), contrib[hit])
    valid = np.arange(L)[None, :] < length[:, None]
    if noise is not None:
        wave += (0.0 + cfg.noise * noise(cchan, tick0.astype(np.int64), (C, L))) * valid
    over = (wave > cfg.min_voltage) & valid
    win = over.copy()
    for d in (1, 2):
        win[:, :-d] |= over[:, d:]
        win[:, d:] |= over[:, :-d]
    win &= valid & keep[:, None]
    nxt = np.zeros(C, np.int64)
    dr, di = [], []
    for i in range(L):
        cand = win[:, i] & (nxt <= i)
        if not cand.any():
            continue
        ts = t_start + i * period
        r = np.flatnonzero(cand & (ts >= window[0]) & (ts <= window[1]))
        dr.append(r)
        di.append(np.full(len(r), i))
        nxt[r] = i + zs
    r = np.concatenate(dr) if dr else np.zeros(0, np.int64)
    i0 = np.concatenate(di) if di else np.zeros(0, np.int64)
    cols = i0[:, None] + np.arange(zs)[None, :]
    volt = np.where(cols < length[r, None], wave[r[:, None], np.minimum(cols, L - 1)], 0.0)
    start = t_start[r] + i0 * period
    adc = np.clip(adc_int16(volt * cfg.adc_conversion + cfg.pedestal + 0.5), cfg.min_adc, cfg.max_adc)
    o = np.lexsort((start, cchan[r]))
    return {"chan": cchan[r][o], "start": start[o], "tdc0": tdc0[r][o],
            "starttdc": np.rint((start - tdc0[r]) / period).astype(np.int64)[o], "volt": volt[o], "adc": adc[o],
            "cluster_chan": cchan, "cluster_tstart": t_start, "cluster_keep": keep}


def adc_int16(x):
    """float -> int16 as the reference's astype(np.int16): truncation to int32, then the low 16 bits."""
    x = np.asarray(x, float)
    i32 = np.trunc(np.clip(x, -2147483648.0, 2147483647.0)).astype(np.int64)
    return ((i32 + 32768) % 65536 - 32768).astype(np.int16)


def keyed_noise(seed, run_of_evkey):
    """Noise hook for synthesize: standard normals keyed by (event, channel, tick)."""
    def f(labels, tick0, shape):
        C, L = shape
        lab = np.repeat(np.asarray(labels, np.int64), L)
        tk = (np.asarray(tick0, np.int64)[:, None] + np.arange(L)[None, :]).ravel()
        evk, ch = lab // CHAN_MULT, lab % CHAN_MULT
        run = np.asarray(run_of_evkey(evk), np.int64)
        return noise_normal(seed, run, evk & ((1 << 20) - 1), evk >> 20, ch, tk).reshape(C, L)
    return f


# ---------------------------------------------------------------------------------------------------------------------
# reco waveforms

def concat_waveforms(key, bar, sipm, start_tdc, adc_flat, lens):
    """Consecutive digis of one channel whose TDCs continue form one waveform (pulsefit.py:319-345)."""
    nd = len(bar)
    lens = np.asarray(lens, np.int64)
    cont = np.zeros(nd, bool)
    if nd > 1:
        cont[1:] = ((key[1:] == key[:-1]) & (bar[1:] == bar[:-1]) & (sipm[1:] == sipm[:-1])
                    & (start_tdc[1:] == start_tdc[:-1] + lens[:-1]))
    gid = np.cumsum(~cont) - 1
    G = int(gid[-1]) + 1 if nd else 0
    glen = np.bincount(gid, weights=lens, minlength=G).astype(np.int64)
    L = int(glen.max()) if G else 0
    first = np.flatnonzero(~cont)
    begin = np.cumsum(lens) - lens
    off = begin - begin[first][gid] if nd else np.zeros(0, np.int64)
    mat = np.zeros((G, L), np.int64)
    tot = int(lens.sum())
    inner = np.arange(tot) - np.repeat(begin, lens)
    mat[np.repeat(gid, lens), np.repeat(off, lens) + inner] = np.asarray(adc_flat, np.int64)
    return gid, mat, glen, start_tdc[first], first


def reco_waveforms(D, cond):
    """Digis -> reco waveforms with calibration (crv/crvfastsim/chain.py:273-286)."""
    ev, ch = D["chan"] // CHAN_MULT, D["chan"] % CHAN_MULT
    o = np.lexsort((D["starttdc"], ch, ev))
    ev, ch, st = ev[o], ch[o], D["starttdc"][o]
    adc = np.asarray(D["adc"])[o]
    lens = np.full(len(o), adc.shape[1], np.int64)
    gid, mat, n, start, first = concat_waveforms(ev, ch // 4, ch % 4, st, adc.ravel(), lens)
    c0 = ch[first]
    return {"ev": ev[first], "bar": c0 // 4, "sipm": c0 % 4, "chan": c0, "adc": mat, "n": n, "start": start,
            "ped": cond.pedestal[c0], "area": cond.pulsearea[c0], "height": cond.pulseheight[c0],
            "toff": cond.timeoffset[c0]}


# ---------------------------------------------------------------------------------------------------------------------
# pulse reconstruction

def _round_half_away(x):
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def _gumbel(t, A, mu, b):
    z = (t - mu) / b
    return A * np.exp(-z - np.exp(-z))


def _near_threshold(y, valid, thr, edge):
    lo = np.full((y.shape[0], 1), -1e9)
    yv = np.where(valid, y, -1e9)
    prev = np.concatenate([lo, yv[:, :-1]], 1)
    nxt = np.concatenate([yv[:, 1:], lo], 1)
    return (valid & (yv >= prev) & (yv > nxt) & (np.abs(yv - thr) <= edge)).any(1)


def find_next_peak(y, n, start, active, cfg):
    """FindNextPeak for every row (pulsefit.py:71-119)."""
    W, L = y.shape
    rows = np.arange(W)
    found = np.zeros(W, bool)
    rising = np.zeros(W, bool)
    stop = ~active
    ps = np.zeros(W, np.int64)
    pe = np.zeros(W, np.int64)
    for b in range(1, L):
        live = ~stop & (b > start) & (b < n)
        if not live.any():
            continue
        a, c = y[:, b - 1], y[:, b]
        up = live & (a < c)
        rising |= up
        ps[up] = b
        pe[up] = b
        pe[live & (a == c) & rising] = b
        down = live & (a > c) & rising
        got = down & (y[rows, pe] > cfg.min_adc_difference)
        found |= got
        stop |= got
        rising &= ~(down & ~got)
    fs, fe = ps - 1, pe + 1
    go = found.copy()
    for k in range(1, cfg.samples_before + 1):
        i = ps - k
        ii = np.clip(i, 0, L - 2)
        ok = go & (i >= 0) & (i >= ps - cfg.samples_before) & (y[rows, ii] <= y[rows, ii + 1])
        fs[ok] = i[ok]
        go = ok & (i != 0)
    go = found.copy()
    for k in range(1, cfg.samples_after + 1):
        i = pe + k
        ii = np.clip(i, 1, L - 1)
        ok = go & (i < n) & (y[rows, ii - 1] >= y[rows, ii])
        fe[ok] = i[ok]
        go = ok
    fs = np.where(found & (ps - fs > 1), fs + 1, fs)
    fe = np.where(found & (fe - pe > 1), fe - 1, fe)
    return found, ps, pe, fs, fe


def _to_ext(u, lo, hi):
    return lo + (hi - lo) * (np.sin(u) + 1.0) * 0.5


def _to_int(p, lo, hi):
    return np.arcsin(np.clip(2.0 * (p - lo) / (hi - lo) - 1.0, -1.0, 1.0))


def fit_gumbel(t, y, mask, p0, lo, hi, iterations=40):
    """Bounded Gumbel least squares, Levenberg-Marquardt in sine-mapped coordinates (pulsefit.py:125-216)."""
    K = t.shape[0]
    w = mask.astype(float)
    half = (hi - lo) * 0.5

    def model(u):
        p = _to_ext(u, lo, hi)
        A, mu, b = p[:, 0:1], p[:, 1:2], p[:, 2:3]
        z = (t - mu) / b
        ez = np.exp(-z)
        g = np.exp(-z - ez)
        f = A * g
        r = (y - f) * w
        fz = f * (ez - 1.0)
        d = half * np.cos(u)
        J = np.stack([g * d[:, 0:1], fz * (-1.0 / b) * d[:, 1:2], fz * (-z / b) * d[:, 2:3]], axis=-1) * w[..., None]
        return r, J

    u = _to_int(p0, lo, hi)
    r, J = model(u)
    chi2 = (r * r).sum(1)
    lam = np.full(K, 1e-3)
    eye = np.eye(3)

    def accept(u, r, J, chi2, un):
        rn, Jn = model(un)
        c2 = (rn * rn).sum(1)
        ok = c2 < chi2
        return (np.where(ok[:, None], un, u), np.where(ok[:, None], rn, r), np.where(ok[:, None, None], Jn, J),
                np.where(ok, c2, chi2), ok)

    for _ in range(iterations):
        H = np.einsum("kpi,kpj->kij", J, J)
        g = np.einsum("kpi,kp->ki", J, r)
        dg = np.einsum("kii->ki", H)
        try:
            du = np.linalg.solve(H + lam[:, None, None] * (dg[:, :, None] * eye + 1e-12 * eye), g[..., None])[..., 0]
        except np.linalg.LinAlgError:
            du = np.zeros_like(u)
        u, r, J, chi2, ok = accept(u, r, J, chi2, u + du)
        lam = np.clip(np.where(ok, lam * 0.3, lam * 10.0), 1e-9, 1e9)
    for _ in range(8):
        H = np.einsum("kpi,kpj->kij", J, J)
        g = np.einsum("kpi,kp->ki", J, r)
        try:
            du = np.linalg.solve(H + 1e-12 * eye, g[..., None])[..., 0]
        except np.linalg.LinAlgError:
            break
        du = np.where(np.isfinite(du), du, 0.0)
        for s in (1.0, 0.5, 0.25, 0.125):
            u, r, J, chi2, ok = accept(u, r, J, chi2, u + s * du)
            du = np.where(ok[:, None], 0.0, du)
    H = np.einsum("kpi,kpj->kij", J, J)
    g = np.einsum("kpi,kp->ki", J, r)
    try:
        step = np.linalg.solve(H + 1e-12 * eye, g[..., None])[..., 0]
        edm = 0.5 * np.einsum("ki,ki->k", g, step)
        ev = np.linalg.eigvalsh(H)
        hess_ok = ev[:, 0] > 1e-12 * np.maximum(ev[:, -1], 1e-300)
    except np.linalg.LinAlgError:
        edm = np.full(K, np.inf)
        hess_ok = np.zeros(K, bool)
    converged = np.isfinite(edm) & (edm <= 1e-3 * np.maximum(chi2, 1.0))
    return _to_ext(u, lo, hi), chi2, converged, hess_ok


PULSE_FLOAT = ("pe", "peph", "time", "height", "beta", "chi2", "letime", "ped", "fit_A", "fit_mu", "fit_b")
PULSE_BOOL = ("failed", "zerondf", "pedfromdb")


def reconstruct(adc, n, start_tdc, pedestal_db, calib_area, calib_height, cfg, period, max_pulses=None):
    """Pulses of a batch of waveforms (pulsefit.py:236-316); max_pulses None = cfg.max_pulses."""
    adc = np.asarray(adc)
    W, L = adc.shape
    if W == 0:
        out = {k: np.zeros(0) for k in PULSE_FLOAT}
        out.update({k: np.zeros(0, np.int64) for k in ("wf", "seq")})
        out.update({k: np.zeros(0, bool) for k in PULSE_BOOL + ("wf_near_threshold",)})
        return out
    rounds = cfg.max_pulses if max_pulses is None else max_pulses
    y = adc.astype(float)
    under = pedestal_db - y[:, 0] > cfg.pedestal_undershoot_threshold
    ped = np.where(under, y[:, 0], pedestal_db)
    y = y - ped[:, None]
    valid = np.arange(L)[None, :] < n[:, None]
    y[~valid] = 0.0
    tgrid = (start_tdc[:, None] + np.arange(L)[None, :]) * period
    start = np.zeros(W, np.int64)
    active = np.ones(W, bool)
    failed_before = np.zeros(W, bool)
    near = _near_threshold(y, valid, cfg.min_adc_difference, cfg.knife_edge_adc)
    parts = []
    e = np.e
    for seq in range(rounds):
        found, ps, pe, fs, fe = find_next_peak(y, n, start, active, cfg)
        if not found.any():
            break
        k = np.flatnonzero(found)
        P = int((fe[k] - fs[k]).max()) + 1
        ypk = y[k, ps[k]]
        t0 = (start_tdc[k] + ps[k]) * period
        t1 = (start_tdc[k] + pe[k]) * period
        tpk = 0.5 * (t0 + t1)
        nk = len(k)
        p0 = np.stack([ypk * e, tpk, np.full(nk, cfg.default_beta)], 1)
        lo = np.stack([ypk * e * cfg.min_pulse_height_ratio, t0 - cfg.max_time_difference,
                       np.full(nk, cfg.min_beta)], 1)
        hi = np.stack([ypk * e * cfg.max_pulse_height_ratio, t1 + cfg.max_time_difference,
                       np.full(nk, cfg.max_beta)], 1)
        idx = fs[k, None] + np.arange(P)[None, :]
        mask = idx <= fe[k, None]
        idc = np.clip(idx, 0, L - 1)
        par, chi2, conv, hok = fit_gumbel(tgrid[k[:, None], idc], y[k[:, None], idc], mask, p0, lo, hi,
                                          cfg.lm_iterations)
        ndf = mask.sum(1) - 3
        span = hi - lo
        bad = (((par - lo) / span < cfg.limit_tolerance) | ((hi - par) / span < cfg.limit_tolerance)).any(1)
        failed = ~conv | ~hok | bad
        A, mu, b = par[:, 0], par[:, 1], par[:, 2]
        height = np.where(failed, ypk, A / e)
        beta = np.where(failed, cfg.default_beta, b)
        tpl = np.where(failed, tpk, mu)
        fseq = failed | failed_before[k]
        parts.append({"wf": k, "seq": np.full(nk, seq),
                      "pe": np.where(failed, ypk * e * cfg.default_beta, A * b) / calib_area[k],
                      "peph": height / calib_height[k], "time": tpl, "height": height, "beta": beta,
                      "chi2": np.where(failed | (ndf <= 0), -1.0, chi2 / np.maximum(ndf, 1)),
                      "letime": tpl - cfg.le_time_factor * beta, "failed": fseq, "zerondf": ndf <= 0,
                      "ped": ped[k], "pedfromdb": ~under[k], "fit_A": A, "fit_mu": mu, "fit_b": b})
        failed_before[k] = fseq
        sub = _round_half_away(_gumbel(tgrid[k], A[:, None], mu[:, None], b[:, None]))
        sub[np.arange(L)[None, :] >= n[k, None]] = 0.0
        y[k] -= sub
        near[k] |= _near_threshold(y[k], valid[k], cfg.min_adc_difference, cfg.knife_edge_adc)
        start[k] = fe[k]
        active = found
    keys = ("wf", "seq") + PULSE_FLOAT + PULSE_BOOL
    if parts:
        res = {kk: np.concatenate([p[kk] for p in parts]) for kk in keys}
        o = np.lexsort((res["seq"], res["wf"]))
        res = {kk: v[o] for kk, v in res.items()}
    else:
        res = {kk: np.zeros(0, bool if kk in PULSE_BOOL else np.int64 if kk in ("wf", "seq") else float)
               for kk in keys}
    res["wf_near_threshold"] = near
    return res


def reconstruct_full(adc, n, start_tdc, pedestal_db, calib_area, calib_height, cfg, period):
    return reconstruct(adc, n, start_tdc, pedestal_db, calib_area, calib_height, cfg, period,
                       max(cfg.max_pulses, int(np.max(n, initial=0))))


def filter_channels(P, channels, status, cfg):
    if not cfg.ignore_channels:
        return P
    keep = (np.asarray(status)[channels[P["wf"]]] & 0b010) == 0
    return {k: v if k == "wf_near_threshold" else v[keep] for k, v in P.items()}


# ---------------------------------------------------------------------------------------------------------------------
# coincidence finder (one event)

N_LAYERS = 4


def type_limits(G, cfg):
    """Per sector type: readout-end extremes, half length, largest time window, sides read out (coinc.py:112-122)."""
    out = {}
    for tt in np.unique(G.sector_type):
        secs = np.flatnonzero(G.sector_type == tt)
        cuts = [cfg.cuts[G.sector_names[s]] for s in secs if G.sector_names[s] in cfg.cuts]
        if not cuts:
            continue
        p0, p1 = G.pos_side0[secs].min(), G.pos_side1[secs].max()
        out[int(tt)] = dict(p0=p0, p1=p1, half=(p1 - p0) / 2, max_dt=max(c.max_dt for c in cuts),
                            side0=bool(G.sipms_side0[secs].any()), side1=bool(G.sipms_side1[secs].any()))
    return out


class _Hit:
    __slots__ = ("idx", "bar", "sector", "layer", "counter", "side", "sipm", "seq", "x", "y", "t", "pe", "cuts",
                 "maxd")

    def copy(self):
        h = _Hit()
        for k in self.__slots__:
            setattr(h, k, getattr(self, k))
        return h


def _greedy_clusters(hits, max_dt, opposite=False, dt_opp=0.0):
    """Greedy single linkage in list order; a scan repeats until a pass adds nothing (coinc.py:125-153)."""
    pool = list(hits)
    out = []
    while pool:
        cl = [pool.pop(0)]
        grew = True
        while grew:
            grew = False
            i = 0
            while i < len(pool):
                h = pool[i]
                link = False
                for c in cl:
                    lim_t = max_dt + (dt_opp if opposite and h.side != c.side else 0.0)
                    if abs(h.x - c.x) <= max(h.maxd, c.maxd) and abs(h.t - c.t) < lim_t:
                        link = True
                        break
                if link:
                    cl.append(pool.pop(i))
                    grew = True
                else:
                    i += 1
        out.append(cl)
    return out


def _combo_ok(combo):
    """Time window and slope cuts of one combination (coinc.py:156-181); returns the x gaps when it passes."""
    mdt = max(h.cuts.max_dt for h in combo)
    ts = [h.t for h in combo]
    if max(ts) - min(ts) > mdt:
        return False
    lo = min(h.cuts.min_slope for h in combo)
    hi = max(h.cuts.max_slope for h in combo)
    msd = max(h.cuts.max_slope_diff for h in combo)
    sl = []
    for a, b in zip(combo[:-1], combo[1:]):
        s = (b.x - a.x) / (b.y - a.y)
        if s < lo or s > hi:
            return False
        sl.append(s)
    if len(combo) > 2 and abs(sl[0] - sl[1]) > msd:
        return False
    if len(combo) > 3 and (abs(sl[0] - sl[2]) > msd or abs(sl[1] - sl[2]) > msd):
        return False
    return True


def _widen(combo):
    srt = sorted(combo, key=lambda h: h.x)
    for i, h in enumerate(srt):
        if i > 0:
            h.maxd = max(h.maxd, h.x - srt[i - 1].x)
        if i + 1 < len(srt):
            h.maxd = max(h.maxd, srt[i + 1].x - h.x)


def _coincidences(cluster, cfg):
    """Hits of a cluster that belong to a passing 2/3/4-layer combination (coinc.py:184-207)."""
    if not cluster:
        return []
    layers = [[] for _ in range(N_LAYERS)]
    for h in cluster:
        hh = h.copy()
        hh.maxd = h.cuts.final_max_distance
        layers[h.layer].append(hh)
    nmin = min(h.cuts.coincidence_layers for h in cluster)
    nmax = max(h.cuts.coincidence_layers for h in cluster)
    if len(cluster) > cfg.big_cluster_threshold and sum(1 for q in layers if q) >= nmin:
        return list(cluster)
    kept = {}
    for nl, need in ((2, nmin == 2), (3, nmin <= 3 <= nmax), (4, nmax == 4)):
        if not need:
            continue
        for ls in combinations(range(N_LAYERS), nl):
            sets = [layers[q] for q in ls]
            if any(not s for s in sets):
                continue
            for combo in _product(sets):
                if all(h.cuts.coincidence_layers > nl for h in combo):
                    continue
                if _combo_ok(combo):
                    _widen(combo)
                    for h in combo:
                        kept[h.idx] = h
    return [kept[i] for i in sorted(kept)]


def _product(sets):
    if not sets:
        yield []
        return
    for h in sets[0]:
        for rest in _product(sets[1:]):
            yield [h] + rest


def _attach(clusters, hits, max_dt):
    """Attach filtered first pulses on missing opposite counter ends (coinc_cpu.py:11-51)."""
    members = [h for cl in clusters for h in cl]
    if not clusters or not hits or not members:
        return
    mcl = [ci for ci, cl in enumerate(clusters) for _ in cl]
    midx = {h.idx for h in members}
    cand = [i for i, h in enumerate(hits) if h.seq == 0 and h.idx not in midx]
    anchors = [a for a, h in enumerate(members) if h.seq == 0]
    if not cand or not anchors:
        return
    occupied = {(mcl[a], h.bar, h.side) for a, h in enumerate(members)}
    best = []
    for c in cand:
        h = hits[c]
        opts = []
        for a in anchors:
            m = members[a]
            if m.bar != h.bar or h.side != 1 - m.side:
                continue
            dt = abs(h.t - m.t)
            if not dt < max_dt:
                continue
            if (mcl[a], h.bar, h.side) in occupied:
                continue
            opts.append((dt, mcl[a]))
        if opts:
            dt, cl = min(opts)
            best.append((cl, h.bar, h.sipm, dt, c))
    best.sort()
    seen = set()
    for cl, bar, sipm, dt, c in best:
        if (cl, bar, sipm) in seen:
            continue
        seen.add((cl, bar, sipm))
        clusters[cl].append(hits[c])


def _properties(tt, cl, G, lim, cfg):
    """Cluster properties (coinc.py:357-392)."""
    pe = np.array([h.pe for h in cl])
    tot = pe.sum()
    if tot < min(h.cuts.min_cluster_pes for h in cl):
        return None
    x = np.array([h.x for h in cl])
    y = np.array([h.y for h in cl])
    pos = (np.array([G.pos[h.bar] for h in cl]) * pe[:, None]).sum(0) / tot
    slope = ((tot * (pe * x * y).sum() - (pe * x).sum() * (pe * y).sum())
             / (tot * (pe * y * y).sum() - (pe * y).sum() ** 2))
    t = np.array([h.t for h in cl])
    side = np.array([h.side for h in cl])
    pos_ = pe > 0
    nh = [int(((side == s) & pos_).sum()) for s in (0, 1)]
    spe = [float(pe[(side == s) & pos_].sum()) for s in (0, 1)]
    st = [float((t * pe)[(side == s) & pos_].sum() / spe[s]) if spe[s] > 0 else 0.0 for s in (0, 1)]
    tmin = [t[(side == s) & pos_].min() if nh[s] else 0.0 for s in (0, 1)]
    tmax = [t[(side == s) & pos_].max() if nh[s] else 0.0 for s in (0, 1)]
    ld = int(G.length_dir[cl[0].sector])
    v = cfg.fiber_signal_speed
    calc = False
    if nh[0] and nh[1]:
        org = 0.5 * (v * (st[0] - st[1]) + (lim["p0"] + lim["p1"]))
        if (lim["p0"] < org < lim["p1"] and tmax[0] - tmin[0] < cfg.max_time_interval
                and tmax[1] - tmin[1] < cfg.max_time_interval):
            calc = True
            pos[ld] = org
            avg = st[0] - (org - lim["p0"]) / v
        else:
            org = pos[ld]
            avg = 0.5 * ((st[0] - (org - lim["p0"]) / v) + (st[1] - (lim["p1"] - org) / v))
    else:
        org = pos[ld]
        avg = (st[0] - (org - lim["p0"]) / v) if nh[0] else (st[1] - (lim["p1"] - org) / v)
    return dict(sectortype=tt, start=float(t.min()), end=float(t.max()), pe=float(tot), slope=float(slope),
                layers=sorted({h.layer for h in cl}), pulses=[h.idx for h in cl], poscalc=calc,
                avgtime=float(avg - cfg.time_offset), pos=pos, sidepe=spe, sidetime=st, sidehits=nh)


def find_event(p, G, status, cfg):
    """Coincidence clusters of one event's pulses (idx, bar, sipm, time, pe, seq) (coinc.py:289-354)."""
    lim = type_limits(G, cfg)
    by_type = {}
    for i in range(len(p["idx"])):
        if cfg.ignore_secondary_pulses and p["seq"][i] > 0:
            continue
        bar = int(p["bar"][i])
        s = int(G.sector[bar])
        name = G.sector_names[s]
        if name not in cfg.cuts:
            continue
        tt = int(G.sector_type[s])
        h = _Hit()
        h.idx, h.bar, h.sector, h.layer = int(p["idx"][i]), bar, s, int(G.layer[bar])
        h.counter, h.sipm, h.seq = int(G.counter_in_type[bar]), int(p["sipm"][i]), int(p["seq"][i])
        h.side = h.sipm % 2
        t = float(p["time"][i])
        t += ((G.pos_side0[s] - lim[tt]["p0"]) if h.side == 0 else (lim[tt]["p1"] - G.pos_side1[s])) \
            / cfg.fiber_signal_speed
        h.t = t
        pe = float(p["pe"][i])
        partner = bar * 4 + h.sipm + (2 if h.sipm < 2 else -2)
        if any((int(status[partner]) >> b) & 1 for b in cfg.compensate_status_bits):
            pe *= 2.0
        h.pe = pe
        h.x, h.y = float(G.x[bar]), float(G.y[bar])
        h.cuts = cfg.cuts[name]
        h.maxd = h.cuts.initial_max_distance
        by_type.setdefault(tt, []).append(h)
    rows = []
    for tt in sorted(by_type):
        H = by_type[tt]
        lm = lim[tt]
        coinc, filtered = [], []
        for side in (0, 1):
            keep = []
            for h in H:
                if h.side != side:
                    continue
                same = left = right = 0.0
                for a in H:
                    if a.side != side or a.layer != h.layer or abs(a.t - h.t) > h.cuts.max_dt_adjacent:
                        continue
                    d = a.counter - h.counter
                    same += a.pe if d == 0 else 0.0
                    left += a.pe if d == -1 else 0.0
                    right += a.pe if d == 1 else 0.0
                if same + left >= h.cuts.pe_threshold or same + right >= h.cuts.pe_threshold:
                    keep.append(h)
            filtered.extend(keep)
            for cl in _greedy_clusters(keep, lm["max_dt"]):
                coinc += _coincidences(cl, cfg)
        both = lm["side0"] and lm["side1"]
        dt_opp = 2.0 * lm["half"] / cfg.fiber_signal_speed
        cls = _greedy_clusters(coinc, lm["max_dt"], both, dt_opp)
        if both and cfg.add_opposite_side_pulses:
            _attach(cls, filtered, lm["max_dt"] + dt_opp)
        for cl in cls:
            r = _properties(tt, cl, G, lm, cfg)
            if r is not None:
                rows.append(r)
    return rows


# ---------------------------------------------------------------------------------------------------------------------
# chain glue

def clusters_from_pulses(W, P, G, status, fcfg, detail=False):
    """Per-event coincidence finding over sorted pulses (crv/crvfastsim/chain.py:325-362)."""
    wf = P["wf"]
    ev = W["ev"][wf]
    o = np.lexsort((P["seq"], wf, ev))
    ev, wf = ev[o], wf[o]
    idx = np.arange(len(ev)) - np.searchsorted(ev, ev)
    bar, sipm, time, pe, seq = W["bar"][wf], W["sipm"][wf], P["time"][o], P["pe"][o], P["seq"][o]
    cl = {k: [] for k in ("cl_event", "cl_type", "cl_pe", "cl_start", "cl_end", "cl_slope", "cl_avgtime",
                          "cl_poscalc")}
    mem = {"cl_pos": [], "mem_cl": [], "mem_idx": [], "mem_event": []}
    side = {"cl_sidepe": [], "cl_sidetime": [], "cl_sidehits": []}
    ue, lo = np.unique(ev, return_index=True)
    hi = np.r_[lo[1:], len(ev)]
    for e, a, b in zip(ue, lo, hi):
        p = dict(idx=idx[a:b], bar=bar[a:b], sipm=sipm[a:b], time=time[a:b], pe=pe[a:b], seq=seq[a:b])
        for r in find_event(p, G, status, fcfg):
            cl["cl_event"].append(e)
            for k, src in (("cl_type", "sectortype"), ("cl_pe", "pe"), ("cl_start", "start"), ("cl_end", "end"),
                           ("cl_slope", "slope"), ("cl_avgtime", "avgtime"), ("cl_poscalc", "poscalc")):
                cl[k].append(r[src])
            n = len(cl["cl_event"]) - 1
            mem["cl_pos"].append(np.asarray(r["pos"], float))
            side["cl_sidepe"].append(np.asarray(r["sidepe"], float))
            side["cl_sidetime"].append(np.asarray(r["sidetime"], float))
            side["cl_sidehits"].append(np.asarray(r["sidehits"], np.int64))
            side.setdefault("cl_layers", []).append(list(r["layers"]))
            mem["mem_cl"] += [n] * len(r["pulses"])
            mem["mem_idx"] += list(r["pulses"])
            mem["mem_event"] += [e] * len(r["pulses"])
    out = {k: np.asarray(v) for k, v in cl.items()}
    out.update({k: np.asarray(v, np.int64) for k, v in mem.items() if k != "cl_pos"})
    out["cl_pos"] = np.asarray(mem["cl_pos"], float).reshape(-1, 3)
    out["cl_sidepe"] = np.asarray(side["cl_sidepe"], float).reshape(-1, 2)
    out["cl_sidetime"] = np.asarray(side["cl_sidetime"], float).reshape(-1, 2)
    out["cl_sidehits"] = np.asarray(side["cl_sidehits"], np.int64).reshape(-1, 2)
    out["cl_layers"] = side.get("cl_layers", [])
    out["pulses"] = dict(ev=ev, idx=idx, bar=bar, sipm=sipm, seq=seq, pe=pe, time=time)
    return out


def pulses_from_waveforms(W, cond, rcfg, period):
    """reconstruct_full + filter_channels + DB time offset (+ event_t0) (crv/crvfastsim/chain.py:317-323)."""
    P = reconstruct_full(W["adc"], W["n"], W["start"], W["ped"], W["area"], W["height"], rcfg, period)
    P = filter_channels(P, W["bar"] * 4 + W["sipm"], cond.status, rcfg)
    if rcfg.use_time_offset_db:
        P["time"] = P["time"] + W["toff"][P["wf"]] * rcfg.time_offset_scale
    if "event_t0" in W:
        P["time"] = P["time"] + W["event_t0"][P["wf"]]
    return P


# ---- lookup-table photon model (photons._substep_photons) ---------------------------------------------------------

LOOKUP_EDGES = ("x", "y", "z", "beta", "theta", "phi", "r")
LOOKUP_TABLES = ("scint", "ckscint", "ckfiber")


class _OrcLookupTable(ctypes.Structure):
    _fields_ = [("prob", ctypes.c_void_p), ("delays", ctypes.c_void_p), ("delay_sum", ctypes.c_void_p),
                ("emis", ctypes.c_void_p), ("emis_sum", ctypes.c_void_p), ("nbins", ctypes.c_int32),
                ("ndelay", ctypes.c_int32), ("nemis", ctypes.c_int32), ("pad", ctypes.c_int32)]


class _OrcLookup(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("half_thickness", "half_width", "half_length", "fiber_separation",
                                               "hole_radius_x", "hole_radius_y", "fiber_radius", "corner_radius",
                                               "fiber_decay_time")] + \
        [("edges", ctypes.c_void_p * 7), ("nedges", ctypes.c_int32 * 7), ("pad", ctypes.c_int32),
         ("cos_phi_edges", ctypes.c_void_p), ("table", _OrcLookupTable * 3), ("cos_theta_edges", ctypes.c_void_p)]


class _OrcRows(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("s", "d", "t0", "t1", "beta", "theta", "dev", "mu", "nsub", "step",
                                               "chan", "n_scint", "n_ck_s", "n_ck_f", "cos_theta")]


def _lookup_struct(L, k):
    """OrcLookup of a lookup table object with the reference's fields (lookup.LookupTable), arrays kept alive by k."""
    S = _OrcLookup(*[float(getattr(L, f)) for f in ("half_thickness", "half_width", "half_length",
                                                    "fiber_separation", "hole_radius_x", "hole_radius_y",
                                                    "fiber_radius", "corner_radius", "fiber_decay_time")])
    for i, e in enumerate(LOOKUP_EDGES):
        S.edges[i] = k(L.edges[e], np.float64)
        S.nedges[i] = len(L.edges[e])
    S.cos_phi_edges = k(np.cos(np.asarray(L.edges["phi"], np.float64)), np.float64)
    S.cos_theta_edges = k(np.cos(np.asarray(L.edges["theta"], np.float64)), np.float64)
    for i, name in enumerate(LOOKUP_TABLES):
        T = L.tables[name]
        d, e = np.asarray(T.delays, np.uint8), np.asarray(T.emis, np.uint8)
        S.table[i] = _OrcLookupTable(k(T.prob, np.float32), k(d, np.uint8), k(T.delay_sum, np.int32),
                                     k(e, np.uint8), k(T.emis_sum, np.int32), len(T.prob), d.shape[1], e.shape[1], 0)
    return S


def substep_photons(L, rows, seed):
    """(step index, channel, time) of the photons of (step, SiPM) rows through lookup table L, keyed by seed, in
    (row, substep, table, arrival) order; rows as the reference's substep rows (photons.py:163-224).  Returns
    (step, chan, time, limit_flag)."""
    k = _Keep()
    S = _lookup_struct(L, k)
    n = len(rows["nsub"])
    mu = rows.get("mu")
    th = rows.get("theta")
    R = _OrcRows(k(rows["s"], np.float64), k(rows["d"], np.float64), k(rows["t0"], np.float64),
                 k(rows["t1"], np.float64), k(rows["beta"], np.float64), None if th is None else k(th, np.float64),
                 k(rows["dev"], np.float64), None if mu is None else k(mu, np.float64), k(rows["nsub"], np.int64),
                 k(rows["step"], np.int64), k(rows["chan"], np.int64), k(rows["n_scint"], np.int64),
                 k(rows["n_ck_s"], np.int64), k(rows["n_ck_f"], np.int64),
                 None if th is not None else k(rows["cos_theta"], np.float64))
    f = lib().orc_substep_photons
    f.restype = ctypes.c_int64
    lim = ctypes.c_int(0)
    m = f(ctypes.byref(S), ctypes.c_uint32(seed), ctypes.byref(R), ctypes.c_int64(n), None, None, None,
          ctypes.byref(lim))
    st, ch, tm = np.zeros(m, np.int64), np.zeros(m, np.int64), np.zeros(m)
    if m:
        f(ctypes.byref(S), ctypes.c_uint32(seed), ctypes.byref(R), ctypes.c_int64(n), _p(st), _p(ch), _p(tm),
          ctypes.byref(lim))
    return st, ch, tm, bool(lim.value)


def substep_bins(L, rows):
    """[substeps, 3] bins of the scintillation, Cherenkov-in-scintillator and Cherenkov-in-fibre tables of every
    substep of every row (row-major; -1 where the substep selects none)."""
    k = _Keep()
    S = _lookup_struct(L, k)
    th = rows.get("theta")
    mu = rows.get("mu")
    R = _OrcRows(k(rows["s"], np.float64), k(rows["d"], np.float64), k(rows["t0"], np.float64),
                 k(rows["t1"], np.float64), k(rows["beta"], np.float64), None if th is None else k(th, np.float64),
                 k(rows["dev"], np.float64), None if mu is None else k(mu, np.float64), k(rows["nsub"], np.int64),
                 k(rows["step"], np.int64), k(rows["chan"], np.int64), k(rows["n_scint"], np.int64),
                 k(rows["n_ck_s"], np.int64), k(rows["n_ck_f"], np.int64),
                 None if th is not None else k(rows["cos_theta"], np.float64))
    out = np.zeros((int(np.sum(rows["nsub"])), 3), np.int32)
    lib().orc_substep_bins(ctypes.byref(S), ctypes.byref(R), ctypes.c_int64(len(rows["nsub"])), _p(out))
    return out


def first_reaching(wts, bins, thr):
    """Delay / emission index for bins and thresholds: the first j whose running sum of wts[bin] reaches thr."""
    w = np.ascontiguousarray(wts, np.uint8)
    b = np.ascontiguousarray(bins, np.int64)
    t = np.ascontiguousarray(thr, np.float64)
    out = np.zeros(len(b), np.int32)
    lib().orc_first_reaching_v(_p(w), ctypes.c_int(w.shape[1]), ctypes.c_int64(len(b)), _p(b), _p(t), _p(out))
    return out


def binomial(seed, n, p):
    """The substep sampler's Binomial(n[i], p[i]) draws (block keyed by i)."""
    n = np.ascontiguousarray(n, np.int64)
    p = np.ascontiguousarray(p, np.float64)
    out = np.zeros(len(n), np.int64)
    lib().orc_binomial_v(ctypes.c_uint32(seed), ctypes.c_int64(len(n)), _p(n), _p(p), _p(out))
    return out


class _OrcLookupSteps(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("x0", "y0", "z0", "x1", "y1", "z1", "px0", "py0", "pz0", "p1", "t0",
                                               "t1", "edep", "len", "bar", "pdg")]


class _OrcLookupGroup(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("center", "l2w", "in_group", "yield_", "speed_k", "mu", "dev",
                                               "ck_scint", "ck_fiber", "pdg_code", "pdg_mass", "pdg_charge")] + \
        [("half_length", ctypes.c_double)] + [(k, ctypes.c_int32) for k in ("reflector", "nbars", "nck_scint",
                                                                             "nck_fiber", "npdg", "pad")]


ROW_KEYS = ("s", "d", "t0", "t1", "beta", "cos_theta", "dev", "mu", "nsub", "step", "chan", "n_scint", "n_ck_s",
            "n_ck_f")


def lookup_rows(group, steps, seed):
    """Rows of one (table, reflector) group (photons.iter_rows with keyed per-substep counts).  group: dict of the
    group arrays (center [nb, 3], l2w [nb, 3], in_group, yield, speed_k, mu, dev [4 nb], ck_scint [n, 2], ck_fiber,
    pdg_code, pdg_mass, pdg_charge, half_length, reflector); steps: dict of the step columns (x0 .. z1, px0, py0, pz0,
    p1, t0, t1, edep, len, bar, pdg).  Returns the row dict (cos_theta in place of theta)."""
    k = _Keep()
    G = _OrcLookupGroup(k(group["center"], np.float64), k(group["l2w"], np.int8), k(group["in_group"], np.int32),
                        k(group["yield"], np.float64), k(group["speed_k"], np.float64), k(group["mu"], np.float64),
                        k(group["dev"], np.float64), k(group["ck_scint"], np.float64), k(group["ck_fiber"], np.float64),
                        k(group["pdg_code"], np.int64), k(group["pdg_mass"], np.float64),
                        k(group["pdg_charge"], np.float64), float(group["half_length"]), int(group["reflector"]),
                        len(group["in_group"]), len(group["ck_scint"]), len(group["ck_fiber"]), len(group["pdg_code"]),
                        0)
    n = len(steps["bar"])
    cols = [k(steps[c], np.float64) for c in ("x0", "y0", "z0", "x1", "y1", "z1", "px0", "py0", "pz0", "p1", "t0",
                                              "t1", "edep", "len")]
    S = _OrcLookupSteps(*cols, k(steps["bar"], np.int32), k(steps["pdg"], np.int64))
    cap = (4 if int(group["reflector"]) == 0 else 2) * n
    out = {key: np.zeros((cap, 3) if key in ("s", "d") else cap,
                         np.int64 if key in ("nsub", "step", "chan", "n_scint", "n_ck_s", "n_ck_f") else np.float64)
           for key in ROW_KEYS}
    f = lib().orc_lookup_rows
    f.restype = ctypes.c_int64
    m = f(ctypes.byref(G), ctypes.c_uint32(seed), ctypes.byref(S), ctypes.c_int64(n), *[_p(out[key]) for key in ROW_KEYS])
    return {key: v[:m] for key, v in out.items()}


# photons.make_photons with lookup tables: host part of photons.iter_rows (crv/crvfastsim/response/photons.py:230-356)

_PARTICLES = {11: (0.51099895, -1), -11: (0.51099895, 1), 13: (105.6583755, -1), -13: (105.6583755, 1),
              22: (0.0, 0), 211: (139.57039, 1), -211: (139.57039, -1), 111: (134.9768, 0), 321: (493.677, 1),
              -321: (493.677, -1), 130: (497.611, 0), 310: (497.611, 0), 2212: (938.272088, 1),
              -2212: (938.272088, -1), 2112: (939.565420, 0), -2112: (939.565420, 0), 12: (0.0, 0), -12: (0.0, 0),
              14: (0.0, 0), -14: (0.0, 0), 3122: (1115.683, 0), 3222: (1189.37, 1), 3112: (1197.449, -1)}


def table_propagation(L):
    """photons.table_propagation (photons.py:230-254): inverse signal speed from the 10 % delay quantile against the
    distance to the SiPM end, attenuation length from the log of the summed probability."""
    E, T = L.edges, L.tables["scint"]
    nx, ny, nz = len(E["x"]) - 1, len(E["y"]) - 1, len(E["z"]) - 1
    p = np.asarray(T.prob, np.float64)[:nx * ny * nz].reshape(nx, ny, nz)
    ds = np.asarray(T.delay_sum, np.float64)[:nx * ny * nz].reshape(nx, ny, nz)
    w = np.where(ds > 0, p / np.where(ds > 0, ds, 1.0), 0.0)
    h = np.einsum("xyz,xyzj->zj", w, np.asarray(T.delays, np.float64)[:nx * ny * nz].reshape(nx, ny, nz, -1))
    d = 0.5 * (np.asarray(E["z"])[1:] + np.asarray(E["z"])[:-1]) + L.half_length
    tot = h.sum(1)
    ok = tot > 0
    q = np.argmax(np.cumsum(h, 1) >= 0.1 * tot[:, None], axis=1)
    inv_v = np.polyfit(d[ok], q[ok].astype(float), 1)[0]
    P = p.sum((0, 1))
    a = (P > 0) & (d > 0.2 * L.half_length) & (d < 1.8 * L.half_length)
    return float(inv_v), float(-1.0 / np.polyfit(d[a], np.log(P[a]), 1)[0])


def bar_ratios(values, geom):
    """photons.bar_ratios (photons.py:257-289)."""
    out = np.ones(geom.nbars)
    if not values:
        return out
    names = np.array(geom.sector_names, dtype=object)
    nmod = np.zeros(len(names), np.int64)
    np.maximum.at(nmod, np.asarray(geom.sector), np.asarray(geom.module) + 1)
    sk = names[np.asarray(geom.sector)]
    mk = np.where(nmod[np.asarray(geom.sector)] > 1, sk + np.asarray(geom.module).astype(str).astype(object), sk)
    known = set(sk) | set(mk) | {"TAG"}
    bad = sorted(set(values) - known)
    if bad:
        raise KeyError(f"unknown propagation keys {bad}; known: {sorted(known)}")
    tag = np.array([str(n).startswith("M") for n in sk])
    for k, v in values.items():
        if k == "TAG":
            out[tag] = v
    for k, v in values.items():
        if k != "TAG" and k in set(sk):
            out[sk == k] = v
    for k, v in values.items():
        if k in set(mk) and k not in set(sk):
            out[mk == k] = v
    if not np.all(out > 0):
        raise ValueError("propagation ratios must be positive")
    return out


def lookup_groups(geom, cfg, tables, deviation):
    """[(table, group arrays)] in photons.iter_rows' order (table names sorted, reflectors sorted)."""
    names = list(geom.sector_names)
    sec = np.asarray(geom.sector)
    nb = int(geom.nbars)
    r_speed, r_atten = bar_ratios(cfg.speed_ratio, geom), bar_ratios(cfg.atten_ratio, geom)
    dev = (np.asarray(deviation, np.float64) * cfg.photon_yield_variation_scale + 1.0) * cfg.photon_yield_scale
    codes = np.array(sorted(_PARTICLES), np.int64)
    yields = np.array([float(cfg.sectors[n].yield_per_mev) for n in names])
    out = []
    for tname in sorted({cfg.sectors[n].table for n in names}):
        L = tables[tname]
        inv_v, att = table_propagation(L)
        for refl in sorted({int(cfg.sectors[n].reflector) for n in names if cfg.sectors[n].table == tname}):
            sids = [i for i, n in enumerate(names) if cfg.sectors[n].table == tname
                    and int(cfg.sectors[n].reflector) == refl]
            g = dict(center=np.asarray(geom.center, np.float64).reshape(nb, 3),
                     l2w=np.asarray(geom.local_to_world, np.int8).reshape(nb, 3),
                     in_group=np.isin(sec, sids).astype(np.int32), yield_=yields[sec],
                     speed_k=inv_v * (1.0 / r_speed - 1.0), mu=(1.0 / r_atten - 1.0) / att, dev=dev,
                     ck_scint=np.asarray(L.ck_scint, np.float64).reshape(-1, 2),
                     ck_fiber=np.asarray(L.ck_fiber, np.float64).reshape(-1, 2), pdg_code=codes,
                     pdg_mass=np.array([_PARTICLES[c][0] for c in codes]),
                     pdg_charge=np.array([_PARTICLES[c][1] for c in codes], np.float64),
                     half_length=float(L.half_length), reflector=refl)
            g["yield"] = g.pop("yield_")
            out.append((L, g))
    return out


def make_photons_lookup(steps, pdg, geom, cfg, tables, deviation, seed):
    """(step, channel, time) of photons.make_photons with lookup tables and keyed draws: rows per group, then the
    substep photons of each group's rows."""
    cols = {k: np.asarray(steps[k], np.float64) for k in ("x0", "y0", "z0", "x1", "y1", "z1", "px0", "py0", "pz0",
                                                          "p1", "t0", "t1", "edep", "len")}
    cols["bar"] = np.asarray(steps["bar"], np.int32)
    cols["pdg"] = np.asarray(pdg, np.int64)
    outs = []
    for L, g in lookup_groups(geom, cfg, tables, deviation):
        rows = lookup_rows(g, cols, seed)
        if len(rows["nsub"]):
            outs.append(substep_photons(L, rows, seed)[:3])
    if not outs:
        return np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0)
    return tuple(np.concatenate([o[i] for o in outs]) for i in range(3))


def find_bin(edges, v):
    """The lookup model's bin search (the stock findBin: the first i with e[i] <= v <= e[i+1]; -1 outside)."""
    e = np.ascontiguousarray(edges, np.float64)
    v = np.ascontiguousarray(v, np.float64)
    out = np.zeros(len(v), np.int32)
    lib().orc_find_bin_v(_p(e), ctypes.c_int(len(e)), ctypes.c_int64(len(v)), _p(v), _p(out))
    return out


def find_bin_cos(edges, c):
    """The phi / theta bins found on cos: bins of arccos(c) over angle edges in [0, pi]."""
    ce = np.ascontiguousarray(np.cos(np.asarray(edges, np.float64)))
    c = np.ascontiguousarray(c, np.float64)
    out = np.zeros(len(c), np.int32)
    lib().orc_find_bin_cos_v(_p(ce), ctypes.c_int(len(ce)), ctypes.c_int64(len(c)), _p(c), _p(out))
    return out


def cerenkov_per_mm(beta, charge, cmap):
    """Cherenkov photons per mm: linear in beta from (0, 0) through the map, flat beyond its end, times |charge|."""
    m = np.ascontiguousarray(cmap, np.float64).reshape(-1, 2)
    b = np.ascontiguousarray(beta, np.float64)
    q = np.ascontiguousarray(charge, np.float64)
    out = np.zeros(len(b))
    lib().orc_cerenkov_v(_p(m), ctypes.c_int(len(m)), ctypes.c_int64(len(b)), _p(b), _p(q), _p(out))
    return out


def particle_beta(pdg, p0, p1):
    """(mass, charge, stock beta) of particle codes with start / end momenta, as the row preparation uses them."""
    codes = np.array(sorted(_PARTICLES), np.int64)
    mass = np.array([_PARTICLES[c][0] for c in codes])
    charge = np.array([_PARTICLES[c][1] for c in codes], np.float64)
    pdg = np.ascontiguousarray(pdg, np.int64)
    p0 = np.ascontiguousarray(p0, np.float64)
    p1 = np.ascontiguousarray(p1, np.float64)
    n = len(pdg)
    m, q, b = np.zeros(n), np.zeros(n), np.zeros(n)
    lib().orc_particle_beta_v(_p(codes), ctypes.c_int(len(codes)), _p(mass), _p(charge), ctypes.c_int64(n), _p(pdg),
                              _p(p0), _p(p1), _p(m), _p(q), _p(b))
    return m, q, b
