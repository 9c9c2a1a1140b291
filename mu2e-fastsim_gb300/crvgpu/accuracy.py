"""Error report of an FP32-mixed chain run against the FP64-plain run of the same events and keys.

Both runs draw the same keyed random numbers, so their outputs describe the same physics and differ only through
arithmetic precision; where a quantity crosses a decision boundary (a sample on an ADC integer, a fit near a failure
test, a pulse near a zero-suppression threshold) the two runs can differ in a discrete way.  Nothing here requires
equal counts: digis are matched by (SiPM label, start TDC), pulses by SiPM label and nearest time, finder hits the
same way, and clusters by (event, sector type, member set), so the report is complete whatever the two runs produced.

Reported per quantity:
  charges      counts, mean PE relative error, and the SiPMs whose charge list differs (an FP32 recovery or firing
               decision at its threshold: a different charge, not an arithmetic error downstream);
  digis        matched fraction; ADC mismatch rate over the matched samples, split into digis of SiPMs whose charges
               agree (waveform arithmetic alone: the fraction of mismatches at a quantisation boundary, i.e. one count
               apart with the FP64 value closer to the ADC step than the FP32-vs-FP64 difference, the largest |dADC|,
               |dV| quantiles) and digis of SiPMs whose charges differ;
  pulses       counts, mean PE relative error (all pulses, and matched well-fitted pairs), |dt| p50 / p99 / max on
               matched well-fitted pairs, matched fraction;
  clusters     counts, the fraction of FP64 clusters with an FP32 cluster of the same event, sector type and member
               pulses, and PE / start-time differences of those pairs.
"""
from __future__ import annotations

import numpy as np

PULSE_MATCH_NS = 2.0      # pulses of one SiPM are several samples (12.55 ns) apart; a match is within 2 ns


def _np(x):
    return x.detach().cpu().numpy() if hasattr(x, "detach") else np.asarray(x)


def _q(a, qs=(0.5, 0.99, 1.0)):
    a = np.asarray(a, float)
    return [float(v) for v in np.quantile(a, qs)] if len(a) else [None] * len(qs)


def match_nearest(key_a, t_a, key_b, t_b, tol):
    """For every item of a, the index of the item of b with the same key and the nearest time (within tol), else -1.
    One-to-one: when two a items want one b item, the nearer one gets it and the other takes its next-nearest free
    neighbour within tol."""
    key_a, t_a, key_b, t_b = (np.asarray(v) for v in (key_a, t_a, key_b, t_b))
    if len(key_a) == 0 or len(key_b) == 0:
        return np.full(len(key_a), -1, np.int64)
    ob = np.lexsort((t_b, key_b))
    kb, tb = key_b[ob], t_b[ob]
    # position of each a item in b's (key, time) order
    oa = np.lexsort((t_a, key_a))
    ka, ta = key_a[oa], t_a[oa]
    allk = np.concatenate([kb, ka])
    allt = np.concatenate([tb, ta])
    src = np.concatenate([np.zeros(len(kb), np.int8), np.ones(len(ka), np.int8)])
    o = np.lexsort((src, allt, allk))
    isb = src[o] == 0
    nb_before = np.cumsum(isb) - isb                     # b items strictly before each position
    pos_sorted = nb_before[~isb]                         # for a items in (key, time) order
    pos = np.empty(len(ka), np.int64)
    pos[:] = pos_sorted
    lo = np.searchsorted(kb, ka, "left")
    hi = np.searchsorted(kb, ka, "right")
    cands = []
    for d in (-1, 0):
        j = pos + d
        ok = (j >= lo) & (j < hi)
        jj = np.clip(j, 0, len(tb) - 1)
        cands.append((np.where(ok, np.abs(tb[jj] - ta), np.inf), jj))
    best = np.where(cands[0][0] <= cands[1][0], cands[0][1], cands[1][1])
    dist = np.minimum(cands[0][0], cands[1][0])
    res = np.full(len(ka), -1, np.int64)
    used = np.zeros(len(tb), bool)
    order = np.argsort(dist, kind="stable")
    order = order[dist[order] <= tol]
    # greedy one-to-one claim: in distance order, a b item goes to the first a item that wants it
    first = np.unique(best[order], return_index=True)[1]
    take = order[np.sort(first)]
    used[best[take]] = True
    res[take] = ob[best[take]]
    rest = np.setdiff1d(order, take)
    for i in rest:                                      # rare: two a items nearest to one b item
        for d in (-1, 0, 1, -2, 2):
            j = pos[i] + d
            if lo[i] <= j < hi[i] and not used[j] and abs(tb[j] - ta[i]) <= tol:
                used[j] = True
                res[i] = ob[j]
                break
    out = np.full(len(key_a), -1, np.int64)
    out[oa] = res
    return out


def changed_labels(l64, t64, q64, l32, t32, q32, t_tol=0.01, pe_rtol=1e-3):
    """SiPM labels whose charge lists differ between the two runs (inputs sorted by label, then time): a label present
    in one run only, a different charge count, or a charge whose time differs by more than t_tol ns or whose PE
    differs by more than pe_rtol relative."""
    u64, s64, c64 = np.unique(l64, return_index=True, return_counts=True)
    u32, s32, c32 = np.unique(l32, return_index=True, return_counts=True)
    both, j64, j32 = np.intersect1d(u64, u32, return_indices=True)
    eq = c64[j64] == c32[j32]
    changed = [np.setxor1d(u64, u32), both[~eq]]
    lab = both[eq]
    if len(lab):
        n = c64[j64][eq]
        rows64 = np.repeat(s64[j64][eq], n) + (np.arange(n.sum()) - np.repeat(np.cumsum(n) - n, n))
        rows32 = np.repeat(s32[j32][eq], n) + (np.arange(n.sum()) - np.repeat(np.cumsum(n) - n, n))
        bad = (np.abs(t64[rows64] - t32[rows32]) > t_tol) | \
              (np.abs(q64[rows64] - q32[rows32]) > pe_rtol * np.maximum(np.abs(q64[rows64]), 1e-300))
        per = np.add.reduceat(bad.astype(np.int64), np.cumsum(n) - n) > 0
        changed.append(lab[per])
    return np.unique(np.concatenate(changed)).astype(np.int64)


def digi_table(D64, D32, adc_conversion, adc_pedestal, changed=None):
    """Digis of two runs matched by (label, start TDC): ADC mismatch rate, and for the digis of SiPMs whose charges
    agree (labels not in `changed`) the fraction of mismatches at a quantisation boundary (one count apart, with the
    integer between the two values closer to the FP64 value than the FP32-vs-FP64 difference), the largest |dADC| and
    |dV| quantiles.  Charges that agree to 0.01 ns still differ by the SiPM stage's FP32 rounding (~1e-4 ns at 1 us):
    on the steep rise of the single-PE template that moves a charge across a 0.5 ns template step now and then, a
    real difference of the input the digitisation then reproduces exactly."""
    changed = np.zeros(0, np.int64) if changed is None else changed
    k64 = D64["chan"].astype(np.int64) * (1 << 24) + (D64["starttdc"].astype(np.int64) + (1 << 23))
    k32 = D32["chan"].astype(np.int64) * (1 << 24) + (D32["starttdc"].astype(np.int64) + (1 << 23))
    com, i64, i32 = np.intersect1d(k64, k32, assume_unique=False, return_indices=True)
    a64, a32 = D64["adc"][i64].astype(np.int64), D32["adc"][i32].astype(np.int64)
    v64, v32 = D64["volt"][i64], D32["volt"][i32]
    same_in = ~np.isin(D64["chan"][i64], changed)
    mis = a64 != a32
    x64 = v64 * adc_conversion + adc_pedestal + 0.5
    x32 = v32 * adc_conversion + adc_pedestal + 0.5
    edge = np.maximum(np.floor(x64), np.floor(x32))
    at_boundary = (np.abs(a64 - a32) == 1) & (np.abs(x64 - edge) <= np.abs(x32 - x64) + 1e-9)
    ms, mc = mis[same_in], mis[~same_in]
    dv = np.abs(v32 - v64)
    return {"fp64": int(len(k64)), "fp32": int(len(k32)), "matched": int(len(com)),
            "matched_frac": float(len(com) / max(len(k64), 1)),
            "adc_samples_compared": int(a64.size), "adc_mismatch_rate": float(mis.sum() / max(a64.size, 1)),
            "adc_mismatch_at_boundary_frac": float(at_boundary[mis].mean()) if mis.any() else 1.0,
            # the rest: an FP32 time offset that moves a charge across a 0.5 ns step of the single-PE template
            "adc_mismatch_template_step_frac": float(1.0 - at_boundary[mis].mean()) if mis.any() else 0.0,
            "adc_mismatch_max_abs": int(np.abs(a64 - a32).max()) if a64.size else 0,
            "same_charges": {
                "adc_samples": int(ms.size), "adc_mismatch_rate": float(ms.sum() / max(ms.size, 1)),
                "adc_mismatch_at_boundary_frac": float(at_boundary[same_in][ms].mean()) if ms.any() else 1.0,
                "adc_mismatch_max_abs": int(np.abs(a64 - a32)[same_in].max()) if ms.size else 0,
                "volt_abs_err_mV_p50_p99_max": [None if v is None else 1e3 * v for v in _q(dv[same_in].ravel())]},
            "different_charges": {
                "adc_samples": int(mc.size), "adc_mismatch_rate": float(mc.sum() / max(mc.size, 1)),
                "adc_mismatch_max_abs": int(np.abs(a64 - a32)[~same_in].max()) if mc.size else 0}}


def waveform_only_table(eng32, r64, adc_conversion, adc_pedestal):
    """The FP32-mixed waveform stage alone: it digitises the FP64 run's own charges, so the inputs are identical and
    every ADC difference is the waveform arithmetic's."""
    R = r64.charges
    D = eng32.dig.run(eng32.params(r64.seed), eng32.tabs, R.label, R.time, R.charge, eng32.tmpl, r64.ev_keys,
                      r64.ev_runs)
    D64 = {k: _np(v) for k, v in r64.digis.items()}
    D32 = {k: _np(v) for k, v in D.items()}
    t = digi_table(D64, D32, adc_conversion, adc_pedestal)
    return {k: t[k] for k in ("fp64", "fp32", "matched_frac", "adc_samples_compared", "adc_mismatch_rate",
                              "adc_mismatch_at_boundary_frac", "adc_mismatch_template_step_frac",
                              "adc_mismatch_max_abs")}


def error_table(r64, r32, adc_conversion, adc_pedestal):
    """FP32-mixed vs FP64 report of two ChainResults of the same batch and seed (both run with keep=True)."""
    out = {}
    # ---- charges: the SiPM stage's FP32 recovery / firing decisions can differ from FP64 at a threshold, which
    # changes a SiPM's charge list; digis of such SiPMs differ for that reason, not through waveform arithmetic
    R64, R32 = r64.charges, r32.charges
    l64, l32 = _np(R64.label), _np(R32.label)
    t64, t32 = _np(R64.time), _np(R32.time)
    q64, q32 = _np(R64.pe), _np(R32.pe)
    changed = changed_labels(l64, t64, q64, l32, t32, q32)
    nlab = len(np.union1d(np.unique(l64), np.unique(l32)))
    out["charges"] = {"fp64": int(len(q64)), "fp32": int(len(q32)),
                      "mean_pe_rel": float(q32.mean() / q64.mean() - 1) if len(q64) and len(q32) else None,
                      "sipms": int(nlab), "sipms_with_different_charges": int(len(changed)),
                      "sipms_with_different_charges_frac": float(len(changed) / max(nlab, 1))}
    # ---- digis by (label, start TDC); ADC mismatches split by whether the SiPM's charges agree
    D64 = {k: _np(v) for k, v in r64.digis.items()}
    D32 = {k: _np(v) for k, v in r32.digis.items()}
    out["digis"] = digi_table(D64, D32, adc_conversion, adc_pedestal, changed)
    # ---- pulses by (SiPM label, nearest time)
    W64 = {k: _np(v) for k, v in r64.waveforms.items()}
    W32 = {k: _np(v) for k, v in r32.waveforms.items()}
    P64 = {k: _np(v) for k, v in r64.pulses.items()}
    P32 = {k: _np(v) for k, v in r32.pulses.items()}
    lab64, lab32 = W64["label"][P64["wf"]], W32["label"][P32["wf"]]
    m = match_nearest(lab64, P64["time"], lab32, P32["time"], PULSE_MATCH_NS)
    ok = m >= 0
    good = ok.copy()
    good[ok] = ~P64["failed"][ok].astype(bool) & ~P32["failed"][m[ok]].astype(bool)
    dt = np.abs(P32["time"][m[good]] - P64["time"][good])
    pe_pairs = (P32["pe"][m[good]].mean() / P64["pe"][good].mean() - 1) if good.any() else None
    out["pulses"] = {"fp64": int(len(lab64)), "fp32": int(len(lab32)), "matched": int(ok.sum()),
                     "matched_frac": float(ok.mean()) if len(ok) else 1.0,
                     "failed_flag_differs": int((P64["failed"][ok].astype(bool)
                                                 != P32["failed"][m[ok]].astype(bool)).sum()),
                     "mean_pe_rel": float(P32["pe"].mean() / P64["pe"].mean() - 1) if len(lab64) and len(lab32)
                     else None,
                     "mean_pe_rel_matched_good": None if pe_pairs is None else float(pe_pairs),
                     "time_abs_err_ns_p50_p99_max": _q(dt)}
    # ---- finder hits and clusters
    H64 = {k: _np(v) for k, v in r64.hits.items()}
    H32 = {k: _np(v) for k, v in r32.hits.items()}

    def hit_keys(H):
        n = len(H["bar"])
        ev = np.repeat(H["ev_key"], H["ev_count"])[:n]
        return ev, ev * 32768 + H["bar"].astype(np.int64) * 4 + H["sipm"]

    ev64, hk64 = hit_keys(H64)
    ev32, hk32 = hit_keys(H32)
    hm = match_nearest(hk32, H32["time"], hk64, H64["time"], PULSE_MATCH_NS)   # FP32 hit -> FP64 hit

    def member_sets(r, H, hit_map):
        C = {k: _np(v) for k, v in r.clusters.items()}
        M = {k: _np(v) for k, v in r.members.items()}
        row0 = H["ev_start"][np.searchsorted(H["ev_key"], M["event"])] if len(M["event"]) else np.zeros(0, np.int64)
        rows = row0 + M["idx"]
        ids = hit_map(rows)
        sets = {}
        for c, h in zip(M["cl"], ids):
            sets.setdefault(int(c), []).append(int(h))
        keys = {}
        for c in range(len(C["pe"])):
            keys[(int(C["event"][c]), int(C["type"][c]), tuple(sorted(sets.get(c, []))))] = c
        return C, keys

    C64, s64 = member_sets(r64, H64, lambda rows: rows)
    unmatched = iter(range(-1, -10 ** 9, -1))
    C32, s32 = member_sets(r32, H32, lambda rows: np.array([hm[r] if hm[r] >= 0 else next(unmatched)
                                                             for r in rows], np.int64))
    same = [(s64[k], s32[k]) for k in s64 if k in s32]
    if same:
        a, b = np.array(same).T
        dpe = np.abs(C32["pe"][b] / C64["pe"][a] - 1)
        dst = np.abs(C32["start"][b] - C64["start"][a])
    else:
        dpe = dst = np.zeros(0)
    out["clusters"] = {"fp64": int(len(C64["pe"])), "fp32": int(len(C32["pe"])),
                       "same_members_frac": float(len(same) / max(len(s64), 1)),
                       "pe_rel_err_p50_p99_max": _q(dpe), "start_abs_err_ns_p50_p99_max": _q(dst)}
    return out
