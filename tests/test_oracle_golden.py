"""The oracle against golden fixtures generated from the reference itself (tests/golden/make_golden.py).

Integer outputs must be identical; floating outputs identical up to 1e-12 relative (the NumPy restatement performs
the reference's operations in the reference's order, so on the generating machine they are bit-identical; the
tolerance only covers a different libm/SIMD exp on another host).
"""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import oracle as O
from crvgpu import config as CF

FLOAT_RTOL = 1e-12


def assert_same(a, b, name):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, f"{name}: shape {a.shape} != {b.shape}"
    if a.dtype.kind in "fc" or b.dtype.kind in "fc":
        np.testing.assert_allclose(a, b, rtol=FLOAT_RTOL, atol=1e-300, err_msg=name)
    else:
        assert np.array_equal(a, b), f"{name}: values differ"


@pytest.mark.parametrize("tag", ["single", "kpp", "uneven", "edge", "p125"])
def test_pulsefit_matches_reference(golden, tag):
    g = golden("pulsefit.npz")
    period = 12.5 if tag == "p125" else float(g["period"][0])
    cfg = CF.RecoConfig(period=period)
    args = [g[f"{tag}_{k}"] for k in ("adc", "n", "start", "ped", "area", "height")]
    f = O.reconstruct_full if tag in ("uneven", "edge") else O.reconstruct
    r = f(*args, cfg, period)
    keys = [k[len(tag) + 5:] for k in g.files if k.startswith(f"{tag}_out_")]
    assert set(keys) == set(r)
    for k in keys:
        assert_same(r[k], g[f"{tag}_out_{k}"], f"{tag}.{k}")


def test_concat_matches_reference(golden):
    g = golden("concat.npz")
    gid, mat, n, start, first = O.concat_waveforms(g["key"], g["bar"], g["sipm"], g["tdc"], g["flat"], g["lens"])
    for k, v in (("gid", gid), ("mat", mat), ("n", n), ("start", start), ("first", first)):
        assert_same(v, g[k], k)


def _wf_cfg(g):
    return CF.WaveformConfig(min_voltage=float(g["min_voltage"][0]), single_pe_stretch=float(g["stretch"][0]))


def test_template_resampling_matches_reference(golden):
    g = golden("waveform.npz")
    t = O.resample_template(g["traw"], g["vraw"], 0.5, float(g["stretch"][0]), 100.0)
    assert_same(t, g["template"], "template")
    t2, v2 = O.gumbel_template_raw(CF.SPE_PEAK_VOLT, 15.0, 10.0)
    assert np.allclose(v2, g["vraw"], rtol=1e-15, atol=0)


@pytest.mark.parametrize("mode", ["clean", "noisy"])
def test_waveform_matches_reference(golden, mode):
    g = golden("waveform.npz")
    cfg = _wf_cfg(g)
    uch, tab = g["uch"], g["tdc0_tab"]
    lut = lambda lab: tab[np.searchsorted(uch, lab)]                     # noqa: E731
    noise = None
    if mode == "noisy":
        Z = g["noise_Z"]
        noise = lambda labels, tick0, shape: Z[:shape[0], :shape[1]]      # noqa: E731
    r = O.synthesize(g["chan"], g["time"], g["charge"], lut, g["template"], cfg, 12.55, tuple(g["window"]), noise)
    for k in ("chan", "start", "tdc0", "starttdc", "volt", "adc", "cluster_chan", "cluster_tstart", "cluster_keep"):
        assert_same(r[k], g[f"{mode}_{k}"], f"{mode}.{k}")
    if mode == "noisy":
        assert tuple(g["noise_shape"]) == (len(r["cluster_chan"]), g["noise_Z"].shape[1])


@pytest.mark.parametrize("i", range(8))
def test_waveform_window_gate_matches_reference(golden, i):
    """Digitisation windows cut from the ungated starts: exact and one-ulp-inside edges, single-start windows, lower
    edges inside long pulse trains (an excluded start does not move the scan on)."""
    g = golden("waveform_gate.npz")
    cfg = _wf_cfg(g)
    uch, tab = g["uch"], g["tdc0_tab"]
    lut = lambda lab: tab[np.searchsorted(uch, lab)]                     # noqa: E731
    r = O.synthesize(g["chan"], g["time"], g["charge"], lut, g["template"], cfg, 12.55, tuple(g["windows"][i]), None)
    for k in ("chan", "start", "tdc0", "starttdc", "volt", "adc"):
        assert_same(r[k], g[f"w{i}_{k}"], f"w{i}.{k}")
    assert len(r["chan"]) > 0


def _geom(g, tag):
    G = SimpleNamespace(**{k: g[f"{tag}_G_{k}"] for k in ("sector", "layer", "counter_in_type", "x", "y", "pos",
                                                           "length_dir", "sector_type", "pos_side0", "pos_side1",
                                                           "sipms_side0", "sipms_side1")})
    G.sector_names = [str(s) for s in g[f"{tag}_G_sector_names"]]
    return G


def _finder(g, tag):
    cuts = {}
    for name, row in zip(_geom(g, tag).sector_names, g[f"{tag}_cuts"]):
        cuts[name] = CF.SectorCuts(*[int(v) if i == 6 else float(v) for i, v in enumerate(row)])
    return CF.FinderConfig(cuts=cuts)


@pytest.mark.parametrize("tag", ["module", "two", "eight"])
def test_coincidences_match_reference(golden, tag):
    g = golden("coinc.npz")
    G, cfg, status = _geom(g, tag), _finder(g, tag), g[f"{tag}_status"]
    P = {k: g[f"{tag}_in_{k}"] for k in ("ev", "idx", "bar", "sipm", "time", "pe", "seq")}
    got = {k: [] for k in ("ev", "type", "pe", "start", "end", "slope", "avgtime", "poscalc", "pos", "sidepe",
                           "sidetime", "sidehits", "nlayers")}
    mem_cl, mem_idx = [], []
    for e in np.unique(P["ev"]):
        m = P["ev"] == e
        for r in O.find_event({k: P[k][m] for k in ("idx", "bar", "sipm", "time", "pe", "seq")}, G, status, cfg):
            n = len(got["ev"])
            got["ev"].append(e); got["type"].append(r["sectortype"]); got["pe"].append(r["pe"])
            got["start"].append(r["start"]); got["end"].append(r["end"]); got["slope"].append(r["slope"])
            got["avgtime"].append(r["avgtime"]); got["poscalc"].append(r["poscalc"]); got["pos"].append(r["pos"])
            got["sidepe"].append(r["sidepe"]); got["sidetime"].append(r["sidetime"])
            got["sidehits"].append(r["sidehits"]); got["nlayers"].append(len(r["layers"]))
            mem_cl += [n] * len(r["pulses"]); mem_idx += list(r["pulses"])
    for k, v in got.items():
        ref = g[f"{tag}_scalar_{k}"]
        v = np.asarray(v, float).reshape(ref.shape) if k == "pos" else np.asarray(v)
        assert_same(v, ref, f"{tag}.{k}")
    assert_same(mem_cl, g[f"{tag}_scalar_mem_cl"], "mem_cl")
    assert_same(mem_idx, g[f"{tag}_scalar_mem_idx"], "mem_idx")
    assert len(got["ev"]) > 0


def attach_case(g, i):
    """Geometry, finder configuration, status and pulses of case i of the reference's attachment tests."""
    import json
    tag = f"a{i}"
    G = _geom(g, tag)
    cuts = {str(n): CF.SectorCuts(*[int(v) if j == 6 else float(v) for j, v in enumerate(row)])
            for n, row in zip(g[f"{tag}_cut_names"], g[f"{tag}_cuts"])}
    flags = json.loads(str(g[f"{tag}_flags"]))
    flags["compensate_status_bits"] = tuple(flags["compensate_status_bits"])
    P = {k: g[f"{tag}_in_{k}"] for k in ("idx", "bar", "sipm", "time", "pe", "seq")}
    return G, CF.FinderConfig(cuts=cuts, **flags), g[f"{tag}_status"], P


def test_coincidences_match_the_reference_attachment_cases(golden):
    """The reference's own boundary cases (strict windows, ties, order, flags; every find_event call of
    crv/tests/test_coinc_attachment_cpu.py): same clusters, members and properties."""
    g = golden("attach.npz")
    n = int(g["n"])
    assert n >= 20
    for i in range(n):
        G, cfg, status, P = attach_case(g, i)
        rows = O.find_event(P, G, status, cfg)
        tag = f"a{i}_scalar_"
        assert len(rows) == len(g[tag + "pe"]), i
        for c, r in enumerate(rows):
            assert list(r["pulses"]) == list(g[tag + "mem_idx"][g[tag + "mem_cl"] == c]), i
            for k in ("pe", "start", "end", "slope", "avgtime"):
                assert_same(np.asarray(r[k]), g[tag + k][c], f"a{i}.{k}")
            assert list(r["sidehits"]) == list(g[tag + "sidehits"][c]), i


def test_pulsefit_matches_the_references_own_tests(golden):
    """Every reconstruct call of the reference's own pulse-fit tests (crv/tests/test_reco_pulsefit.py: 200 injected
    single pulses, a pulse below threshold, a pedestal undershoot; 12.5 ns), replayed: the reference's outputs."""
    g = golden("pulsetests.npz")
    period = float(g["period"][0])
    assert int(g["n"]) == 3
    for i in range(int(g["n"])):
        tag = f"r{i}"
        args = [g[f"{tag}_{k}"] for k in ("adc", "n", "start", "ped", "area", "height")]
        r = O.reconstruct(*args, CF.RecoConfig(period=period), period)
        keys = [k[len(tag) + 5:] for k in g.files if k.startswith(f"{tag}_out_")]
        assert set(keys) == set(r)
        for k in keys:
            assert_same(r[k], g[f"{tag}_out_{k}"], f"{tag}.{k}")


def test_chain_glue_matches_the_references_own_tests(golden):
    """crv/tests/test_chain.py replayed (make_golden.py chaintests): reco waveforms from digis are identical
    (concatenation of continuing digis, (event, channel, start) order, calibration per channel); TDC0 is one draw per
    (event, FEB) in both FEB-key modes: the keyed draws partition the labels exactly as the reference's draws do."""
    g = golden("chaintests.npz")
    for i in range(int(g["nw"])):
        D = {k: g[f"w{i}_{k}"] for k in ("chan", "starttdc", "adc")}
        cond = SimpleNamespace(**{k: g[f"w{i}_cond_{k}"] for k in ("pedestal", "pulsearea", "pulseheight",
                                                                    "timeoffset", "roc", "feb")})
        W = O.reco_waveforms(D, cond)
        keys = [k[len(f"w{i}_out_"):] for k in g.files if k.startswith(f"w{i}_out_")]
        assert set(W) == set(keys)
        for k in keys:
            assert_same(W[k], g[f"w{i}_out_{k}"], f"w{i}.{k}")
    for i in range(int(g["nt"])):
        labels, ref = g[f"t{i}_labels"], g[f"t{i}_out"]
        cond = SimpleNamespace(roc=g[f"t{i}_cond_roc"], feb=g[f"t{i}_cond_feb"])
        width, key = float(g[f"t{i}_width"][0]), str(g[f"t{i}_key"])
        t = O.tdc0_of_labels(labels, cond, 9, width, key, lambda e: np.zeros(len(e), np.int64))
        _, a = np.unique(t, return_inverse=True)
        _, b = np.unique(ref, return_inverse=True)
        pairs = set(zip(a.ravel().tolist(), b.ravel().tolist()))
        assert len(pairs) == len(set(a.ravel().tolist())) == len(set(b.ravel().tolist())), (i, key)
        assert np.all((t >= 0) & (t < width))


def test_pulse_configuration_wiring_matches_the_references_own_tests(golden):
    """crv/tests/test_chain_config_wiring.py and test_chain_reco_contract.py replayed (make_golden.py wiring): with the
    default, a custom and a no-offset RecoConfig, 12- and 36-sample waveforms, status-masked channels, explicit
    offsets, ten pulses in one waveform and no waveforms at all, the oracle's pulses (reconstruct_full +
    filter_channels + DB offsets x scale, chain.py:317-323) sorted as chain.clusters sorts them equal the reference's
    pulse table."""
    import json
    from dataclasses import fields
    g = golden("wiring.npz")
    period = float(g["period"][0])
    ours = {f.name for f in fields(CF.RecoConfig)}
    total = 0
    for i in range(int(g["n"])):
        ref_cfg = json.loads(str(g[f"r{i}_reco"]))
        assert set(ref_cfg) <= ours, set(ref_cfg) - ours
        rcfg = CF.RecoConfig(**{**ref_cfg, "period": period})
        W = {k[len(f"r{i}_W_"):]: g[k] for k in g.files if k.startswith(f"r{i}_W_")}
        cond = SimpleNamespace(status=g[f"r{i}_cond_status"], timeoffset=g[f"r{i}_cond_timeoffset"])
        if "toff" not in W:
            W["toff"] = cond.timeoffset[W["bar"] * 4 + W["sipm"]]
        P = O.pulses_from_waveforms(W, cond, rcfg, period)
        o = np.lexsort((P["seq"], P["wf"], W["ev"][P["wf"]]))
        wf = P["wf"][o]
        got = dict(ev=W["ev"][wf], bar=W["bar"][wf], sipm=W["sipm"][wf], seq=P["seq"][o], pe=P["pe"][o],
                   time=P["time"][o])
        for k, v in got.items():
            assert_same(v, g[f"r{i}_P_{k}"], f"r{i}.{k}")
        total += len(wf)
    assert total > 20


def test_pulsefit_matches_the_references_normal_cache_batches(golden):
    """crv/tests/test_pulsefit_normal_cache.py replayed (make_golden.py pulsecache; 12.5 ns): its edge batch (flat
    waveform, saturated prefix, pedestal undershoot, short valid length) and synthetic batch give the reference's
    reconstruct_full outputs."""
    g = golden("pulsecache.npz")
    period = float(g["period"][0])
    cfg = CF.RecoConfig(period=period)
    for i in range(int(g["n"])):
        args = [g[f"r{i}_{k}"] for k in ("adc", "n", "start", "ped", "area", "height")]
        r = O.reconstruct_full(*args, cfg, period)
        keys = [k[len(f"r{i}_out_"):] for k in g.files if k.startswith(f"r{i}_out_")]
        assert set(keys) == set(r)
        for k in keys:
            assert_same(r[k], g[f"r{i}_out_{k}"], f"r{i}.{k}")
