"""The drop-in chain's host glue on the CPU: chain.reco_waveforms (crv/crvfastsim/chain.py:273-286) on digis made by
the oracle equals the oracle's reco_waveforms, for digis in the order chain.digis returns them and shuffled."""
import numpy as np

from oracle import oracle as O
from tests.helpers import workload


def _digis():
    from crvgpu import waveform as W
    from crvgpu.config import WaveformConfig
    geom, cond, cfg, steps = workload(48, seed=9)
    Q, _ = O.charges(steps, geom, cond, cfg.response, cfg.sipm, 13, cfg.window[1])
    wc = cfg.waveform or WaveformConfig()
    tmpl = W.single_pe_template(wc)
    run_of = lambda keys: np.zeros(len(np.asarray(keys).ravel()), np.int64)  # noqa: E731
    tdc0 = lambda labels: O.tdc0_of_labels(labels, cond, 13, wc.period, cfg.feb_phase_key, run_of)  # noqa: E731
    return O.synthesize(Q["chan"], Q["time"], Q["charge"], tdc0, tmpl, wc, wc.period, cfg.window, None), cond


def test_reco_waveforms_matches_the_oracle_in_either_order():
    from crvgpu import chain as CH
    D, cond = _digis()
    assert len(D["chan"]) > 50
    ref = O.reco_waveforms(D, cond)
    perm = np.random.default_rng(2).permutation(len(D["chan"]))
    for DD in (D, {k: np.asarray(v)[perm] for k, v in D.items() if k in ("chan", "start", "tdc0", "starttdc", "volt",
                                                                           "adc")}):
        W = CH.reco_waveforms(DD, cond)
        for k in ("ev", "bar", "sipm", "adc", "n", "start", "ped", "area", "height"):
            assert np.array_equal(np.asarray(W[k]), np.asarray(ref[k])), k


def test_concat_waveforms_matches_the_reference_fixture_and_the_oracle(golden):
    """pulsefit.concat_waveforms (crv/crvfastsim/reco/pulsefit.py:319-345): the engine's host grouping equals the
    reference's output on the committed fixture, and the oracle's on digis of one length (the row-copy path, with
    continued waveforms of up to five digis) and of mixed lengths."""
    from crvgpu.pulsefit import concat_waveforms as C
    g = golden("concat.npz")
    for got, k in zip(C(g["key"], g["bar"], g["sipm"], g["tdc"], g["flat"], g["lens"]),
                      ("gid", "mat", "n", "start", "first")):
        assert np.array_equal(got, g[k]), k
    rng = np.random.default_rng(5)
    nd, L = 4000, 12
    key = np.sort(rng.integers(0, 300, nd))
    ch = rng.integers(0, 8, nd)
    o = np.lexsort((ch, key))
    key, ch = key[o], ch[o]
    tdc = rng.integers(0, 10 ** 6, nd)
    for i in range(1, nd):
        if rng.random() < 0.3 and ch[i] == ch[i - 1] and key[i] == key[i - 1]:
            tdc[i] = tdc[i - 1] + L
    for lens in (np.full(nd, L, np.int64), rng.integers(1, 20, nd)):
        flat = rng.integers(-100, 4096, int(lens.sum()))
        ref = O.concat_waveforms(key, ch // 4, ch % 4, tdc, flat, lens)
        got = C(key, ch // 4, ch % 4, tdc, flat, lens)
        for a, b in zip(got, ref):
            assert a.dtype == b.dtype and np.array_equal(a, b)
        assert int(ref[2].max()) > L
    assert all(len(v) == 0 for v in C(key[:0], ch[:0], ch[:0], tdc[:0], np.zeros(0, np.int64), np.zeros(0, np.int64)))
