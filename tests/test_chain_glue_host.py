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
