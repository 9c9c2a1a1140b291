"""GPU waveform synthesis + zero suppression (digis) against the oracle (FP64 bit-exact: ADC samples, volts, starts,
TDCs), with and without keyed noise; FP32-mixed ADC mismatches confined to quantisation boundaries."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import workload

pytestmark = pytest.mark.gpu


def oracle_digis(Q, cond, cfg, seed, runs, noise=True):
    from crvgpu import waveform as W
    from crvgpu.config import WaveformConfig
    wc = cfg.waveform or WaveformConfig()
    tmpl = W.single_pe_template(wc)
    run_of = lambda keys: np.array([runs.get(int(k), 0) for k in np.asarray(keys).ravel()], np.int64)  # noqa: E731
    width = wc.period if cfg.feb_phase_width is None else cfg.feb_phase_width
    tdc0 = lambda labels: O.tdc0_of_labels(labels, cond, seed, width, cfg.feb_phase_key, run_of)  # noqa: E731
    nz = O.keyed_noise(seed, run_of) if noise else None
    return O.synthesize(Q["chan"], Q["time"], Q["charge"], tdc0, tmpl, wc, wc.period, cfg.window, nz)


@pytest.fixture(scope="module")
def charges():
    from crvgpu import response as R
    geom, cond, cfg, steps = workload(96, seed=7)
    Q = R.charges(steps, None, geom, cond, cfg, None, key=31)
    return geom, cond, cfg, steps, Q


@pytest.mark.parametrize("noise", [False, True])
def test_digis_fp64_bit_exact(charges, noise):
    from crvgpu import waveform as W
    geom, cond, cfg, steps, Q = charges
    cfg.noise = noise
    runs = {(1 << 20) | int(e): 1 for e in np.unique(steps["event"])}
    D = W.digis(Q, cond, cfg, None, key=55, geom=geom, runs=runs)
    Do = oracle_digis(Q, cond, cfg, 55, runs, noise)
    assert len(D["chan"]) == len(Do["chan"]) > 100
    for k in ("chan", "start", "tdc0", "starttdc", "volt", "adc"):
        assert np.array_equal(D[k], Do[k]), k


def test_digis_fp32_adc_mismatch_at_quantisation_boundaries(charges):
    from crvgpu import waveform as W
    geom, cond, cfg, steps, Q = charges
    cfg.noise = False
    runs = {(1 << 20) | int(e): 1 for e in np.unique(steps["event"])}
    D64 = W.digis(Q, cond, cfg, None, key=55, geom=geom, runs=runs)
    cfg.precision = "fp32"
    D32 = W.digis(Q, cond, cfg, None, key=55, geom=geom, runs=runs)
    cfg.precision = "fp64"
    assert np.array_equal(D64["chan"], D32["chan"]) and np.array_equal(D64["starttdc"], D32["starttdc"])
    diff = D64["adc"].astype(int) - D32["adc"].astype(int)
    # FP32 moves a sample by float rounding only: across an ADC step, or across a 0.5 ns template-grid step of one
    # contribution; either changes the sample by at most one count
    assert np.abs(diff).max() <= 1
    rate = (diff != 0).mean()
    print(f"FP32 ADC mismatch rate {rate:.2e} of {diff.size} samples")
    assert rate < 5e-3


def gate_windows(starts, chan, train_label=50000):
    """Digitisation windows cut from ungated digi starts: exact and one-ulp-inside edges, single-start windows, lower
    edges inside long pulse trains (labels >= train_label)."""
    S = np.unique(starts)
    q = lambda f: float(S[int(f * (len(S) - 1))])                        # noqa: E731
    first = np.array([starts[chan == c].min() for c in np.unique(chan[chan >= train_label])])
    P = 12.55
    return [(q(0.2), q(0.8)), (np.nextafter(q(0.2), np.inf), np.nextafter(q(0.8), -np.inf)),
            (q(0.5), np.nextafter(q(0.5), np.inf)), (np.nextafter(q(0.5), -np.inf), q(0.5)),
            (float(np.median(first)) + 5.5 * P, 1500.0), (float(first.min()) + 13.0 * P, float(first.max()) + 30.25 * P),
            (200.0, 1500.0)]


def test_digis_window_gate_bit_exact(golden):
    """The window gate of the ZS scan on long pulse trains (an excluded start does not move the scan on; both bounds
    inclusive): GPU digis equal the oracle's under windows cut from the ungated starts."""
    from crvgpu import waveform as W
    from crvgpu.config import CHAN_MULT, ChainConfig, WaveformConfig
    from crvgpu.geometry import default_conditions, module_geometry
    g = golden("waveform_gate.npz")
    Q = {"chan": g["chan"], "time": g["time"], "charge": g["charge"]}
    wc = WaveformConfig(min_voltage=float(g["min_voltage"][0]), single_pe_stretch=float(g["stretch"][0]))
    nb = int((Q["chan"] % CHAN_MULT).max()) // 4 + 1
    geom = module_geometry(n_modules=(nb + 63) // 64)
    cond = default_conditions(geom)

    def both(window):
        cfg = ChainConfig(waveform=wc, window=window, noise=False)
        return W.digis(Q, cond, cfg, None, key=77, geom=geom), oracle_digis(Q, cond, cfg, 77, {}, noise=False)

    D, Do = both((-1e5, 1e5))
    windows = gate_windows(Do["start"], Do["chan"])
    for w in [None] + windows:
        if w is not None:
            D, Do = both(w)
        assert len(Do["chan"]) > 0
        for k in ("chan", "start", "tdc0", "starttdc", "volt", "adc"):
            assert np.array_equal(D[k], Do[k]), (w, k)
