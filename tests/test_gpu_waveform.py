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
    for k in ("chan", "start", "tdc0", "starttdc", "volt", "adc", "cluster_chan", "cluster_tstart", "cluster_keep"):
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


@pytest.mark.parametrize("form", ["callable", "array", "batched"])
def test_synthesize_dropin_equals_the_references_outputs(golden, tmp_path, form):
    """waveform.synthesize with the caller's TDC0 (callable or array over labels, and batches of whole clusters) on the
    reference's own fixture: every digi field and the per-cluster outputs equal the reference's bit for bit."""
    from crvgpu import waveform as W
    from crvgpu.config import WaveformConfig
    g = golden("waveform.npz")
    spe = tmp_path / "spe.txt"
    np.savetxt(spe, np.c_[g["traw"], g["vraw"]], fmt="%.17g")
    cfg = WaveformConfig(min_voltage=float(g["min_voltage"][0]), single_pe_stretch=float(g["stretch"][0]),
                         single_pe_file=str(spe))
    assert np.array_equal(W.single_pe_template(cfg), g["template"])
    uch, tab = g["uch"], g["tdc0_tab"]
    calls = []

    def lut(lab):
        calls.append(len(lab))
        return tab[np.searchsorted(uch, lab)]
    if form == "array":
        dense = np.full(int(uch.max()) + 1, np.nan)
        dense[uch] = tab
        tdc0 = dense
    else:
        tdc0 = lut
    kw = {"max_charges": 1000} if form == "batched" else {}
    r = W.synthesize(g["chan"], g["time"], g["charge"], tdc0, cfg, tuple(g["window"]), None, **kw)
    for k in ("chan", "start", "tdc0", "starttdc", "volt", "adc", "cluster_chan", "cluster_tstart", "cluster_keep"):
        a, b = np.asarray(r[k]), np.asarray(g[f"clean_{k}"])
        assert a.shape == b.shape and a.dtype.kind == b.dtype.kind, (k, a.shape, b.shape, a.dtype, b.dtype)
        assert np.array_equal(a, b), k
    if form == "batched":
        assert len(calls) > 5 and sum(calls) == len(g["clean_cluster_chan"])


def test_tdc0_per_feb_is_the_digis_draw_and_groups_by_feb():
    """chain.tdc0_per_feb: the keyed TDC0 the digis use (oracle bit for bit), one value per (event, ROC, FEB) or
    (event, FEB), in [0, width); the reference's ValueErrors for a bad width or key."""
    from crvgpu import chain as CH
    geom, cond, cfg, steps = workload(16, seed=3)
    ev = np.unique((np.asarray(steps["subrun"], np.int64) << 20) | np.asarray(steps["event"], np.int64))
    labels = (ev[:, None] * 32768 + np.arange(0, 4 * geom.nbars, 3)[None, :]).ravel()
    runs = {int(k): 1 for k in ev}
    run_of = lambda keys: np.ones(len(np.asarray(keys).ravel()), np.int64)  # noqa: E731
    for key, width in (("roc_feb", 12.55), ("feb", 6.0)):
        t = CH.tdc0_per_feb(labels, cond, None, width, key, seed=77, runs=runs)
        to = O.tdc0_of_labels(labels, cond, 77, width, key, run_of)
        assert np.array_equal(t, to)
        assert np.all((t >= 0) & (t < width))
        ch = labels % 32768
        feb = cond.feb[ch] if key == "feb" else cond.roc[ch] * 1000 + cond.feb[ch]
        grp = (labels // 32768) * 1_000_000 + feb
        for gk in np.unique(grp)[:50]:
            assert len(np.unique(t[grp == gk])) == 1
    for bad in (dict(width=13.0), dict(width=float("nan")), dict(key="roc")):
        with pytest.raises(ValueError):
            CH.tdc0_per_feb(labels, cond, None, **{"width": 12.0, "key": "roc_feb", **bad}, seed=1)
