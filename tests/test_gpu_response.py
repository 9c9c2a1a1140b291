"""GPU response stage (photons -> SiPM charges) against the CPU oracle.

FP64: bit-exact (same keyed Philox draws, same exp/log steps and roundings).  FP32-mixed: statistical agreement and
integer outputs equal except for draws within float resolution of their thresholds.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import run_of, workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R():
    from crvgpu import response
    return response


def test_photons_stage_bit_exact(R):
    geom, cond, cfg, steps = workload(40, seed=1)
    s, c, t, k = R.make_photons(steps, None, geom, cfg.response, None, cond.deviation, None, key=77)
    so, co, to, ko = O.make_photons(steps, geom, cfg.response, cond.deviation, 77)
    assert len(t) == len(to) > 1000
    assert np.array_equal(s, so) and np.array_equal(c, co) and np.array_equal(k, ko)
    assert np.array_equal(t, to)


def test_charges_fp64_bit_exact(R):
    geom, cond, cfg, steps = workload(64, seed=2)
    cond.status[[5, 17, 100, 201]] = [1, 4, 2, 5]       # masked (bits 0, 2) and unmasked (bit 1) channels
    Q = R.charges(steps, None, geom, cond, cfg, None, key=1234)
    Qo, diag = O.charges(steps, geom, cond, cfg.response, cfg.sipm, 1234, cfg.window[1])
    assert diag["status"] == 0
    assert len(Q["time"]) == len(Qo["time"]) > 1000
    for k in ("chan", "time", "charge", "pe", "photon"):
        assert np.array_equal(Q[k], Qo[k]), k
    masked = {5, 17, 201}
    assert not np.isin(Q["chan"] % 32768, list(masked)).any()


def test_sipm_stage_bit_exact_and_fired_pixels(R):
    geom, cond, cfg, steps = workload(24, seed=3)
    so, co, to, ko = O.make_photons(steps, geom, cfg.response, cond.deviation, 5)
    evk = (np.asarray(steps["subrun"], np.int64) << 20) | np.asarray(steps["event"], np.int64)
    label = evk[so] * 32768 + co
    run = np.asarray(steps["run"], np.int64)[so]
    G = R.simulate(label, to, so, None, cfg.sipm, None, t_end=cfg.window[1], key=5, draw_key=ko, run=run)
    rof = run_of(steps)
    Qo, u, nq, nfp, st = O.sipm_groups(label, to, so, ko, lambda L: rof(L // 32768), cfg.sipm, 5, cfg.window[1])
    assert st == 0
    for k in ("chan", "time", "charge", "pe", "photon"):
        assert np.array_equal(G[k], Qo[k]), k
    assert np.array_equal(G["_group_labels"], u)
    assert np.array_equal(G["_group_fired"], nfp)
    assert np.array_equal(G["_group_charges"], nq)


def test_charges_fp32_mixed_statistics(R):
    geom, cond, cfg, steps = workload(200, seed=4)
    Q64 = R.charges(steps, None, geom, cond, cfg, None, key=9)
    cfg.precision = "fp32"
    Q32 = R.charges(steps, None, geom, cond, cfg, None, key=9)
    n64, n32 = len(Q64["pe"]), len(Q32["pe"])
    assert abs(n32 / n64 - 1) < 4 / np.sqrt(n64)
    assert abs(Q32["pe"].sum() / Q64["pe"].sum() - 1) < 4 / np.sqrt(n64)
    # same SiPMs are hit
    assert np.array_equal(np.unique(Q64["chan"]), np.unique(Q32["chan"]))


def test_large_photon_counts_take_the_second_pass(R):
    """A SiPM with more photons than the first pass's shared-memory capacity is simulated by the large-capacity pass
    and still matches the oracle."""
    geom, cond, cfg, steps = workload(4, seed=6, mean_steps=400.0)
    Q = R.charges(steps, None, geom, cond, cfg, None, key=3)
    Qo, diag = O.charges(steps, geom, cond, cfg.response, cfg.sipm, 3, cfg.window[1])
    counts = np.bincount(np.unique(diag["photon_label"], return_inverse=True)[1])
    assert counts.max() > 512
    for k in ("chan", "time", "charge", "pe", "photon"):
        assert np.array_equal(Q[k], Qo[k]), k


def _lrint_photons(S=600, seed=12):
    """Photons on S SiPMs (Poisson 60 each, spread over 1.5 us) with draw keys = index within the SiPM."""
    rng = np.random.default_rng(seed)
    n = rng.poisson(60, S)
    label = np.repeat((1 << 20 | 3) * 32768 + np.arange(S, dtype=np.int64), n)
    t = np.repeat(rng.uniform(0, 1500, S), n) + rng.exponential(7.4, len(label))
    key = np.arange(len(label)) - np.repeat(np.cumsum(n) - n, n)
    return label, t, np.arange(len(label)), key


@pytest.mark.parametrize("edge", [False, True])
def test_sipm_lrint_bit_exact_and_fired_pixels(R, golden, edge):
    """pixel_id "lrint" on a photon map with content in bins 6-33 and (39, 39) (pixel 40 reached, cross-talk from
    it), or with content only at (39, 39); cross-talk and afterpulses on: GPU == oracle, fired pixels included."""
    from dataclasses import replace
    from crvgpu.config import SiPMConfig
    pmap = golden("pixelid.npz")["pmap"].copy()
    if edge:
        pmap[:] = 0.0
        pmap[39, 39] = 1.0
    sc = replace(SiPMConfig(pixel_id="lrint"), cross_talk=0.05, trap0_prob=0.02)
    label, t, photon, key = _lrint_photons()
    G = R.simulate(label, t, photon, pmap, sc, None, t_end=1606.4, key=21, draw_key=key)
    Qo, u, nq, nfp, st = O.sipm_groups(label, t, photon, key, lambda L: np.zeros(len(L), np.int64), sc, 21, 1606.4,
                                       pmap)
    assert st == 0 and len(Qo["pe"]) > 5000
    for k in ("chan", "time", "charge", "pe", "photon"):
        assert np.array_equal(G[k], Qo[k]), k
    assert np.array_equal(G["_group_fired"], nfp) and np.array_equal(G["_group_charges"], nq)


def test_charges_lrint_bit_exact(R):
    """The chain's charges under pixel_id "lrint" (uniform photon map): GPU == oracle."""
    from dataclasses import replace
    geom, cond, cfg, steps = workload(48, seed=5)
    cfg.sipm = replace(cfg.sipm, pixel_id="lrint")
    Q = R.charges(steps, None, geom, cond, cfg, None, key=4321)
    Qo, diag = O.charges(steps, geom, cond, cfg.response, cfg.sipm, 4321, cfg.window[1])
    assert diag["status"] == 0 and len(Q["time"]) > 1000
    for k in ("chan", "time", "charge", "pe", "photon"):
        assert np.array_equal(Q[k], Qo[k]), k
    cfg.sipm = replace(cfg.sipm, pixel_id="truncate")
    Qt = R.charges(steps, None, geom, cond, cfg, None, key=4321)
    assert len(Qt["time"]) != len(Q["time"]) or not np.array_equal(Qt["pe"], Q["pe"])
