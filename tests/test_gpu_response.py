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
