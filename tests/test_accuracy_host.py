"""Host logic of the FP32-vs-FP64 error report (crvgpu.accuracy): nearest-time matching within a key."""
import numpy as np

from crvgpu.accuracy import match_nearest


def brute(ka, ta, kb, tb, tol):
    pairs = sorted((abs(ta[i] - tb[j]), i, j) for i in range(len(ka)) for j in range(len(kb))
                   if ka[i] == kb[j] and abs(ta[i] - tb[j]) <= tol)
    out = np.full(len(ka), -1)
    used = set()
    for _, i, j in pairs:
        if out[i] < 0 and j not in used:
            out[i] = j
            used.add(j)
    return out


def test_match_nearest_equals_greedy_brute_force():
    rng = np.random.default_rng(1)
    for trial in range(40):
        na, nb = rng.integers(0, 60, 2)
        ka, kb = rng.integers(0, 6, na), rng.integers(0, 6, nb)
        ta, tb = rng.uniform(0, 200, na), rng.uniform(0, 200, nb)
        # the chain's pulses of one SiPM are far apart: keep that property (no two items of a side within 3 tol)
        def spread(k, t):
            o = np.lexsort((t, k))
            t = t.copy()
            t[o] = np.where(np.r_[True, k[o][1:] != k[o][:-1]], 0, 7.0).cumsum() + np.arange(len(t))[np.argsort(o)] * 0
            return t + rng.uniform(-0.5, 0.5, len(t))
        ta, tb = spread(ka, ta), spread(kb, tb)
        got = match_nearest(ka, ta, kb, tb, 2.0)
        assert np.array_equal(got, brute(ka, ta, kb, tb, 2.0)), trial


def test_match_nearest_empty_sides():
    assert match_nearest(np.zeros(0), np.zeros(0), np.arange(3), np.arange(3.0), 1).shape == (0,)
    assert (match_nearest(np.arange(3), np.arange(3.0), np.zeros(0), np.zeros(0), 1) == -1).all()
