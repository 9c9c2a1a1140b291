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


def test_changed_labels_finds_every_kind_of_difference():
    from crvgpu.accuracy import changed_labels
    l64 = np.array([1, 1, 2, 3, 3, 3, 5])
    t64 = np.array([1.0, 2.0, 5.0, 1.0, 2.0, 3.0, 9.0])
    q64 = np.ones(7)
    l32 = np.array([1, 1, 2, 3, 3, 4])            # 3 lost a charge, 4 new, 5 missing
    t32 = np.array([1.0, 2.0005, 5.5, 1.0, 2.0, 7.0])   # 1 within tolerance, 2 moved by 0.5 ns
    q32 = np.ones(6)
    assert changed_labels(l64, t64, q64, l32, t32, q32).tolist() == [2, 3, 4, 5]
    q32b = q32.copy()
    q32b[0] = 1.01
    assert 1 in changed_labels(l64, t64, q64, l32, t32, q32b)
