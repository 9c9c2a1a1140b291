"""The finder's FP32 rejection before its FP64 link test (csrc/crv_coinc.cuh, linked_fast and the greedy clustering's
cluster range test) must never reject a pair that the FP64 test links: restated here in NumPy float32 (both with and
without a fused multiply-add in the bound) on times drawn around the window edge, at magnitudes up to 1e5 ns."""
import numpy as np


def trunc32(x):
    """FP64 -> FP32 by truncating the mantissa (the kernels' d2f_trunc for normal FP32 magnitudes)."""
    x = np.asarray(x, np.float64)
    b = x.view(np.uint64)
    e = ((b >> 52) & 0x7FF).astype(np.int64)
    ok = (e >= 897) & (e <= 1150)
    u = (((b >> 32) & 0x80000000) | ((e - 896).astype(np.uint64) << 23) | ((b >> 29) & 0x7FFFFF)).astype(np.uint32)
    out = u.view(np.float32).copy()
    out[~ok] = x[~ok].astype(np.float32)
    return out


def bound(tc, tb, mt_hi, fused):
    s = np.abs(tc) + np.abs(tb) + mt_hi
    if fused:                                   # one rounding: the product and the sum in FP64, then to FP32
        return (np.float64(np.float32(4.8e-7)) * s.astype(np.float64) + mt_hi.astype(np.float64)).astype(np.float32)
    return (np.float32(4.8e-7) * s + mt_hi).astype(np.float32)


def test_fp32_rejection_never_drops_a_link():
    rng = np.random.default_rng(5)
    n = 2_000_000
    for scale in (10.0, 2000.0, 1e5):
        max_dt = rng.uniform(1.0, 30.0, n)
        ta = rng.uniform(-scale, scale, n)
        # differences concentrated within a few ulps of the window edge, and uniform ones
        edge = max_dt * (1.0 + rng.normal(0.0, 1e-6, n)) * rng.choice([-1.0, 1.0], n)
        d = np.where(rng.random(n) < 0.7, edge, rng.uniform(-3 * max_dt, 3 * max_dt))
        tb = ta + d
        linked64 = np.abs(ta - tb) < max_dt
        mt_hi = trunc32(max_dt)
        tc, tm = trunc32(ta), trunc32(tb)
        diff = np.abs(tc - tm).astype(np.float32)
        for fused in (False, True):
            reject = diff > bound(tc, tm, mt_hi, fused)
            assert not np.any(reject & linked64), (scale, fused, int(np.sum(reject & linked64)))
            far = np.abs(ta - tb) > 1.01 * max_dt              # and it rejects the pairs clearly beyond the window
            assert np.mean(reject[far]) > 0.999, (scale, fused)
        # the cluster range test: a candidate beyond [lo, hi] by the bound at the largest member magnitude
        lo = np.minimum(tm, tm - np.abs(rng.normal(0, 1, n)).astype(np.float32))
        hi = tm
        big = np.maximum(np.abs(lo), np.abs(hi))
        for fused in (False, True):
            mg = bound(tc, big, mt_hi, fused)
            skip = ((tc - hi).astype(np.float32) > mg) | ((lo - tc).astype(np.float32) > mg)
            assert not np.any(skip & linked64), (scale, fused)
