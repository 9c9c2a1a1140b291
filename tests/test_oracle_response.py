"""The keyed CPU restatement of the stochastic stages against the reference's own known-answer tests and statistics
(crv/tests/test_photons.py:82-104; reference SiPM/photon-count statistics in tests/golden/stats.npz; pixel ids of both
rules in tests/golden/pixelid.npz)."""
from dataclasses import replace

import numpy as np
import ctypes

import pytest

from crvgpu import config as CF
from oracle import oracle as O


def sipm(chan, time, sc, seed=1, t_end=1e5, pmap=None):
    photon = np.arange(len(chan))
    key = np.zeros(len(chan), np.int64)
    # draw key: index of the photon within its SiPM
    o = np.argsort(chan, kind="stable")
    u, st, cnt = np.unique(chan[o], return_index=True, return_counts=True)
    key[o] = np.arange(len(chan)) - np.repeat(st, cnt)
    Q, lab, nq, nfp, status = O.sipm_groups(chan, time, photon, key, lambda L: np.zeros(len(L), np.int64), sc, seed,
                                            t_end, pmap)
    assert status == 0
    return Q


def test_single_photons_give_full_pe_and_the_crosstalk_rate():
    sc = replace(CF.SiPMConfig(), cross_talk=0.04, trap0_prob=0.0)
    n = 200_000
    Q = sipm(np.arange(n, dtype=np.int64), np.zeros(n), sc)
    assert np.allclose(Q["pe"], 1.0)
    p = O.p_fire(sc, sc.overvoltage)
    live = 1 - 0.1 * 0.1
    ct = 4 * (1 - (1 - sc.cross_talk) ** 0.25)
    assert abs(len(Q["pe"]) / n - p * live * (1 + ct)) < 0.004


def test_recovery_reduces_a_second_firing():
    sc = replace(CF.SiPMConfig(), cross_talk=0.0, trap0_prob=0.0)
    pmap = np.zeros((40, 40)); pmap[5, 5] = 1.0
    n = 50_000
    Q = sipm(np.repeat(np.arange(n, dtype=np.int64), 2), np.tile([0.0, 1.0], n), sc, pmap=pmap)
    late = Q["pe"][Q["time"] == 1.0]
    v1 = 1 - np.exp(-1 / sc.time_constant)
    assert np.isclose(late.min(), v1) and np.isclose(late.max(), 1.0)


def test_sipm_statistics_match_the_reference(golden):
    g = golden("stats.npz")
    sc = replace(CF.SiPMConfig(), cross_talk=0.05, trap0_prob=0.02)
    rng = np.random.default_rng(int(g["sipm_tspread_seed"][0]))
    S = int(g["sipm_S"][0])
    n = g["sipm_n"]
    chan = np.repeat(np.arange(S, dtype=np.int64), n)
    t = np.repeat(rng.uniform(0, 1500, S), n) + rng.exponential(7.4, len(chan))
    Q = sipm(chan, t, sc, seed=5, t_end=1606.4)
    nph = len(chan)
    ref_pe, ref_q, ref_low = float(g["sipm_pe_sum"][0]), int(g["sipm_charges"][0]), float(g["sipm_frac_low"][0])
    # PE and charge counts per photon within 4 / sqrt(n) (the reference's JAX-twin tolerance)
    tol = 4 / np.sqrt(ref_q)
    assert abs(Q["pe"].sum() / ref_pe - 1) < tol
    assert abs(len(Q["pe"]) / ref_q - 1) < tol
    assert abs((Q["pe"] < 0.99).mean() - ref_low) < 0.003
    assert nph == int(g["sipm_nphot"][0])


def test_photon_count_rule_matches_the_reference_distribution(golden):
    g = golden("stats.npz")
    L = O.lib()
    for m in (0.5, 3.0, 9.9, 10.1, 40.0, 200.0):
        n = 200_000
        avg = np.full(n, m)
        cnt = np.empty(n, np.int64)
        L.orc_counts_from_mean(ctypes.c_uint32(7), ctypes.c_int64(n), O._p(avg), O._p(cnt))
        ref_mean, ref_var = g[f"count_{m}"]
        se = np.sqrt(ref_var / n)
        assert abs(cnt.mean() - ref_mean) < 6 * se + 1e-9, (m, cnt.mean(), ref_mean)
        assert abs(cnt.var() / ref_var - 1) < 0.03, (m, cnt.var(), ref_var)


def test_keyed_draws_do_not_depend_on_batching():
    """Events processed alone give the same charges as inside a batch."""
    from tests.helpers import workload
    geom, cond, cfg, steps = workload(12, seed=3)
    Q, _ = O.charges(steps, geom, cond, cfg.response, cfg.sipm, 99, cfg.window[1])
    ev = np.asarray(steps["event"])
    e = int(ev[len(ev) // 2])
    sub = steps.rows(ev == e)
    Q1, _ = O.charges(sub, geom, cond, cfg.response, cfg.sipm, 99, cfg.window[1])
    m = (Q["chan"] // 32768) == ((1 << 20) | e)
    for k in ("chan", "time", "charge", "pe"):
        assert np.array_equal(Q[k][m], Q1[k])


def test_photon_delays_are_sorted_exponential_order_statistics():
    """Each (step, SiPM) row's emission delays come out in key order, and the normalised spacings
    (t_j - t_(j-1)) * (n - j) / decay_time of every row are i.i.d. Exp(1) (Renyi's representation), so the row holds
    the same distribution as the reference's n independent exponential delays (photons.py:163-224) sorted."""
    from scipy import stats
    from tests.helpers import workload
    geom, cond, cfg, steps = workload(40, seed=5)
    step, chan, t, key = O.make_photons(steps, geom, cfg.response, np.zeros(len(steps["event"])), 17)
    row = step * 8 + (chan % 4)
    o = np.lexsort((key, row))
    row, t, key = row[o], t[o], key[o]
    first = np.r_[True, row[1:] != row[:-1]]
    start = np.maximum.accumulate(np.where(first, np.arange(len(row)), 0))
    j = np.arange(len(row)) - start
    assert np.array_equal(j, key & 0xFFFF)
    n = np.bincount(np.cumsum(first) - 1)[np.cumsum(first) - 1]
    dt = np.diff(t)[~first[1:]]
    assert (dt >= 0).all()
    x = dt * (n[1:][~first[1:]] - j[1:][~first[1:]]) / cfg.response.decay_time
    assert len(x) > 20_000
    assert stats.kstest(x, "expon").pvalue > 1e-3


def _pix_cfg(pid, **kw):
    return replace(CF.SiPMConfig(pixel_id=pid), **kw)


@pytest.mark.parametrize("pid", ["truncate", "lrint"])
def test_pixel_ids_follow_the_reference_histogram(golden, pid):
    """Pixel ids x * 41 + y drawn from a map with content in bins 6-33 and (39, 39): same support as the reference's
    draw (lrint reaches pixel 40 only from bin 39), frequencies within a two-sample chi-square bound."""
    g = golden("pixelid.npz")
    ref = g[f"hist_{pid}"].astype(float)
    pix = O.sipm_pixels(np.arange(400_000), _pix_cfg(pid, inactive=()), 3, pmap=g["pmap"])
    ours = np.bincount(pix, minlength=41 * 41).astype(float)
    assert ours[ref == 0].sum() == 0 and ref[ours == 0].sum() == 0
    m = (ref + ours) > 0
    chi2 = ((ours[m] - ref[m]) ** 2 / (ours[m] + ref[m])).sum()
    dof = m.sum() - 1
    assert chi2 < dof + 6 * np.sqrt(2 * dof), (chi2, dof)


def test_lrint_is_the_bin_or_the_next_pixel(golden):
    """The same draws under both rules: lrint moves to the next pixel in x and in y each with probability 1/2, and
    from a map with content in bins 6-33 reaches pixel 34, which has no content (crv/tests/test_sipm_pixel_id.py:21-31
    states these properties of the reference's draw)."""
    pmap = golden("pixelid.npz")["pmap"].copy()
    pmap[39, 39] = 0.0
    keys = np.arange(200_000)
    t = O.sipm_pixels(keys, _pix_cfg("truncate", inactive=()), 11, pmap=pmap)
    lr = O.sipm_pixels(keys, _pix_cfg("lrint", inactive=()), 11, pmap=pmap)
    tx, ty, lx, ly = t // 41, t % 41, lr // 41, lr % 41
    assert tx.min() == 6 and tx.max() == 33 and ty.min() == 6 and ty.max() == 33
    assert np.all(pmap[tx, ty] > 0)
    dx, dy = lx - tx, ly - ty
    assert set(np.unique(dx)) == {0, 1} and set(np.unique(dy)) == {0, 1}
    assert abs((dx == 0).mean() - 0.5) < 0.01 and abs(((dx == 0) & (dy == 0)).mean() - 0.25) < 0.01
    assert lx.max() == 34 and ly.max() == 34


def test_dead_pixels_apply_to_the_rounded_pixel():
    """A photon whose bin is live but whose lrint pixel is dead is lost (the dead table is over pixel ids)."""
    pmap = np.zeros((40, 40))
    pmap[17, 17] = 1.0                                   # next to the dead 18..21 block
    keys = np.arange(20_000)
    pix = O.sipm_pixels(keys, _pix_cfg("lrint"), 2, pmap=pmap)
    assert abs((pix == -1).mean() - 0.25) < 0.02         # (18, 18) is dead
    assert set(np.unique(pix[pix >= 0])) == {17 * 41 + 17, 17 * 41 + 18, 18 * 41 + 17}


def test_crowded_sipms_saturate_like_the_reference(golden):
    """400 photons at once on each of 400 SiPMs, no cross-talk: PE per SiPM of both rules within 0.5 % of the
    reference's, and truncation saturates more (fewer distinct pixels)."""
    g = golden("pixelid.npz")
    pe = {}
    chan = np.repeat(np.arange(400, dtype=np.int64), 400)
    for pid in ("truncate", "lrint"):
        Q = sipm(chan, np.zeros(len(chan)), _pix_cfg(pid, cross_talk=0.0, trap0_prob=0.0), seed=8, pmap=g["pmap"])
        pe[pid] = Q["pe"].sum() / 400
        ref = float(g[f"crowded_pe_{pid}"][0])
        assert abs(pe[pid] / ref - 1) < 0.005, (pid, pe[pid], ref)
    assert pe["truncate"] < pe["lrint"] * 0.99


def test_lrint_charge_statistics_match_the_reference(golden):
    """Cross-talk 0.05 and afterpulses 0.02 under lrint on the 6-33 map: charges and PE per photon within 4 / sqrt(n),
    low-PE fraction within 0.003."""
    g = golden("pixelid.npz")
    trng = np.random.default_rng(int(g["lrint_seed"][0]))
    S = int(g["lrint_S"][0])
    n = trng.poisson(80, S)
    chan = np.repeat(np.arange(S, dtype=np.int64), n)
    t = np.repeat(trng.uniform(0, 1500, S), n) + trng.exponential(7.4, len(chan))
    Q = sipm(chan, t, _pix_cfg("lrint", cross_talk=0.05, trap0_prob=0.02), seed=6, t_end=1606.4, pmap=g["pmap"])
    ref_q, ref_pe = int(g["lrint_charges"][0]), float(g["lrint_pe_sum"][0])
    tol = 4 / np.sqrt(ref_q)
    assert abs(len(Q["pe"]) / ref_q - 1) < tol
    assert abs(Q["pe"].sum() / ref_pe - 1) < tol
    assert abs((Q["pe"] < 0.99).mean() - float(g["lrint_frac_low"][0])) < 0.003
