"""The keyed CPU restatement of the stochastic stages against the reference's own known-answer tests and statistics
(crv/tests/test_photons.py:82-104; reference SiPM/photon-count statistics in tests/golden/stats.npz)."""
from dataclasses import replace

import numpy as np
import ctypes

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
