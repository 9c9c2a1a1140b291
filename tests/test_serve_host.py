"""Serving loop host logic (CPU): the job generator draws the workload's knob ranges and Poisson arrivals; design
points map onto the engine configuration; latency statistics."""
import numpy as np
import pytest


def test_random_jobs_follow_the_workload_ranges():
    from crvgpu.serve import random_jobs
    jobs = random_jobs(2000, np.random.default_rng(3), pool_events=2_000_000, rate=4.0)
    ev = np.array([j.n_events for j in jobs])
    assert ev.min() >= 1000 and ev.max() <= 1_000_000
    assert 0.3 < np.mean(np.log10(ev) < 4.5) < 0.7               # log-uniform over three decades
    for name, lo, hi in (("yield_per_mev", 30, 50), ("lambda_long", 3500, 6500), ("threshold_pe", 3, 8),
                         ("window_ns", 5, 20)):
        v = np.array([getattr(j, name) for j in jobs])
        assert v.min() >= lo and v.max() <= hi
    arr = np.array([j.arrival for j in jobs])
    gaps = np.diff(arr)
    assert np.all(gaps >= 0) and abs(gaps.mean() - 0.25) < 0.03 and abs(gaps.std() - 0.25) < 0.04
    assert all(j.first + j.n_events <= 2_000_000 for j in jobs)


def test_job_config_maps_the_knobs():
    from crvgpu.config import SPE_PEAK_VOLT
    from crvgpu.serve import Job, job_config
    c = job_config(Job(0, 10, yield_per_mev=33.0, lambda_long=4200.0, threshold_pe=6.5, window_ns=17.0), "fp64")
    assert c.response.yield_per_mev == 33.0 and c.response.lambda_long == 4200.0
    assert c.waveform.min_voltage == pytest.approx(6.5 * SPE_PEAK_VOLT)
    assert c.finder.cuts["EX"].max_dt == 17.0 and c.finder.cuts["EX"].coincidence_layers == 3
    assert c.precision == "fp64"


def test_latency_stats():
    from crvgpu.serve import JobResult, latency_stats
    rs = [JobResult(i, 1000 * (i + 1), {}, 0, arrival=float(i), start=float(i), finish=float(i) + 0.5 * (i + 1),
                    slot=0) for i in range(10)]
    st = latency_stats(rs, iso_rate=4000.0)
    assert st["jobs"] == 10 and st["p50_s"] == pytest.approx(np.percentile([0.5 * (i + 1) for i in range(10)], 50))
    assert st["p99_over_isolated"] == pytest.approx(2.0)
    assert st["events_per_s"] == pytest.approx(55000 / 14.0)
