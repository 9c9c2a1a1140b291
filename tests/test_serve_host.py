"""Serving loop host logic (CPU): the job generator draws the workload's knob ranges and Poisson arrivals; design
points map onto the engine configuration; latency statistics; the scheduler (chunking, shortest-remaining-first and
earliest-deadline picks, late arrivals joining at the next chunk, results joined in event order) over simulated slots."""
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


@pytest.fixture
def host_torch(monkeypatch):
    """The serving loop's torch handle without the engine's CUDA-device gate (the fake slots below run no kernels)."""
    import torch
    from crvgpu import serve
    monkeypatch.setattr(serve, "_torch", lambda: torch)


class _FakeServe:
    """ServeEngine's scheduler and result assembly over slots whose chunk work is simulated on the host: a chunk of
    events [a, b) takes `per_event` seconds per event and yields a cluster column with one entry per event."""

    def __new__(cls, n_slots, chunk, per_event=2e-6, express=False):
        import time
        import torch
        from crvgpu.serve import ServeEngine, _Slot

        class Fake(ServeEngine):
            def _run_chunk(self, slot, job, a, b):
                time.sleep(per_event * (b - a))
                self.log.append((job.id, a, b, slot.index, time.perf_counter()))
                return {"pe": torch.arange(a, b, dtype=torch.float64), "event": torch.full((b - a,), job.id)}

        eng = object.__new__(Fake)
        eng.chunk = chunk
        eng.slots = [_Slot(i, None, None) for i in range(n_slots)]
        if express:
            eng.slots.append(_Slot(n_slots, None, None, express=True))
        eng.log = []
        return eng


def test_serving_results_join_chunks_in_event_order(host_torch):
    from crvgpu.serve import Job
    srv = _FakeServe(3, 100, per_event=3e-5)                  # 3 ms per chunk: every slot thread is up by then
    jobs = [Job(0, 950, first=10), Job(1, 40, first=5000), Job(2, 301, first=700)]
    res = srv.run(jobs, realtime=False)
    assert [r.id for r in res] == [0, 1, 2]
    for j, r in zip(jobs, res):
        assert np.array_equal(r.clusters["pe"], np.arange(j.first, j.first + j.n_events))
        assert r.n_clusters == j.n_events and r.finish >= r.start
    assert len(srv.log) == 10 + 1 + 4                          # chunks of at most 100 events
    assert len({s for *_, s, _ in srv.log}) > 1                # the burst ran on several slots


def test_srpt_serves_small_jobs_first_and_late_arrivals_at_the_next_chunk(host_torch):
    from crvgpu.serve import Job
    srv = _FakeServe(1, 50, per_event=1e-4)                    # 5 ms per 50-event chunk, 200 ms for the big job
    big, small = Job(0, 2000, first=0), Job(1, 100, first=5000, arrival=0.05)
    res = srv.run([big, small], realtime=True)
    # the small job arrives while the big one runs and is served at the next chunk boundary, before the big one ends
    assert res[1].finish < res[0].finish
    order = [jid for jid, *_ in srv.log]
    first_small = order.index(1)
    assert 0 < first_small < order.count(0) and order[first_small:first_small + 2] == [1, 1]


def test_deadline_scheduling_orders_by_deadline(host_torch):
    from crvgpu.serve import Job
    srv = _FakeServe(1, 50, per_event=1e-6)
    # all at once: earliest deadline = arrival + 2 x isolated time, so the smallest job first, as SRPT
    jobs = [Job(0, 400), Job(1, 50), Job(2, 200)]
    srv.run(jobs, realtime=False, policy="edf", iso_rate=1e6)
    firsts = []
    for jid, *_ in srv.log:
        if jid not in firsts:
            firsts.append(jid)
    assert firsts == [1, 2, 0]
    with pytest.raises(ValueError):
        srv.run(jobs, realtime=False, policy="fifo")
    with pytest.raises(ValueError):
        srv.run(jobs, realtime=False, policy="edf")             # needs the isolated rate


def test_isolated_time_interpolates_the_measured_sizes():
    from crvgpu.serve import JobResult, isolated_time, latency_stats
    table = {1000: 0.010, 10000: 0.040, 100000: 0.340}
    assert np.isclose(isolated_time(table, 1000), 0.010) and np.isclose(isolated_time(table, 55000), 0.19)
    assert np.isclose(isolated_time(table, 200000), 0.340 + 100000 * 0.3 / 90000)
    rs = [JobResult(i, n, {}, 0, 0.0, 0.0, 2 * float(isolated_time(table, n)), 0) for i, n in
          enumerate([1000, 5000, 20000, 100000])]
    st = latency_stats(rs, iso_table=table)
    assert np.isclose(st["p99_over_isolated"], 2.0) and st["slowdown_by_size"]["1000-10000"]["jobs"] == 2


def test_slowdown_policy_needs_isolated_times():
    from crvgpu.serve import ServeEngine
    srv = ServeEngine.__new__(ServeEngine)
    with pytest.raises(ValueError, match="isolated run times"):
        srv.run([], policy="slowdown")
    with pytest.raises(ValueError, match="unknown scheduling policy"):
        srv.run([], policy="fifo")


def test_slowdown_policy_serves_a_small_late_job_before_a_long_wait_grows(host_torch):
    from crvgpu.serve import Job
    srv = _FakeServe(1, 50, per_event=1e-6)
    jobs = [Job(0, 400), Job(1, 50), Job(2, 200)]
    res = srv.run(jobs, realtime=False, policy="slowdown", iso_table={50: 50e-6, 400: 400e-6})
    assert [r.id for r in res] == [0, 1, 2] and all(r.finish >= r.start for r in res)
    firsts = []
    for jid, *_ in srv.log:
        if jid not in firsts:
            firsts.append(jid)
    assert sorted(firsts) == [0, 1, 2]


def test_express_slot_takes_one_chunk_jobs_and_nothing_else(host_torch):
    from crvgpu.serve import Job
    srv = _FakeServe(2, 50, per_event=1e-4, express=True)       # 5 ms per 50-event chunk
    big = Job(0, 2000, first=0)
    small = [Job(1 + i, 30, first=5000 + 100 * i, arrival=0.01 + 0.015 * i) for i in range(4)]
    res = srv.run([big] + small, realtime=True)
    for jid, a, b, slot, _ in srv.log:
        if jid == 0:
            assert slot in (0, 1)                                # multi-chunk work stays on the normal slots
        else:
            assert slot == 2                                     # one-chunk jobs on the idle express slot
    assert all(r.finish < res[0].finish for r in res[1:])
    for j, r in zip([big] + small, res):
        assert np.array_equal(r.clusters["pe"], np.arange(j.first, j.first + j.n_events))
