"""Multi-rank path on the CPU: two gloo ranks each run the oracle chain on their event range; the merged cluster
table equals the single-process run over all events (keyed draws make the result independent of the split)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from crvgpu import shard


def test_event_ranges_cover_and_balance():
    for n, w in ((10, 3), (1 << 20, 8), (5, 8), (0, 2)):
        rs = [shard.event_range(n, w, r) for r in range(w)]
        assert rs[0][0] == 0 and rs[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(rs[:-1], rs[1:]))
        sizes = [b - a for a, b in rs]
        assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.event_range(10, 2, 2)


def _steps(n):
    from crvgpu import geometry as GM
    return GM.synthetic_steps(n, GM.module_geometry(), seed=3)


def _chain(steps):
    from oracle import oracle as O
    from crvgpu import config as CF, geometry as GM, waveform as WV
    geom = GM.module_geometry()
    cond = GM.default_conditions(geom)
    cfg = CF.ChainConfig()
    G = GM.sector_geom(geom)
    Q, _ = O.charges(steps, geom, cond, cfg.response, cfg.sipm, 9, cfg.window[1])
    wc = CF.WaveformConfig()
    run_of = lambda keys: np.ones(len(np.asarray(keys).ravel()), np.int64)  # noqa: E731
    tdc0 = lambda labels: O.tdc0_of_labels(labels, cond, 9, wc.period, "roc_feb", run_of)  # noqa: E731
    D = O.synthesize(Q["chan"], Q["time"], Q["charge"], tdc0, WV.single_pe_template(wc), wc, wc.period, cfg.window,
                     O.keyed_noise(9, run_of))
    W = O.reco_waveforms(D, cond)
    rc = CF.RecoConfig()
    P = O.pulses_from_waveforms(W, cond, rc, rc.period)
    out = O.clusters_from_pulses(W, P, G, cond.status, CF.workload_finder(G.sector_names))
    return {k: out[k] for k in ("cl_event", "cl_pe", "cl_avgtime", "mem_cl", "mem_idx")}


def _rank(rank, world, port, n_events, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # every rank sees the same step table and processes the rows of its event range
    a, b = shard.event_range(n_events, world, rank)
    steps = _steps(n_events)
    ev = np.asarray(steps["event"])
    parts = [None] * world
    local = _chain(steps.rows((ev >= a) & (ev < b))) if b > a else {}
    dist.all_gather_object(parts, local)
    if rank == 0:
        q.put(shard.merge_tables(parts))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_gloo_matches_single_process():
    n = 96
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # one process over all events at once
    whole = _chain(_steps(n))
    assert set(merged) == set(whole)
    for k in merged:
        assert np.array_equal(merged[k], whole[k]), k
    assert len(merged["cl_event"]) > 0                  # the comparison covers real clusters
