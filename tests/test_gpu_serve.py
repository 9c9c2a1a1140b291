"""Serving loop on the GPU: a job's clusters are the same alone, in a mix of concurrent jobs (other slots, other
knobs, overlapping on the device) and through a plain ChainEngine run of the same design point; different knobs give
different results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pool(n_events, seed=21):
    from crvgpu import geometry as GM
    from crvgpu.response import upload_steps
    geom = GM.module_geometry()
    cond = GM.default_conditions(geom)
    steps = GM.synthetic_steps(n_events, geom, seed=seed)
    return geom, cond, upload_steps(steps, nbars=geom.nbars)


def _same(a, b):
    assert set(a) == set(b)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_job_results_are_identical_alone_and_in_the_mix():
    from crvgpu.serve import Job, ServeEngine
    geom, cond, pool = _pool(4096)
    srv = ServeEngine(geom, cond, pool, hbm_budget=1 << 40, max_slots=3, chunk_events=1024)
    assert len(srv.slots) == 3
    jobs = [Job(0, 1500, first=100, seed=11, yield_per_mev=35.0, lambda_long=4000.0, threshold_pe=4.0, window_ns=12.0),
            Job(1, 2500, first=1200, seed=12, yield_per_mev=48.0, lambda_long=6000.0, threshold_pe=6.0, window_ns=8.0),
            Job(2, 800, first=3000, seed=13)]
    alone = [srv.run([j], realtime=False)[0] for j in jobs]
    mixed = srv.run(jobs, realtime=False)
    assert len({r.slot for r in mixed}) > 1                 # the mix really ran on several slots
    for a, m in zip(alone, mixed):
        assert a.n_clusters > 0
        _same(a.clusters, m.clusters)
    # a different design point of the same events changes the result
    j0b = Job(0, 1500, first=100, seed=11, yield_per_mev=45.0, lambda_long=4000.0, threshold_pe=4.0, window_ns=12.0)
    other = srv.run([j0b], realtime=False)[0]
    assert other.n_clusters != alone[0].n_clusters or not np.array_equal(other.clusters["pe"],
                                                                           alone[0].clusters["pe"])


def test_serve_job_matches_a_direct_chain_run():
    import torch
    from crvgpu.chain import ChainEngine
    from crvgpu.serve import Job, ServeEngine, job_config, slice_events
    geom, cond, pool = _pool(3000, seed=22)
    job = Job(0, 2000, first=500, seed=5, yield_per_mev=33.0, threshold_pe=7.0, window_ns=18.0)
    srv = ServeEngine(geom, cond, pool, hbm_budget=1 << 40, max_slots=1, chunk_events=512)
    got = srv.run([job], realtime=False)[0]
    eng = ChainEngine(geom, cond, job_config(job, "fp32", srv.sector))
    r = eng.run(slice_events(pool, job.first, job.first + job.n_events), job.seed)
    ref = {k: v.cpu().numpy() for k, v in r.clusters.items()}
    torch.cuda.synchronize()
    _same(got.clusters, ref)


def test_serving_modes_agree():
    """Per-stage slots and resident slots (one or two concurrent) give the same clusters."""
    from crvgpu.serve import Job, ServeEngine
    geom, cond, pool = _pool(2048, seed=23)
    jobs = [Job(0, 900, first=10, seed=3, window_ns=15.0), Job(1, 700, first=1000, seed=4, threshold_pe=6.0),
            Job(2, 300, first=1500, seed=4, yield_per_mev=45.0)]
    outs = []
    for kw in (dict(resident=False), dict(resident=True), dict(resident=True, max_slots=2)):
        kw.setdefault("max_slots", 1)
        srv = ServeEngine(geom, cond, pool, hbm_budget=1 << 40, chunk_events=512, **kw)
        outs.append(srv.run(jobs, realtime=False))
    # deadline scheduling changes the order chunks run in, not the results
    outs.append(srv.run(jobs, realtime=False, policy="edf", iso_rate=1e5))
    outs.append(srv.run(jobs, realtime=False, policy="slowdown", iso_table={1000: 0.01, 100000: 0.5}))
    with pytest.raises(ValueError):
        srv.run(jobs, realtime=False, policy="edf")
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert a.n_clusters > 0
            _same(a.clusters, b.clusters)


def test_lookup_model_jobs_alone_in_the_mix_and_direct():
    """Serving with the lookup-table photon model (the production call's tables, crv/crvfastsim/chain.py:197-213):
    each job's clusters are the same alone, in the mix, and through a direct resident lookup chain of its design
    point over the same events."""
    import torch
    from crvgpu import chain as CH
    from crvgpu.lookup import LookupModel
    from crvgpu.resident import ChainCaps, ResidentChain
    from crvgpu.response import upload_steps
    from crvgpu.serve import Job, ServeEngine, job_config, slice_events
    from tests.helpers import module_lookup
    geom, cond, tables, lcfg, steps, pdg = module_lookup(600, seed=5)
    pool = upload_steps(steps, nbars=geom.nbars)
    assert pool.order is None
    model = LookupModel(geom, lcfg, tables, cond.deviation, precision="fp32")
    cols = model.upload_steps(steps, pdg)
    srv = ServeEngine(geom, cond, pool, hbm_budget=1 << 40, max_slots=2, chunk_events=128, lookup=model,
                      lookup_config=lcfg, lookup_steps=cols)
    jobs = [Job(0, 300, first=10, seed=31, threshold_pe=4.0, window_ns=12.0),
            Job(1, 250, first=320, seed=32, threshold_pe=6.0, window_ns=8.0),
            Job(2, 100, first=200, seed=33)]
    alone = [srv.run([j], realtime=False)[0] for j in jobs]
    mixed = srv.run(jobs, realtime=False)
    assert alone[0].n_clusters > 0 and alone[1].n_clusters > 0
    for a, m in zip(alone, mixed):
        _same(a.clusters, m.clusters)
    # a direct resident lookup chain over the job's chunks (the lookup model keys its draws by the step's row in the
    # batch, as the stage API's rows, so the comparison takes the serving chunks)
    j = jobs[0]
    eng = CH.ChainEngine(geom, cond, job_config(j, "fp32", srv.sector, lcfg), G=srv.G)
    caps = ChainCaps(events=128, steps=8192, photons=4096, charges=4096, slots=4096, digis=4096, pulses=4096,
                     max_steps_per_event=64)
    rc = ResidentChain(eng, caps, real_dtype=pool.x.dtype, graph=False, grow=True, max_grow=12, lookup=model)
    parts = []
    for a in range(j.first, j.first + j.n_events, 128):
        ds, lk = slice_events(pool, a, min(a + 128, j.first + j.n_events), cols)
        parts.append({k: v.cpu().numpy() for k, v in rc.run(ds, j.seed, lookup_steps=lk).clusters.items()})
    direct = {k: np.concatenate([q[k] for q in parts]) for k in parts[0]}
    _same(alone[0].clusters, direct)
    torch.cuda.synchronize()
