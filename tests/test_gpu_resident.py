"""The resident chain (one crv_chain call per batch, replayed as a CUDA graph) gives the same clusters, bit for bit, as
the per-stage ChainEngine on the same steps and seed; batches of other sizes replay the same graph; a batch that
overflows a capacity is rejected with the sizes it needed, and with growth enabled it is re-run to the same result."""
import pytest

from tests.helpers import workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    from crvgpu import chain as CH
    from crvgpu.config import ChainConfig
    from crvgpu.response import upload_steps
    from dataclasses import replace
    geom, cond, cfg, steps = workload(600, seed=31)
    cond.status[[5, 41, 90]] = [2, 1, 4]
    cfg32 = replace(cfg, precision="fp32")
    ds = upload_steps(steps, nbars=geom.nbars)
    assert isinstance(cfg32, ChainConfig)
    return geom, cond, cfg32, ds, CH


def _trial_caps(eng, ds):
    """Capacities from a trial batch run with ample capacities."""
    from crvgpu.resident import ChainCaps, ResidentChain
    big = ChainCaps(events=ds.nevents, steps=ds.nsteps, photons=400 * ds.nsteps + 4096, charges=200 * ds.nsteps + 4096,
                    slots=100 * ds.nsteps + 4096, digis=100 * ds.nsteps + 4096, pulses=100 * ds.nsteps + 4096,
                    max_steps_per_event=max(1, ds.max_steps))
    rc = ResidentChain(eng, big, graph=False)
    rc.run(ds, 7)
    return ChainCaps.from_counts(rc.last_counts, ds.nevents, ds.nsteps, ds.max_steps, margin=1.3)


def _same(res, ref):
    import torch
    assert res.counts["clusters"] == ref.n_clusters and res.counts["members"] == ref.n_members
    for k, v in ref.clusters.items():
        assert torch.equal(res.clusters[k], v), k
    for k, v in ref.members.items():
        assert torch.equal(res.members[k], v), k


@pytest.mark.parametrize("graph", [True, False])
def test_resident_chain_matches_the_stage_engine(setup, graph):
    geom, cond, cfg, ds, CH = setup
    from crvgpu.resident import ResidentChain
    eng = CH.ChainEngine(geom, cond, cfg)
    ref = eng.run(ds, 2024)
    rc = ResidentChain(eng, _trial_caps(eng, ds), graph=graph)
    res = rc.run(ds, 2024)
    assert ref.n_clusters > 0
    c = res.counts
    assert (c["charges"], c["digis"], c["waveforms"], c["pulses"], c["hits"]) == \
        (ref.n_charges, ref.n_digis, ref.n_waveforms, ref.n_pulses, ref.n_hits)
    _same(res, ref)
    assert rc.launches_per_run > 20
    # a second batch through the same graph (replay) and another seed (captured again)
    _same(rc.run(ds, 2024), ref)
    _same(rc.run(ds, 99), eng.run(ds, 99))


def test_smaller_batches_replay_the_same_graph(setup):
    geom, cond, cfg, ds, CH = setup
    from crvgpu.resident import ResidentChain
    from crvgpu.serve import slice_events
    eng = CH.ChainEngine(geom, cond, cfg)
    rc = ResidentChain(eng, _trial_caps(eng, ds), graph=True)
    rc.run(ds, 5)
    g = rc._graph
    for a, b in ((0, 250), (250, 600), (100, 101), (37, 400)):
        part = slice_events(ds, a, b)
        _same(rc.run(part, 5), eng.run(part, 5))
    assert rc._graph is g                                       # no capture after the first batch


def test_capacity_overflow_rejects_the_batch_and_growth_recovers(setup):
    geom, cond, cfg, ds, CH = setup
    from dataclasses import replace
    from crvgpu import _capi
    from crvgpu.resident import BatchRejected, ResidentChain
    eng = CH.ChainEngine(geom, cond, cfg)
    ref = eng.run(ds, 3)
    caps = _trial_caps(eng, ds)
    for field, need in (("pulses", "PULSES_OUT"), ("digis", "DIGIS_OUT"), ("charges", "CHARGES_OUT"),
                        ("photons", "PHOTONS_TOTAL"), ("slots", "DIGIS")):
        small = replace(caps, **{field: 64})
        rc = ResidentChain(eng, small, graph=True)
        with pytest.raises(BatchRejected) as ei:
            rc.run(ds, 3)
        assert ei.value.flags == _capi.ST_CAPACITY
        assert ei.value.need[_capi.NEED[need]] > 64, field
        grown = ResidentChain(eng, small, graph=True, grow=True)
        _same(grown.run(ds, 3), ref)
        assert getattr(grown.caps, field) > 64
    # more steps per event than the capacity: rejected on the host before any launch
    rc = ResidentChain(eng, replace(caps, max_steps_per_event=1), graph=True)
    with pytest.raises(ValueError):
        rc.run(ds, 3)


def test_fp64_resident_chain_matches(setup):
    geom, cond, cfg, ds, CH = setup
    from dataclasses import replace
    from crvgpu.resident import ResidentChain
    from crvgpu.serve import slice_events
    eng = CH.ChainEngine(geom, cond, replace(cfg, precision="fp64"))
    part = slice_events(ds, 0, 200)
    rc = ResidentChain(eng, _trial_caps(eng, part), graph=True)
    _same(rc.run(part, 11), eng.run(part, 11))


def test_empty_batch_and_step_capacity_growth(setup):
    """A batch without events gives no clusters through the same graph; a batch with more steps than the capacity
    grows it on the host when growth is on (and is refused otherwise) before anything runs."""
    geom, cond, cfg, ds, CH = setup
    from dataclasses import replace
    from crvgpu.resident import ResidentChain
    from crvgpu.serve import slice_events
    eng = CH.ChainEngine(geom, cond, cfg)
    caps = _trial_caps(eng, ds)
    rc = ResidentChain(eng, caps, graph=True)
    r = rc.run(slice_events(ds, 5, 5), 4)
    assert r.n_events == 0 and all(v == 0 for v in r.counts.values())
    _same(rc.run(ds, 4), eng.run(ds, 4))                  # the graph is still good after the empty batch
    small = replace(caps, steps=ds.nsteps // 2)
    with pytest.raises(ValueError):
        ResidentChain(eng, small, graph=True).run(ds, 4)
    grown = ResidentChain(eng, small, graph=True, grow=True)
    _same(grown.run(ds, 4), eng.run(ds, 4))
    assert grown.caps.steps >= ds.nsteps


def test_one_graph_serves_every_design_point(setup):
    """A captured chain graph takes a new seed and new serving knobs (yield, attenuation length, threshold and the
    finder window, the last through the finder tables updated in place) without a new capture, and every design point
    equals the per-stage engine run at that point; a change beyond the knobs captures again."""
    from dataclasses import replace
    from crvgpu.resident import ResidentChain
    from crvgpu.serve import Job, job_config
    geom, cond, cfg, ds, CH = setup
    from crvgpu.geometry import sector_geom
    sector = str(sector_geom(geom).sector_names[0])
    jobs = [Job(0, 1, yield_per_mev=40.0, lambda_long=5000.0, threshold_pe=5.0, window_ns=10.0, seed=11),
            Job(1, 1, yield_per_mev=31.0, lambda_long=3600.0, threshold_pe=7.5, window_ns=18.0, seed=12),
            Job(2, 1, yield_per_mev=48.5, lambda_long=6400.0, threshold_pe=3.2, window_ns=5.5, seed=13)]
    heavy = job_config(Job(9, 1, yield_per_mev=50.0, lambda_long=6500.0, threshold_pe=3.0, window_ns=20.0), "fp32",
                       sector)
    caps = _trial_caps(CH.ChainEngine(geom, cond, heavy), ds)          # room for every design point below
    eng = CH.ChainEngine(geom, cond, job_config(jobs[0], "fp32", sector))
    rc = ResidentChain(eng, caps, graph=True, grow=True)
    for j in jobs:
        c = job_config(j, "fp32", sector)
        rc.configure(c)
        res = rc.run(ds, j.seed)
        ref = CH.ChainEngine(geom, cond, c).run(ds, j.seed)
        _same(res, ref)
    assert rc.captures == 1 and rc.replays == len(jobs)
    # noise off is not a serving knob: the graph is captured again, and still right
    c = replace(job_config(jobs[1], "fp32", sector), noise=False)
    rc.configure(c)
    _same(rc.run(ds, 5), CH.ChainEngine(geom, cond, c).run(ds, 5))
    assert rc.captures == 2


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_lookup_model_inside_the_resident_chain(precision):
    """The resident chain with the lookup-table photon model (crv_chain_lookup; chain.charges with lookup tables,
    crv/crvfastsim/chain.py:197-213) gives, bit for bit, the clusters of the stage path: chain.charges with the same
    tables and seed, then the per-stage engine from those charges.  One graph serves a second seed and a second batch
    (the lookup kernels take the seed from the graph's parameter block)."""
    import numpy as np
    import torch
    from crvgpu import chain as CH
    from crvgpu.config import ChainConfig
    from crvgpu.lookup import LookupModel
    from crvgpu.resident import ChainCaps, ResidentChain
    from crvgpu.response import upload_steps
    from tests.helpers import module_lookup
    geom, cond, tables, lcfg, steps, pdg = module_lookup(300, seed=4)
    cond.status[[6, 44, 91]] = [1, 4, 2]                    # absent and no data (dropped), compensated (kept)
    cfg = ChainConfig(lookup=lcfg, precision=precision)
    ds = upload_steps(steps, nbars=geom.nbars)
    model = LookupModel(geom, lcfg, tables, cond.deviation, precision=precision)
    cols = model.upload_steps(steps, pdg)
    eng = CH.ChainEngine(geom, cond, cfg)
    caps = ChainCaps(events=ds.nevents, steps=ds.nsteps, photons=1024, charges=1024, slots=1024, digis=1024,
                     pulses=1024, max_steps_per_event=max(1, ds.max_steps))
    rc = ResidentChain(eng, caps, real_dtype=torch.float64, graph=True, grow=True, max_grow=8, lookup=model)
    caps_before = None
    for seed in (77, 78):
        if seed == 78:
            caps_before = rc.captures
        Q = CH.charges(steps, None, geom, cond, cfg, None, key=seed, tabs=tables, pdg=pdg)
        assert len(Q["time"]) > 10000
        dq = {"label": torch.from_numpy(np.asarray(Q["chan"], np.int64)).cuda(),
              **{k: torch.from_numpy(np.ascontiguousarray(Q[k])).cuda() for k in ("time", "charge", "pe", "photon")}}
        ref = eng.run(ds, seed, charges=dq)
        res = rc.run(ds, seed, lookup_steps=cols)
        assert ref.n_clusters > 0
        c = res.counts
        assert (c["charges"], c["digis"], c["waveforms"], c["pulses"], c["hits"]) == \
            (len(Q["time"]), ref.n_digis, ref.n_waveforms, ref.n_pulses, ref.n_hits)
        _same(res, ref)
        _same(rc.run(ds, seed, lookup_steps=cols), ref)      # the same graph again
    assert rc.captures == caps_before                       # the second seed needed no new capture
