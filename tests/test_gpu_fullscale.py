"""Full-scale detector (5,504 counters in 86 modules of five bar lengths, Poisson(60) steps plus 0.5 noise steps per
counter per event): charges bit-exact with the oracle, and coincidences on events with thousands of finder hits (the
finder's global-memory pass) identical to the oracle's, event by event."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def full_run():
    from crvgpu import chain as CH
    from crvgpu import config as CF
    from crvgpu import geometry as GM
    from crvgpu.response import upload_steps
    geom = GM.module_geometry(86)
    cond = GM.default_conditions(geom)
    cfg = CF.ChainConfig()
    steps = GM.synthetic_steps(2, geom, seed=31, mean_steps=60.0, noise_per_counter=0.5)
    eng = CH.ChainEngine(geom, cond, cfg)
    res = eng.run(upload_steps(steps, nbars=geom.nbars), seed=77, keep=True)
    return geom, cond, cfg, steps, eng, res, GM.sector_geom(geom)


def host(t):
    return t.cpu().numpy()


def test_fullscale_charges_bit_exact(full_run):
    geom, cond, cfg, steps, eng, res, G = full_run
    assert len(steps["bar"]) > 5000
    Qo, _ = O.charges(steps, geom, cond, cfg.response, cfg.sipm, 77, cfg.window[1])
    R = res.charges
    for k, o in (("label", "chan"), ("time", "time"), ("charge", "charge"), ("pe", "pe")):
        assert np.array_equal(host(getattr(R, k)), Qo[o]), k


def test_fullscale_coincidences_on_large_events(full_run):
    from crvgpu import config as CF
    geom, cond, cfg, steps, eng, res, G = full_run
    H = {k: host(v) for k, v in res.hits.items()}
    assert H["ev_count"].max() > 1024                  # beyond the shared-memory passes
    fcfg = CF.workload_finder(G.sector_names)
    got_cl = {k: host(v) for k, v in res.clusters.items()}
    got_mem = {k: host(v) for k, v in res.members.items()}
    ref_members, ref_pe = [], []
    for e in range(len(H["ev_start"])):
        a, n = int(H["ev_start"][e]), int(H["ev_count"][e])
        p = dict(idx=np.arange(n), bar=H["bar"][a:a + n], sipm=H["sipm"][a:a + n], time=H["time"][a:a + n],
                 pe=H["pe"][a:a + n], seq=H["seq"][a:a + n])
        for r in O.find_event(p, G, cond.status, fcfg):
            ref_members.append((int(H["ev_key"][e]), tuple(r["pulses"])))
            ref_pe.append(r["pe"])
    got_members = [(int(got_cl["event"][i]), tuple(got_mem["idx"][got_mem["cl"] == i])) for i in range(len(got_cl["pe"]))]
    assert len(ref_members) > 0
    assert got_members == ref_members
    np.testing.assert_allclose(got_cl["pe"], ref_pe, rtol=1e-12)
