"""The device-resident chain (steps -> charges -> digis -> reco waveforms -> pulses -> coincidences) against the
oracle chain on the same keyed streams.

Each stage is checked on the GPU's own input of that stage (so a last-bit difference upstream cannot hide a logic
difference downstream): charges and digis bit-exact, reco waveforms identical, pulse counts/flags identical with
parameters within 1e-8 relative, coincidence membership identical.  The end-to-end cluster table agrees with the
oracle's run of the whole chain.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chain_run():
    from crvgpu import chain as CH
    from crvgpu import geometry as GM
    from crvgpu.response import upload_steps
    geom, cond, cfg, steps = workload(160, seed=12)
    cond.status[[3, 40, 77]] = [2, 1, 4]
    eng = CH.ChainEngine(geom, cond, cfg)
    ds = upload_steps(steps, nbars=geom.nbars)
    res = eng.run(ds, seed=2024, keep=True)
    return geom, cond, cfg, steps, eng, res, GM.sector_geom(geom)


def host(t):
    return t.cpu().numpy()


def test_chain_charges_and_digis_bit_exact(chain_run):
    from crvgpu import waveform as W
    geom, cond, cfg, steps, eng, res, G = chain_run
    Qo, _ = O.charges(steps, geom, cond, cfg.response, cfg.sipm, 2024, cfg.window[1])
    R = res.charges
    for k, o in (("label", "chan"), ("time", "time"), ("charge", "charge"), ("pe", "pe"), ("photon", "photon")):
        assert np.array_equal(host(getattr(R, k)), Qo[o]), k
    runs = {(1 << 20) | int(e): 1 for e in np.unique(steps["event"])}
    run_of = lambda keys: np.array([runs.get(int(k), 0) for k in np.asarray(keys).ravel()], np.int64)  # noqa: E731
    wc = eng.wcfg
    tdc0 = lambda labels: O.tdc0_of_labels(labels, cond, 2024, wc.period, cfg.feb_phase_key, run_of)  # noqa: E731
    Do = O.synthesize(Qo["chan"], Qo["time"], Qo["charge"], tdc0, W.single_pe_template(wc), wc, wc.period,
                      cfg.window, O.keyed_noise(2024, run_of))
    D = {k: host(v) for k, v in res.digis.items()}
    assert len(D["chan"]) == len(Do["chan"]) > 50
    for k in ("chan", "start", "tdc0", "starttdc", "volt", "adc"):
        assert np.array_equal(D[k], Do[k]), k


def test_chain_waveforms_pulses_and_coincidences(chain_run):
    from crvgpu import config as CF
    geom, cond, cfg, steps, eng, res, G = chain_run
    D = {k: host(v) for k, v in res.digis.items()}
    Wo = O.reco_waveforms(D, cond)
    Wg = {k: host(v) for k, v in res.waveforms.items()}
    assert len(Wg["label"]) == len(Wo["ev"])
    assert np.array_equal(Wg["label"] // 32768, Wo["ev"]) and np.array_equal(Wg["label"] % 32768, Wo["chan"])
    assert np.array_equal(Wg["n"], Wo["n"]) and np.array_equal(Wg["start"], Wo["start"])
    # pulses on the oracle's padded waveforms
    rcfg = CF.RecoConfig()
    Po = O.reconstruct_full(Wo["adc"], Wo["n"], Wo["start"], Wo["ped"], Wo["area"], Wo["height"], rcfg, rcfg.period)
    Pg = {k: host(v) for k, v in res.pulses.items()}
    for k in ("wf", "seq"):
        assert np.array_equal(Pg[k], Po[k]), k
    for k in ("failed", "zerondf", "pedfromdb"):
        assert np.array_equal(Pg[k].astype(bool), Po[k]), k
    for k in ("pe", "time"):
        rel = np.abs(Pg[k] - Po[k]) / np.maximum(np.abs(Po[k]), 1e-300)
        assert rel.max() <= 1e-8, (k, rel.max())
    # coincidences on the GPU's own finder input, event by event through the oracle
    H = {k: host(v) for k, v in res.hits.items()}
    fcfg = CF.FinderConfig()
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
    got_members = []
    for i in range(len(got_cl["pe"])):
        got_members.append((int(got_cl["event"][i]), tuple(got_mem["idx"][got_mem["cl"] == i])))
    assert got_members == ref_members
    np.testing.assert_allclose(got_cl["pe"], ref_pe, rtol=1e-12)
    assert res.n_clusters == len(ref_members)


def test_chain_end_to_end_matches_oracle_chain(chain_run):
    from crvgpu import config as CF
    geom, cond, cfg, steps, eng, res, G = chain_run
    H = {k: host(v) for k, v in res.hits.items()}
    D = {k: host(v) for k, v in res.digis.items()}
    Wo = O.reco_waveforms(D, cond)
    rcfg = CF.RecoConfig()
    Po = O.pulses_from_waveforms(Wo, cond, rcfg, rcfg.period)
    out = O.clusters_from_pulses(Wo, Po, G, cond.status, CF.FinderConfig())
    assert len(out["cl_event"]) == res.n_clusters
    assert np.array_equal(out["cl_event"], host(res.clusters["event"]))
    assert np.array_equal(out["mem_idx"], host(res.members["idx"]))
    np.testing.assert_allclose(out["cl_avgtime"], host(res.clusters["avgtime"]), rtol=1e-9, atol=1e-9)
    assert res.n_events == 160 and res.n_hits == len(out["pulses"]["ev"])


def test_dropin_clusters_device_glue_equals_host_sequence_and_oracle(chain_run):
    """chain.clusters (crv/crvfastsim/chain.py:296-330) on reco waveforms: its device glue (fit, ignored channels,
    DB time offsets, event t0, event order, finder input) equals the host sequence of the reference's calls
    (reconstruct_full -> filter_channels -> lexsort -> find_events) bit for bit, with the waveform rows in event order
    and shuffled, and the clusters equal the oracle chain's."""
    from crvgpu import chain as CH
    from crvgpu import config as CF
    geom, cond, cfg, steps, eng, res, G = chain_run
    D = {k: host(v) for k, v in res.digis.items()}
    Wo = O.reco_waveforms(D, cond)
    rng = np.random.default_rng(4)
    perm = rng.permutation(len(Wo["n"]))
    shuffled = {k: (v[perm] if isinstance(v, np.ndarray) and len(v) == len(perm) else v) for k, v in Wo.items()}
    with_t0 = {**Wo, "event_t0": rng.uniform(-3, 3, len(Wo["n"]))}
    fcfg = CF.FinderConfig()
    rcfg = CF.RecoConfig()
    ccfg = CF.ChainConfig(finder=fcfg, pulse_reco=rcfg)
    for W in (Wo, shuffled, with_t0):
        dev, tm = CH.clusters(W, cond, geom, G, ccfg, detail=True)
        hst, _ = CH._clusters_host(W, cond, G, fcfg, rcfg, ccfg, {}, True)
        dev, hst = dev[0], hst[0]
        assert tm["pulses"] == len(hst["pulses"]["ev"]) > 100
        for k, v in hst.items():
            if k == "pulses":
                for q in v:
                    assert np.array_equal(dev[k][q], v[q]), q
            else:
                assert np.array_equal(dev[k], v), k
    out = O.clusters_from_pulses(Wo, O.pulses_from_waveforms(Wo, cond, rcfg, rcfg.period), G, cond.status, fcfg)
    got = CH.clusters(Wo, cond, geom, G, ccfg, detail=True)[0][0]
    assert len(out["cl_event"]) > 0
    assert np.array_equal(got["cl_event"], out["cl_event"]) and np.array_equal(got["mem_idx"], out["mem_idx"])
    np.testing.assert_allclose(got["cl_avgtime"], out["cl_avgtime"], rtol=1e-9, atol=1e-9)
