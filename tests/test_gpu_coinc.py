"""GPU coincidence finder against the reference's own find_event outputs (golden fixtures on three geometries:
a 4 x 16 module with tracks, noise and showers; two sector types with one single-sided; eight bars with quantised
times and PEs that exercise ties and opposite-side attachment).  Membership (and its order) identical; cluster
properties within 1e-12 relative (sums in a different order)."""
from types import SimpleNamespace

import numpy as np
import pytest

from crvgpu import config as CF

pytestmark = pytest.mark.gpu


def geom_of(g, tag):
    G = SimpleNamespace(**{k: g[f"{tag}_G_{k}"] for k in ("sector", "layer", "counter_in_type", "x", "y", "pos",
                                                           "length_dir", "sector_type", "pos_side0", "pos_side1",
                                                           "sipms_side0", "sipms_side1")})
    G.sector_names = [str(s) for s in g[f"{tag}_G_sector_names"]]
    return G


def finder_of(g, tag, G):
    cuts = {}
    for name, row in zip(G.sector_names, g[f"{tag}_cuts"]):
        cuts[name] = CF.SectorCuts(*[int(v) if i == 6 else float(v) for i, v in enumerate(row)])
    return CF.FinderConfig(cuts=cuts)


@pytest.mark.parametrize("tag", ["module", "two", "eight"])
def test_coincidences_match_reference_fixtures(golden, tag):
    from crvgpu import coinc as CO
    g = golden("coinc.npz")
    G = geom_of(g, tag)
    cfg = finder_of(g, tag, G)
    P = {k: g[f"{tag}_in_{k}"] for k in ("ev", "idx", "bar", "sipm", "time", "pe", "seq")}
    cl, mem = CO.find_events(P["ev"], P["idx"], P["bar"], P["sipm"], P["time"], P["pe"], P["seq"], G,
                             g[f"{tag}_status"], cfg)
    ref = lambda k: g[f"{tag}_scalar_{k}"]  # noqa: E731
    assert len(cl["pe"]) == len(ref("pe")) > 0
    assert np.array_equal(cl["event"], ref("ev"))
    assert np.array_equal(cl["type"], ref("type"))
    assert np.array_equal(mem["cl"], ref("mem_cl"))
    assert np.array_equal(mem["idx"], ref("mem_idx"))
    assert np.array_equal(cl["poscalc"].astype(bool), ref("poscalc"))
    assert np.array_equal(cl["sidehits"], ref("sidehits"))
    assert np.array_equal(cl["nlayers"], ref("nlayers"))
    for k, r in (("pe", "pe"), ("start", "start"), ("end", "end"), ("slope", "slope"), ("avgtime", "avgtime"),
                 ("pos", "pos"), ("sidepe", "sidepe"), ("sidetime", "sidetime")):
        np.testing.assert_allclose(cl[k], ref(r), rtol=1e-12, atol=1e-9, err_msg=k)


def test_find_event_single_event_signature(golden):
    from crvgpu import coinc as CO
    g = golden("coinc.npz")
    G = geom_of(g, "eight")
    cfg = finder_of(g, "eight", G)
    P = {k: g[f"eight_in_{k}"] for k in ("ev", "idx", "bar", "sipm", "time", "pe", "seq")}
    e = np.unique(P["ev"])[3]
    m = P["ev"] == e
    rows = CO.find_event({k: P[k][m] for k in ("idx", "bar", "sipm", "time", "pe", "seq")}, G, g["eight_status"], cfg)
    sel = g["eight_scalar_ev"] == e
    assert len(rows) == int(sel.sum())
    first = np.flatnonzero(sel)
    for r, i in zip(rows, first):
        assert r["pulses"] == list(g["eight_scalar_mem_idx"][g["eight_scalar_mem_cl"] == i])


def test_coincidences_match_the_reference_attachment_cases(golden):
    """The reference's own attachment boundary cases (every find_event call of crv/tests/test_coinc_attachment_cpu.py:
    strict windows, ties, order, configuration flags) on the GPU: same clusters and members, properties within 1e-12."""
    from crvgpu import coinc as CO
    from tests.test_oracle_golden import attach_case
    g = golden("attach.npz")
    for i in range(int(g["n"])):
        G, cfg, status, P = attach_case(g, i)
        rows = CO.find_event(P, G, status, cfg)
        tag = f"a{i}_scalar_"
        assert len(rows) == len(g[tag + "pe"]), i
        for c, r in enumerate(rows):
            assert list(r["pulses"]) == list(g[tag + "mem_idx"][g[tag + "mem_cl"] == c]), i
            for k in ("pe", "start", "end", "slope", "avgtime"):
                np.testing.assert_allclose(r[k], g[tag + k][c], rtol=1e-12, atol=1e-9, err_msg=f"a{i}.{k}")
            assert list(r["sidehits"]) == list(g[tag + "sidehits"][c]), i
