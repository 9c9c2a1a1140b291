"""Oracle of the lookup-table photon model (photons._substep_photons, crv/crvfastsim/response/photons.py:163-224)
against the reference's own outputs: a synthetic table and rows with the reference's statistics over 16 generator
seeds (tests/golden/lookup.npz, made by tests/golden/make_golden.py).  The reference draws from a sequential
generator and the oracle from keyed Philox blocks, so the comparison is statistical: photons per row (chi-square per
degree of freedom), total photons, and the distribution of arrival delays (Kolmogorov-Smirnov distance)."""
import os
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "lookup.npz")


def lookup_fixture():
    z = np.load(GOLDEN)
    edges = {k: z[f"edge_{k}"] for k in O.LOOKUP_EDGES}
    tabs = {k: SimpleNamespace(**{f: z[f"{k}_{f}"] for f in ("prob", "delays", "delay_sum", "emis", "emis_sum")})
            for k in O.LOOKUP_TABLES}
    geo = {k[4:]: float(z[k]) for k in z.files if k.startswith("geo_")}
    rows = {k[4:]: z[k] for k in z.files if k.startswith("row_")}
    return SimpleNamespace(edges=edges, tables=tabs, **geo), rows, z


def test_substep_oracle_matches_the_reference_statistically():
    L, rows, z = lookup_fixture()
    R, S = len(rows["nsub"]), int(z["ref_seeds"])
    counts, hist, total = np.zeros(R), np.zeros(64), 0
    for s in range(S):
        st, ch, tm, lim = O.substep_photons(L, rows, 500 + s)
        assert not lim
        ri = (st - 3) // 7
        assert np.array_equal(ch, rows["chan"][ri])
        counts += np.bincount(ri, minlength=R)
        hist += np.bincount(np.clip((tm - rows["t0"][ri]).astype(np.int64), 0, 63), minlength=64)
        total += len(st)
    counts, hist = counts / S, hist / S
    ref_counts, ref_hist, ref_total = z["ref_counts"], z["ref_delay_hist"], float(z["ref_total"]) / S
    assert ref_total > 50000
    assert abs(total / S / ref_total - 1) < 0.01
    m = (ref_counts + counts) > 2
    chi2 = np.mean((counts[m] - ref_counts[m]) ** 2 / ((counts[m] + ref_counts[m]) / S))
    assert 0.8 < chi2 < 1.25
    ks = np.max(np.abs(np.cumsum(hist) / hist.sum() - np.cumsum(ref_hist) / ref_hist.sum()))
    assert ks < 0.01


def test_substep_oracle_is_keyed():
    """Rows give the same photons alone and in a batch (draws keyed by step, channel, substep, arrival)."""
    L, rows, _ = lookup_fixture()
    st, ch, tm, _ = O.substep_photons(L, rows, 9)
    part = {k: v[100:140] for k, v in rows.items()}
    st2, ch2, tm2, _ = O.substep_photons(L, part, 9)
    sel = np.isin(st, part["step"])
    assert sel.sum() == len(st2) > 0
    assert np.array_equal(st[sel], st2) and np.array_equal(tm[sel], tm2)
    st3, _, tm3, _ = O.substep_photons(L, rows, 10)
    assert len(st3) != len(st) or not np.array_equal(tm3, tm)


@pytest.mark.parametrize("n,p", [(10, 0.3), (1000, 0.002), (5000, 0.7), (100000, 0.01), (50, 0.999), (7, 1.0),
                                 (0, 0.5), (12, 0.0)])
def test_substep_binomial_moments(n, p):
    x = O.binomial(17, np.full(40000, n), np.full(40000, p))
    assert x.min() >= 0 and x.max() <= n
    mean, var = n * p, n * p * (1 - p)
    if var == 0:
        assert np.all(x == mean)
        return
    assert abs(x.mean() - mean) < 5 * np.sqrt(var / len(x))
    assert abs(x.var() / var - 1) < 0.05


def lookup_chain_fixture():
    """Tables, geometry, configuration, steps and reference statistics of tests/golden/lookup_chain.npz."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "lookup_chain.npz"))
    tables = {}
    for name in ("tabA", "tabB"):
        geo = {k[len(name) + 5:]: float(z[k]) for k in z.files if k.startswith(f"{name}_geo_")}
        tables[name] = SimpleNamespace(
            name=name, reflector=int(z[f"{name}_reflector"]), ck_scint=z["ck"], ck_fiber=z["ck"] * 0.5,
            edges={k: z[f"{name}_edge_{k}"] for k in O.LOOKUP_EDGES},
            tables={t: SimpleNamespace(**{f: z[f"{name}_{t}_{f}"] for f in ("prob", "delays", "delay_sum", "emis",
                                                                              "emis_sum")}) for t in O.LOOKUP_TABLES},
            **geo)
    nb = 12
    geom = SimpleNamespace(nbars=nb, sector=np.r_[np.zeros(8, np.int64), np.ones(4, np.int64)],
                           module=np.r_[np.repeat([0, 1], 4), np.zeros(4, np.int64)],
                           local_to_world=np.array([[0, 1, 2]] * 8 + [[1, 0, 2]] * 4, np.int8),
                           center=np.c_[np.arange(nb) * 30.0, np.arange(nb) * 55.0 - 300.0, np.full(nb, 100.0)],
                           sector_names=["EX", "T1"])
    sector = lambda t, r, y: SimpleNamespace(table=t, reflector=r, yield_per_mev=y)  # noqa: E731
    cfg = SimpleNamespace(sectors={"EX": sector("tabA", 0, 1500.0), "T1": sector("tabB", -1, 1200.0)},
                          photon_yield_scale=0.94, photon_yield_variation_scale=1.0, speed_ratio={"EX": 1.1},
                          atten_ratio={"T1": 0.9, "EX1": 1.2})
    steps = {k[5:]: z[k] for k in z.files if k.startswith("step_")}
    return tables, geom, cfg, steps, z


def test_lookup_setup_matches_the_reference():
    """Table propagation fits and per-bar ratios: the oracle's and the engine's host setup give the reference's
    values."""
    from crvgpu import lookup as LK
    tables, geom, cfg, _, z = lookup_chain_fixture()
    for name, L in tables.items():
        assert np.allclose(O.table_propagation(L), z[f"{name}_propagation"], rtol=1e-12, atol=0)
        assert np.allclose(LK.table_propagation(L), z[f"{name}_propagation"], rtol=1e-12, atol=0)
    for impl in (O.bar_ratios, LK.bar_ratios):
        assert np.array_equal(impl(cfg.speed_ratio, geom), z["speed_ratio"])
        assert np.array_equal(impl(cfg.atten_ratio, geom), z["atten_ratio"])
    with pytest.raises(KeyError):
        LK.bar_ratios({"XX": 1.1}, geom)


def test_lookup_make_photons_oracle_matches_the_reference_statistically():
    tables, geom, cfg, steps, z = lookup_chain_fixture()
    S = int(z["ref_seeds"])
    pairs = {tuple(p): i for i, p in enumerate(z["ref_pairs"])}
    ref_mean = z["ref_pair_mean"]
    got = np.zeros(len(pairs))
    extra = 0
    hist, total = np.zeros(96), 0
    for s in range(S):
        st, ch, tm = O.make_photons_lookup(steps, z["pdg"], geom, cfg, tables, z["deviation"], 700 + s)
        for a, b in zip(st, ch):
            i = pairs.get((a, b))
            if i is None:
                extra += 1
            else:
                got[i] += 1
        hist += np.bincount(np.clip((tm - steps["t0"][st]).astype(np.int64), 0, 95), minlength=96)
        total += len(st)
    got /= S
    ref_total = float(z["ref_total"]) / S
    assert ref_total > 5000
    assert abs(total / S / ref_total - 1) < 0.02
    assert extra / S < 0.01 * ref_total                  # (step, channel) pairs the reference never lit are rare
    m = (ref_mean + got) > 2
    chi2 = np.mean((got[m] - ref_mean[m]) ** 2 / ((got[m] + ref_mean[m]) / S))
    assert 0.7 < chi2 < 1.4
    ks = np.max(np.abs(np.cumsum(hist) / hist.sum() - np.cumsum(z["ref_delay_hist"]) / z["ref_delay_hist"].sum()))
    assert ks < 0.02


def test_lookup_helpers_pass_the_references_known_answers():
    """The reference's own helper tests (crv/tests/test_photons.py:13-29): findBin's inclusive edges, Cherenkov
    interpolation with the charge, particle charges (ions decoded) and the stock beta; plus the cos-space phi bins
    against arccos."""
    e = np.array([0.0, 1.0, 2.0, 3.0])
    assert O.find_bin(e, [-0.1, 0.0, 0.5, 1.0, 2.999, 3.0, 3.1]).tolist() == [-1, 0, 0, 0, 2, 2, -1]
    cmap = np.array([[0.5, 0.0], [0.6, 10.0], [1.0, 50.0]])
    assert np.allclose(O.cerenkov_per_mm([0.25, 0.55, 0.8, 1.2], [1, 1, -2, 1], cmap), [0.0, 5.0, 60.0, 50.0])
    m, q, b = O.particle_beta([13, -11, 22, 2212, 1000020040, 999], [105.66] * 6, [105.66] * 6)
    assert q.tolist() == [-1, 1, 0, 1, 2, 0]
    assert m[4] == pytest.approx(4 * 931.49410242) and m[5] == 0.0
    _, _, b2 = O.particle_beta([13, 22], [105.6583755, 0.0], [105.6583755, 0.0])
    assert b2[0] == pytest.approx(1 / np.sqrt(2)) and b2[1] == 1.0
    phi_edges = np.linspace(0.0, np.pi, 6)
    ang = np.r_[0.0, np.pi, np.random.default_rng(1).uniform(0, np.pi, 2000)]
    assert np.array_equal(O.find_bin_cos(phi_edges, np.cos(ang)), O.find_bin(phi_edges, ang)) or \
        np.mean(O.find_bin_cos(phi_edges, np.cos(ang)) == O.find_bin(phi_edges, ang)) > 0.999


def test_engine_lookup_groups_match_the_oracle_setup(monkeypatch):
    """The engine's host setup of the lookup model (groups in the reference's order, per-bar yield, extra delay and
    attenuation, channel yield factors, Cherenkov maps) equals the oracle's restatement (tables built as host tensors:
    no kernels run)."""
    import torch
    from crvgpu import lookup as LK
    monkeypatch.setattr(LK, "_torch", lambda: torch)
    tables, geom, cfg, _, z = lookup_chain_fixture()
    model = LK.LookupModel(geom, cfg, tables, z["deviation"], device="cpu")
    ref = O.lookup_groups(geom, cfg, tables, z["deviation"])
    assert [(g["table"], g["reflector"]) for g in model.groups] == [(L.name, g["reflector"]) for L, g in ref]
    for g, (L, og) in zip(model.groups, ref):
        assert np.array_equal(g["in_group"].numpy(), og["in_group"])
        for k, ok in (("yield_", "yield"), ("speed_k", "speed_k"), ("mu", "mu"), ("ck_scint", "ck_scint"),
                      ("ck_fiber", "ck_fiber")):
            assert np.array_equal(g[k].numpy().reshape(np.shape(og[ok])), og[ok]), k
        assert g["DL"].half_length == og["half_length"]
    assert np.array_equal(model.dev.numpy(), ref[0][1]["dev"])
    with pytest.raises(ValueError):
        bad = type(cfg)(**{**vars(cfg), "sectors": {**cfg.sectors, "T1": type(cfg.sectors["T1"])(
            table="tabB", reflector=0, yield_per_mev=1.0)}})
        LK.LookupModel(geom, bad, tables, z["deviation"], device="cpu")   # reflector 0 on a reflector-1 table


def test_lookup_rows_match_the_references_rows():
    """Row preparation against the reference's own iter_rows (photons.py:305-356): every field but the drawn photon
    counts is deterministic, so the oracle's rows must equal the reference's (cos theta against the cosine of its
    theta: arccos then cos, so within 1e-12)."""
    tables, geom, cfg, steps, z = lookup_chain_fixture()
    cols = {k: np.asarray(steps[k], np.float64) for k in ("x0", "y0", "z0", "x1", "y1", "z1", "px0", "py0", "pz0",
                                                          "p1", "t0", "t1", "edep", "len")}
    cols["bar"], cols["pdg"] = np.asarray(steps["bar"], np.int32), z["pdg"]
    got = [O.lookup_rows(g, cols, 5) for _, g in O.lookup_groups(geom, cfg, tables, z["deviation"])]
    # the reference yields a block per (table, reflector, SiPM); a group here holds its SiPM blocks in that order
    blocks = z["rows_groups"]
    assert [len(r["nsub"]) for r in got] == [int(blocks[blocks[:, 0] == t, 1].sum()) for t in (0, 1)]
    cat = {k: np.concatenate([r[k] for r in got]) for k in got[0]}
    for k in ("s", "d", "t0", "t1", "nsub", "beta", "dev", "mu", "step", "chan"):
        assert np.array_equal(cat[k], z[f"rows_{k}"]), k
    assert np.allclose(cat["cos_theta"], np.cos(z["rows_theta"]), rtol=0, atol=1e-12)


def test_substep_bins_match_the_references_bins():
    """Geometry and binning of every substep against the reference's own substep kernel: the bins it read from each
    table (recorded by the fixture generator, in substep order) are the bins the oracle (and, bit-exact with it, the
    GPU) selects."""
    L, rows, z = lookup_fixture()
    sub = {k: v[:120] for k, v in rows.items()}
    bins = O.substep_bins(L, sub)
    for t, name in enumerate(O.LOOKUP_TABLES):
        ours = bins[:, t][bins[:, t] >= 0]
        ref = z[f"ref_bins_{name}"]
        assert len(ref) > 1000 or name == "ckfiber" and len(ref) > 1000 // 4
        assert np.array_equal(ours, ref), name


def test_delay_and_emission_search_match_the_reference():
    """The index search of the delay and emission draws against the reference's _first_above (photons.py:118-137) on
    4,000 random bins and thresholds: identical indices."""
    L, _, z = lookup_fixture()
    T = L.tables["scint"]
    assert np.array_equal(O.first_reaching(T.delays, z["ref_search_bins"], z["ref_search_dthr"]), z["ref_search_delay"])
    assert np.array_equal(O.first_reaching(T.emis, z["ref_search_bins"], z["ref_search_ethr"]), z["ref_search_emis"])


def test_propagation_helpers_match_the_references_own_tests(golden):
    """crv/tests/test_propagation.py replayed (make_golden.py propagation): the fit on its known-value table (speed
    160 mm/ns, attenuation 6000 mm) and the per-bar ratios on its 11-sector geometry equal the reference's, in the
    engine's host setup and in the oracle; an unknown module key raises the same KeyError."""
    import json
    from types import SimpleNamespace
    from crvgpu import lookup as LK
    from crvgpu import lookup_file as LF
    g = golden("propagation.npz")
    for i in range(int(g["n_tp"])):
        a = lambda k: g[f"tp{i}_{k}"]                                            # noqa: E731
        L = LF.LookupTable(str(a("name")), tuple(a("version")), int(a("reflector")), *a("constants"), a("ck_scint"),
                           a("ck_fiber"), {k: a(f"edges_{k}") for k in LF.EDGES},
                           {t: LF.Table(*(a(f"{t}_{f}") for f in ("prob", "delays", "delay_sum", "emis", "emis_sum")))
                            for t in LF.TABLES})
        for fit in (LK.table_propagation(L), O.table_propagation(L)):
            assert np.array_equal(np.asarray(fit), a("fit")), (fit, a("fit"))
    for i in range(int(g["n_bk"])):
        G = SimpleNamespace(sector=g[f"bk{i}_G_sector"], module=g[f"bk{i}_G_module"], nbars=int(g[f"bk{i}_G_nbars"]),
                            sector_names=[str(s) for s in g[f"bk{i}_G_sector_names"]])
        sk, mk = LK.bar_keys(G)
        assert sk.astype(str).tolist() == g[f"bk{i}_sector_keys"].tolist()
        assert mk.astype(str).tolist() == g[f"bk{i}_module_keys"].tolist()
    for i in range(int(g["n_br"])):
        G = SimpleNamespace(sector=g[f"br{i}_G_sector"], module=g[f"br{i}_G_module"], nbars=int(g[f"br{i}_G_nbars"]),
                            sector_names=[str(s) for s in g[f"br{i}_G_sector_names"]])
        values = json.loads(str(g[f"br{i}_values"]))
        for fn in (LK.bar_ratios, O.bar_ratios):
            if f"br{i}_error" in g.files:
                with pytest.raises(KeyError) as e:
                    fn(values, G)
                assert e.value.args[0] == str(g[f"br{i}_error"])
            else:
                assert np.array_equal(fn(values, G), g[f"br{i}_out"])
