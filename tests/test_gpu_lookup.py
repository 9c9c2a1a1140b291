"""The lookup-table photon model on the GPU (crv_substep_photons) against the oracle: the same photons, bit for bit
and in the same (row, substep, table, arrival) order, on the reference-pinned synthetic table and rows, with and
without extra attenuation and fibre decay; keyed draws (a batch split gives the same photons); output capacity growth."""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import oracle as O
from tests.test_oracle_lookup import lookup_fixture

pytestmark = pytest.mark.gpu


def _check(L, rows, seed):
    from crvgpu import lookup as LK
    st, ch, tm = LK.substep_photons(L, rows, seed)
    ost, och, otm, lim = O.substep_photons(L, rows, seed)
    assert not lim and len(st) > 1000
    assert np.array_equal(st, ost) and np.array_equal(ch, och)
    assert np.array_equal(tm, otm)
    return st, tm


def test_substeps_match_the_oracle_bit_for_bit():
    L, rows, _ = lookup_fixture()
    _check(L, rows, 500)
    # no extra attenuation, no fibre decay (the reference bench's table)
    L0 = SimpleNamespace(**{**vars(L), "fiber_decay_time": 0.0})
    r0 = {k: v for k, v in rows.items() if k != "mu"}
    _check(L0, r0, 77)


def test_substeps_are_keyed_and_capacity_grows():
    from crvgpu import lookup as LK
    L, rows, _ = lookup_fixture()
    st, tm = _check(L, rows, 3)
    eng = LK.SubstepEngine()
    eng.per_row = 0.01                                   # far too small: the engine grows the output and re-runs
    DL = LK.DeviceLookup(L)
    part = {k: v[200:700] for k, v in rows.items()}
    s2, c2, t2 = (x.cpu().numpy() for x in eng.run(DL, LK.DeviceRows(part), 3))
    sel = np.isin(st, part["step"])
    assert np.array_equal(st[sel], s2) and np.array_equal(tm[sel], t2)
    assert eng.per_row > 0.01


def test_lookup_rows_and_make_photons_match_the_oracle():
    """Row preparation (every row field) and the whole lookup-table make_photons: bit for bit as the oracle, with two
    tables (reflector 0 and -1), speed and attenuation ratios, skipped non-finite steps, ions and neutral particles."""
    import torch
    from crvgpu import lookup as LK
    from tests.test_oracle_lookup import lookup_chain_fixture
    tables, geom, cfg, steps, z = lookup_chain_fixture()
    model = LK.LookupModel(geom, cfg, tables, z["deviation"])
    cols = model.upload_steps(steps, z["pdg"])
    ogroups = O.lookup_groups(geom, cfg, tables, z["deviation"])
    assert len(ogroups) == len(model.groups) == 2
    ocols = {k: np.asarray(steps[k], np.float64) for k in ("x0", "y0", "z0", "x1", "y1", "z1", "px0", "py0", "pz0",
                                                           "p1", "t0", "t1", "edep", "len")}
    ocols["bar"], ocols["pdg"] = np.asarray(steps["bar"], np.int32), z["pdg"]
    for g, (_, og) in zip(model.groups, ogroups):
        out, m = model.rows(g, cols, len(z["pdg"]), 11)
        ref = O.lookup_rows(og, ocols, 11)
        assert m == len(ref["nsub"]) > 0
        for k, v in ref.items():
            assert np.array_equal(out[k][:m].cpu().numpy(), v), k
    st, ch, tm = (x.cpu().numpy() for x in model.make_photons(steps, z["pdg"], 11))
    ost, och, otm = O.make_photons_lookup(steps, z["pdg"], geom, cfg, tables, z["deviation"], 11)
    assert len(st) > 5000
    assert np.array_equal(st, ost) and np.array_equal(ch, och) and np.array_equal(tm, otm)
    torch.cuda.synchronize()


def test_fp32_substeps_match_fp64():
    """FP32-mixed substeps against the FP64 path on the same keys: the 24-bit uniforms are the top bits of the FP64
    path's words, so arrivals and delays differ only where a draw lands within 2^-24 of a threshold or FP32 geometry
    moves a substep across a bin edge; photon times differ by the FP32 rounding of their offsets."""
    from crvgpu import lookup as LK
    L, rows, _ = lookup_fixture()
    R = len(rows["nsub"])
    s64, _, t64 = LK.substep_photons(L, rows, 40)
    s32, _, t32 = LK.substep_photons(L, rows, 40, precision="fp32")
    c64 = np.bincount((s64 - 3) // 7, minlength=R)
    c32 = np.bincount((s32 - 3) // 7, minlength=R)
    assert abs(len(s32) / len(s64) - 1) < 1e-3
    same = c32 == c64
    assert same.mean() > 0.99
    # photons of rows with equal counts, in the same order: times within the FP32 offset rounding, rarely a delay bin
    keep64 = same[(s64 - 3) // 7]
    keep32 = same[(s32 - 3) // 7]
    dt = np.abs(t32[keep32] - t64[keep64])
    assert np.median(dt) < 1e-4 and np.mean(dt < 1e-3) > 0.99
    with pytest.raises(ValueError):
        LK.substep_photons(L, rows, 1, precision="fp16")


def test_charges_with_lookup_tables_match_the_oracle():
    """chain.charges with lookup tables (the reference's production path, crv/crvfastsim/chain.py:197-213): lookup
    photons, status-masked SiPMs dropped, labels by event, SiPM stage up to the window's end: bit for bit as the
    oracle's photons through the oracle's SiPM stage."""
    from crvgpu import chain as CH
    from crvgpu.config import ChainConfig
    from tests.test_oracle_lookup import lookup_chain_fixture
    tables, geom, lcfg, steps, z = lookup_chain_fixture()
    n = len(z["pdg"])
    steps = dict(steps, event=np.arange(n) // 40, subrun=np.ones(n, np.int64), run=np.full(n, 3, np.int64))
    status = np.zeros(4 * geom.nbars, np.int64)
    status[[5, 18, 33]] = [1, 4, 2]                        # absent, no data (dropped) and compensated (kept)
    cond = SimpleNamespace(status=status, deviation=z["deviation"])
    cfg = ChainConfig(lookup=lcfg)
    Q = CH.charges(steps, None, geom, cond, cfg, None, key=21, tabs=tables, pdg=z["pdg"])
    s, c, t = O.make_photons_lookup(steps, z["pdg"], geom, lcfg, tables, z["deviation"], 21)
    keep = (status[c] & 0b101) == 0
    s, c, t = s[keep], c[keep], t[keep]
    label = ((steps["subrun"][s] << 20) | steps["event"][s]) * 32768 + c
    o = np.argsort(label, kind="stable")
    u, start, cnt = np.unique(label[o], return_index=True, return_counts=True)
    key = np.empty(len(label), np.int64)
    key[o] = np.arange(len(label)) - np.repeat(start, cnt)  # index of the photon within its SiPM, input order
    Qo, _, _, _, st = O.sipm_groups(label, t, s, key, lambda L: np.full(len(L), 3), cfg.sipm, 21, cfg.window[1])
    assert st == 0 and len(Qo["time"]) > 1000
    for k in ("chan", "time", "charge", "pe", "photon"):
        assert np.array_equal(Q[k], Qo[k]), k
    with pytest.raises(ValueError):
        CH.charges(steps, None, geom, cond, ChainConfig(), None, key=21, tabs=tables, pdg=z["pdg"])


def test_lookup_edge_cases():
    """Empty rows, rows without photons, a row beyond the substep key limit (rejected, not truncated), and steps whose
    times are not finite (skipped, as the reference skips them)."""
    from crvgpu import lookup as LK
    from crvgpu.response import EngineError
    from tests.test_oracle_lookup import lookup_chain_fixture
    L, rows, _ = lookup_fixture()
    empty = {k: v[:0] for k, v in rows.items()}
    st, ch, tm = LK.substep_photons(L, empty, 1)
    assert len(st) == len(ch) == len(tm) == 0
    quiet = dict(rows, n_scint=np.zeros_like(rows["n_scint"]), n_ck_s=np.zeros_like(rows["n_ck_s"]),
                 n_ck_f=np.zeros_like(rows["n_ck_f"]))
    assert len(LK.substep_photons(L, quiet, 1)[0]) == 0
    assert len(LK.substep_photons(L, quiet, 1, precision="fp32")[0]) == 0
    long_row = {k: v[:4].copy() for k, v in rows.items()}
    long_row["nsub"][2] = (1 << 20) + 1
    with pytest.raises(EngineError):
        LK.substep_photons(L, long_row, 1)
    tables, geom, lcfg, steps, z = lookup_chain_fixture()
    nan_steps = dict(steps, t0=np.full(len(z["pdg"]), np.nan))
    model = LK.LookupModel(geom, lcfg, tables, z["deviation"])
    s, c, t = model.make_photons(nan_steps, z["pdg"], 3)
    assert s.numel() == c.numel() == t.numel() == 0
