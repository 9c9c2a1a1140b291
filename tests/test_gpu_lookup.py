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
