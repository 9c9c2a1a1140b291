"""Host logic of the resident chain: explicit capacities (every entry required, positive ints, nothing unknown) and
their growth from the sizes a rejected batch needed."""
import numpy as np
import pytest


def _caps(**over):
    from crvgpu.resident import ChainCaps
    d = dict(events=1024, steps=50000, photons=10 ** 7, charges=10 ** 6, slots=10 ** 5, digis=10 ** 5, pulses=10 ** 5,
             max_steps_per_event=128)
    d.update(over)
    return ChainCaps(**d)


def test_capacities_are_explicit_positive_ints():
    from crvgpu.resident import ChainCaps
    c = _caps()
    assert ChainCaps.from_dict(c.as_dict()) == c
    d = c.as_dict()
    del d["pulses"]
    with pytest.raises(ValueError, match="missing"):
        ChainCaps.from_dict(d)
    with pytest.raises(ValueError, match="extra"):
        ChainCaps.from_dict({**c.as_dict(), "thermal": 5})
    for bad in (0, -3, 2.0, True, "8"):
        with pytest.raises(ValueError):
            _caps(digis=bad)
    with pytest.raises(ValueError):
        _caps(max_steps_per_event=40000)


def test_capacities_match_the_c_struct_layout():
    import ctypes
    from crvgpu import _capi
    c = _caps(events=3, steps=5, photons=7, charges=11, slots=13, digis=17, pulses=19, max_steps_per_event=23)
    s = c.c()
    assert ctypes.sizeof(s) == 7 * 8 + 2 * 4
    assert [getattr(s, k) for k in _capi.CHAIN_CAPS] == [3, 5, 7, 11, 13, 17, 19, 23]


def test_growth_follows_the_needed_sizes():
    from crvgpu import _capi
    N = _capi.NEED
    c = _caps()
    need = np.zeros(16, np.int64)
    need[N["PULSES_OUT"]] = 400000
    need[N["DIGIS_OUT"]] = 150000
    need[N["STEPS_PER_EVENT"]] = 300
    g = c.grown(need, margin=1.25)
    assert g.pulses == 500000 and g.digis == 187500 and g.max_steps_per_event == 300
    assert (g.photons, g.charges, g.slots, g.events, g.steps) == (c.photons, c.charges, c.slots, c.events, c.steps)
    need[:] = 0
    need[N["SLOTS_TOTAL"]] = 1                 # SiPM slots scale with the photon capacity
    assert c.grown(need).photons > c.photons
    need[:] = 0
    need[N["MEMBERS"]] = 2 * 10 ** 5
    assert c.grown(need).pulses == 250000


def test_caps_from_trial_counts():
    from crvgpu.resident import ChainCaps
    counts = dict(charges=5000, digis=800, waveforms=700, pulses=900, events=60, hits=880, clusters=30, members=120,
                  photons=90000, slots=1200)
    c = ChainCaps.from_counts(counts, events=64, steps=2600, max_steps_per_event=70, margin=1.5)
    assert (c.photons, c.charges, c.slots, c.digis, c.pulses) == (135000, 7500, 1800, 1200, 1350)
    assert (c.events, c.steps, c.max_steps_per_event) == (64, 2600, 70)


def test_chain_count_slots_match_the_header():
    import os
    import re
    from crvgpu import _capi
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "crvgpu.h")).read()
    slots = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"#define CRV_CHAIN_([A-Z]+) (\d+)", hdr)}
    assert [k for k, _ in sorted(slots.items(), key=lambda kv: kv[1])] == list(_capi.CHAIN_COUNTS)


def test_planted_flags_are_never_consumed(monkeypatch):
    """As the reference's fail-closed contract test: a status block with a flag set turns the batch into
    BatchRejected with the sizes needed; only a clean status returns outputs (planted in host tensors, no kernels)."""
    import torch
    from crvgpu import _capi, resident
    from crvgpu.resident import BatchRejected, ResidentChain
    monkeypatch.setattr(resident, "_torch", lambda: torch)

    class Status:
        def __init__(self):
            self.t = torch.zeros(17, dtype=torch.int64)

    rc = object.__new__(ResidentChain)
    rc.counts = torch.arange(10, dtype=torch.int64) + 1
    rc.status = Status()
    rc._n_events = 7
    rc.cl = {"pe": torch.arange(20, dtype=torch.float64)}
    rc.mem = {"cl": torch.arange(20, dtype=torch.int64)}
    for flag, slot in ((_capi.ST_CAPACITY, "PULSES_OUT"), (_capi.ST_LIMIT, None), (_capi.ST_ORDER, None)):
        rc.status.t.zero_()
        rc.status.t[0] = flag
        if slot:
            rc.status.t[1 + _capi.NEED[slot]] = 123456
        with pytest.raises(BatchRejected) as ei:
            rc.finish()
        assert ei.value.flags == flag
        if slot:
            assert ei.value.need[_capi.NEED[slot]] == 123456
    rc.status.t.zero_()
    res = rc.finish()
    counts = dict(zip(_capi.CHAIN_COUNTS, range(1, 11)))
    assert res.counts == counts and res.n_events == 7
    assert torch.equal(res.clusters["pe"], torch.arange(counts["clusters"], dtype=torch.float64))
    assert torch.equal(res.members["cl"], torch.arange(counts["members"]))
