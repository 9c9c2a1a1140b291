"""The readout mask (crvgpu.readout) against every call the reference's own readout-mask tests make
(crv/tests/test_readout_mask.py, recorded by make_golden.py readout; crv/crvfastsim/readout.py:9-72): the same masks
and effective statuses, and the same ValueError messages for every invalid geometry, counters configuration, status
and mask.  No GPU."""
import builtins
import json
import os
from dataclasses import dataclass

import numpy as np
import pytest

from crvgpu import readout as RO

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "readout_calls.json")


def _raising(exc, msg):
    """A property that raises exc(msg) when read (a recorded geometry attribute whose read failed)."""
    def get(self):
        raise exc(msg)
    return property(get)


def decode(v):
    if isinstance(v, list):
        raise TypeError("bare lists are tagged")
    if not isinstance(v, dict):
        return v
    if "nd" in v:
        return np.array(v["data"], dtype=np.dtype(v["nd"])).reshape(v["shape"])
    if "npbool" in v:
        return np.bool_(v["npbool"])
    if "npint" in v:
        return np.int64(v["npint"])
    if "nan" in v:
        return float("nan")
    if "list" in v:
        return [decode(x) for x in v["list"]]
    if "tuple" in v:
        return tuple(decode(x) for x in v["tuple"])
    if "map" in v:
        return {k: decode(x) for k, x in v["map"]}
    if "obj" in v:
        attrs, props = {}, {}
        for k, x in v["obj"].items():
            if isinstance(x, dict) and "raises" in x:
                props[k] = _raising(getattr(builtins, x["raises"][0]), x["raises"][1])
            else:
                attrs[k] = decode(x)
        cls = type("Recorded", (), props)
        o = cls()
        for k, x in attrs.items():
            setattr(o, k, x)
        return o
    raise ValueError(f"unknown tag {sorted(v)}")


def calls():
    with open(GOLDEN) as f:
        return json.load(f)


def test_every_recorded_call_gives_the_references_result():
    recorded = calls()
    assert len(recorded) >= 100
    for i, c in enumerate(recorded):
        fn = getattr(RO, c["fn"])
        args = [decode(a) for a in c["args"]]
        if "error" in c:
            kind, msg = c["error"]
            with pytest.raises(getattr(builtins, kind)) as e:
                fn(*args)
            assert str(e.value) == msg, (i, c["fn"])
        else:
            out, ref = np.asarray(fn(*args)), decode(c["out"])
            assert out.dtype == ref.dtype and out.shape == ref.shape and np.array_equal(out, ref), (i, c["fn"])


@dataclass
class _Cond:
    status: np.ndarray
    readout_mask: np.ndarray = None


def test_apply_masks_absent_sides_and_keeps_extra_channels():
    """Two sectors (A: SiPMs on side 0 only, B: both sides) over three bars, conditions with four extra channels."""
    geom = type("G", (), {})()
    geom.sector_names, geom.sector, geom.nbars = ["A", "B"], np.array([0, 1, 0]), 3
    cfg = {"crs.sipmsAtSide0A": True, "crs.sipmsAtSide1A": False, "crs.sipmsAtSide0B": True,
           "crs.sipmsAtSide1B": True}
    cond = _Cond(np.zeros(16, np.int64))
    masked = RO.apply(cond, geom, cfg)
    assert cond.readout_mask is None and masked is not cond
    assert masked.readout_mask.tolist() == [True, False, True, False] + [True] * 4 + [True, False] * 2 + [True] * 4
    st = RO.effective_status(masked)
    assert st.tolist() == [0, 1, 0, 1] + [0] * 4 + [0, 1, 0, 1] + [0] * 4
    with pytest.raises(ValueError, match="conditions cover 8 channels, the geometry has 12"):
        RO.apply(_Cond(np.zeros(8, np.int64)), geom, cfg)


def test_the_chain_uses_the_readout_status():
    """The device tables take their status from crvgpu.readout (absent sensors carry bit 0)."""
    from crvgpu.response import effective_status
    cond = _Cond(np.array([0, 2, 4, 0]), np.array([True, False, True, False]))
    assert effective_status(cond).tolist() == [0, 3, 4, 1]
    with pytest.raises(ValueError, match="boolean numpy array"):
        effective_status(_Cond(np.zeros(4, np.int64), np.ones(4, int)))


def test_the_engine_refuses_masks_that_split_a_bar_side():
    """Masks built by sensor_mask cover whole sides and pass; one that masks SiPM 2 but not SiPM 0 of a bar is refused
    (the finder reads a pulse's same-side partner in the unmasked status)."""
    from crvgpu.response import check_readout_mask
    geom = type("G", (), {})()
    geom.sector_names, geom.sector, geom.nbars = ["A", "B"], np.array([0, 1, 0]), 3
    cfg = {"crs.sipmsAtSide0A": True, "crs.sipmsAtSide1A": False, "crs.sipmsAtSide0B": False,
           "crs.sipmsAtSide1B": True}
    check_readout_mask(RO.apply(_Cond(np.zeros(12, np.int64)), geom, cfg), 3)
    check_readout_mask(_Cond(np.zeros(12, np.int64)), 3)
    split = np.ones(12, bool)
    split[4 * 1 + 2] = False
    with pytest.raises(NotImplementedError, match="whole bar sides"):
        check_readout_mask(_Cond(np.zeros(12, np.int64), split), 3)
