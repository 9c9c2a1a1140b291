"""A step table written in the CrvStepTableDumper layout (crv/art/CrvFastSim/src/CrvStepTableDumper_module.cc:123-134:
run/subrun/event unsigned, bar/sp/nstep int, t0/t1 double, the rest float) and read back through crvgpu.tables goes
into chain.charges as it is, and gives the oracle's charges bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import workload

pytestmark = pytest.mark.gpu


def test_charges_from_a_step_table_file(tmp_path):
    from crvgpu import chain as CH
    from crvgpu import tables as TB
    geom, cond, cfg, steps = workload(96, seed=14)
    rng = np.random.default_rng(5)
    n = len(steps["bar"])
    d = {a: rng.uniform(-2, 2, n).astype(np.float32) for a in "xyz"}
    dump = {"run": np.asarray(steps["run"]).astype(np.uint32), "subrun": np.asarray(steps["subrun"]).astype(np.uint32),
            "event": np.asarray(steps["event"]).astype(np.uint32), "nstep": np.zeros(n, np.int32),
            "bar": np.asarray(steps["bar"], np.int32), "sp": np.ones(n, np.int32),
            "t0": np.asarray(steps["t"], np.float64) - 0.25, "t1": np.asarray(steps["t"], np.float64) + 0.25,
            "edep": np.asarray(steps["edep"], np.float32), "len": np.asarray(steps["len"], np.float32)}
    for a in "xyz":
        dump[f"{a}0"] = (np.asarray(steps[a], np.float32) - d[a]).astype(np.float32)
        dump[f"{a}1"] = (np.asarray(steps[a], np.float32) + d[a]).astype(np.float32)
    path = str(tmp_path / "crvsteps.root")
    TB.write(path, dump, None)
    s = TB.read(path, "steps")
    Q = CH.charges(s, None, geom, cond, cfg, None, key=31)
    Qo, _ = O.charges(s, geom, cond, cfg.response, cfg.sipm, 31, cfg.window[1])
    assert len(Q["time"]) > 1000
    for k in ("chan", "time", "charge", "pe", "photon"):
        assert np.array_equal(Q[k], Qo[k]), k
