"""GPU pulse reconstruction against the reference's own outputs (golden fixtures) and the oracle.

FP64: pulse counts, sequence numbers and flags identical.  Fitted parameters: every pulse within 1e-8 relative, and
at least 95 % of the pulses' PE and time within 1e-9.  exp and the reduction order differ in the last bit between NumPy and CUDA;
at the minimum chi2 is flat to ~1e-16 relative, which leaves the minimiser defined only to ~1e-9..1e-8 relative, so
a few ill-conditioned fits land 1e-9..3e-9 apart.  FP32-mixed: mean PE within 0.3 % and time within 0.05 ns of FP64
on the non-failed fits.
"""
import numpy as np
import pytest

from crvgpu import config as CF

pytestmark = pytest.mark.gpu

RTOL = 1e-9          # for at least FRAC of the pulses (PE and time)
FRAC = 0.95
RMAX = 1e-8          # for every pulse and parameter
EXACT = ("wf", "seq", "failed", "zerondf", "pedfromdb", "wf_near_threshold")
CLOSE = ("pe", "peph", "time", "height", "beta", "chi2", "letime", "ped", "fit_A", "fit_mu", "fit_b")


def compare(got, ref, tag):
    for k in EXACT:
        assert np.array_equal(np.asarray(got[k]).astype(np.int64), np.asarray(ref[k]).astype(np.int64)), (tag, k)
    worst = {}
    ok_fit = ~np.asarray(ref["failed"], bool)
    for k in CLOSE:
        a, b = np.asarray(got[k], float), np.asarray(ref[k], float)
        if k.startswith("fit_"):          # raw fit values of a failed (non-converged) fit are diagnostics only
            a, b = a[ok_fit], b[ok_fit]
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
        rel[(a == b)] = 0.0
        worst[k] = (float(rel.max()) if len(rel) else 0.0, float((rel <= RTOL).mean()) if len(rel) else 1.0)
        assert worst[k][0] <= RMAX, (tag, k, worst[k])
        if k in ("pe", "time"):
            assert worst[k][1] >= FRAC, (tag, k, worst[k])
    return worst


@pytest.mark.parametrize("tag", ["single", "kpp", "uneven", "edge", "p125"])
def test_pulsefit_matches_reference_fixtures(golden, tag):
    from crvgpu import pulsefit as PF
    g = golden("pulsefit.npz")
    period = 12.5 if tag == "p125" else float(g["period"][0])
    cfg = CF.RecoConfig(period=period)
    args = [g[f"{tag}_{k}"] for k in ("adc", "n", "start", "ped", "area", "height")]
    f = PF.reconstruct_full if tag in ("uneven", "edge") else PF.reconstruct
    r = f(*args, cfg)
    ref = {k[len(tag) + 5:]: g[k] for k in g.files if k.startswith(f"{tag}_out_")}
    worst = compare(r, ref, tag)
    print(tag, "max rel diff / fraction within 1e-9",
          {k: f"{v[0]:.1e}/{v[1]:.4f}" for k, v in worst.items()})


def cfg2_like(n_wf=3000, seed=5):
    """Uneven waveforms of the batched-fit workload: 1-12 pulses, lengths over {32..512}, pedestal 100, noise 2 ADC,
    PE log-uniform 5-500, beta U(10, 25)."""
    from tests.helpers import uneven_waveforms
    return uneven_waveforms(np.random.default_rng(seed), n_wf)


def test_pulsefit_fp32_mixed_accuracy():
    from crvgpu import pulsefit as PF
    adc, n, st, ped, area, height = cfg2_like(1500)
    cfg = CF.RecoConfig()
    r64 = PF.reconstruct_full(adc, n, st, ped, area, height, cfg)
    r32 = PF.reconstruct_full(adc, n, st, ped, area, height, cfg, precision="fp32")
    # same pulse list except for rare knife-edge flips; compare on common (wf, seq) with both fits good
    k64 = r64["wf"] * 4096 + r64["seq"]
    k32 = r32["wf"] * 4096 + r32["seq"]
    common, i64, i32 = np.intersect1d(k64, k32, return_indices=True)
    assert len(common) > 0.98 * len(k64)
    good = ~r64["failed"][i64] & ~r32["failed"][i32]
    pe64, pe32 = r64["pe"][i64][good], r32["pe"][i32][good]
    assert abs(pe32.mean() / pe64.mean() - 1) < 3e-3
    dt = np.abs(r32["time"][i32][good] - r64["time"][i64][good])
    assert np.median(dt) < 0.05


def test_graph_fitter_and_launch_shapes_match_the_engine():
    import torch
    from crvgpu import config as CF
    from crvgpu.params import make_params
    from crvgpu.pulsefit import DEFAULT_SHAPE, GraphFitter, PulseEngine, set_shape
    from tests.helpers import uneven_waveforms
    adc, n, start, ped, area, height = uneven_waveforms(np.random.default_rng(8), 300)
    W, L = adc.shape
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(np.asarray(a).astype(dt))).cuda()  # noqa: E731
    args = dict(off=d(np.arange(W) * L, np.int64), n=d(n, np.int32), start_tdc=d(start, np.int64),
                ped=d(ped, np.float64), area=d(area, np.float64), height=d(height, np.float64))
    adc16 = d(adc, np.int16)
    for prec in ("fp32", "fp64"):
        P = make_params(reco=CF.RecoConfig(), precision=prec)
        eng = PulseEngine()
        eng.out_factor = 16.0
        ref = eng.run(P, **args, adc16=adc16, max_pulses=2 ** 31 - 1, nsamples=W * L)
        try:
            set_shape((64, 8, 4))                      # another launch shape: same results
            other = eng.run(P, **args, adc16=adc16, max_pulses=2 ** 31 - 1, nsamples=W * L)
            gf = GraphFitter(P, W + 37, W * L + 1000, 16 * W)   # padded capacity, replayed graph
            got = gf.fit(args["off"], args["n"], args["start_tdc"], args["ped"], args["area"], args["height"], adc16)
            got2 = gf.fit(args["off"], args["n"], args["start_tdc"], args["ped"], args["area"], args["height"], adc16)
        finally:
            set_shape(DEFAULT_SHAPE)
        for k in ref:
            assert torch.equal(other[k], ref[k]), (prec, k)
            assert torch.equal(got[k], ref[k]), (prec, k)
            assert torch.equal(got2[k], ref[k]), (prec, k)


def test_pulsefit_matches_the_references_own_tests(golden):
    """The reference's own pulse-fit test calls (injected single pulses, below threshold, pedestal undershoot; 12.5
    ns) on the GPU: integer outputs identical, parameters as the reference within the fit's 1e-8."""
    from crvgpu import pulsefit as PF
    g = golden("pulsetests.npz")
    period = float(g["period"][0])
    for i in range(int(g["n"])):
        tag = f"r{i}"
        args = [g[f"{tag}_{k}"] for k in ("adc", "n", "start", "ped", "area", "height")]
        r = PF.reconstruct(*args, CF.RecoConfig(period=period))
        ref = {k[len(tag) + 5:]: g[k] for k in g.files if k.startswith(f"{tag}_out_")}
        compare(r, ref, tag)
