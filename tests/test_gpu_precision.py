"""FP32-mixed chain against the FP64-plain chain on the same events and keys: the workload's accuracy contract.

Bounds (the workload's): mean pulse PE within 0.3 %, pulse time within 0.05 ns (99th percentile of matched, well-fitted
pulses), ADC-sample mismatches confined to quantisation boundaries; coincidence membership nearly always the same.
The full report is crvgpu.accuracy.error_table; bench.py prints it for a 65,536-event batch.
"""
import json

import pytest

from tests.helpers import workload

pytestmark = pytest.mark.gpu


def test_fp32_mixed_chain_error_table_within_the_contract():
    from crvgpu import chain as CH, config as CF
    from crvgpu.accuracy import error_table
    from crvgpu.response import upload_steps
    geom, cond, _, steps = workload(2048, seed=31)
    ds = upload_steps(steps, nbars=geom.nbars)
    e64 = CH.ChainEngine(geom, cond, CF.ChainConfig(precision="fp64"))
    e32 = CH.ChainEngine(geom, cond, CF.ChainConfig(precision="fp32"))
    r64, r32 = e64.run(ds, 9, keep=True), e32.run(ds, 9, keep=True)
    t = error_table(r64, r32, e32.wcfg.adc_conversion, e32.wcfg.pedestal)
    print(json.dumps(t, indent=1))
    assert abs(t["charges"]["mean_pe_rel"]) < 3e-3
    assert abs(t["pulses"]["mean_pe_rel"]) < 3e-3
    assert t["pulses"]["matched_frac"] > 0.995
    assert t["pulses"]["time_abs_err_ns_p50_p99_max"][1] < 0.05
    assert t["digis"]["matched_frac"] > 0.999
    assert t["digis"]["adc_mismatch_rate"] < 1e-3
    # where the SiPM charges agree, ADC mismatches are one-count flips at a quantisation boundary, but for the rare
    # sample where the SiPM stage's FP32 times move a charge across a template step (reproduced exactly by the FP64
    # digitisation of the FP32 charges)
    same = t["digis"]["same_charges"]
    assert same["adc_mismatch_at_boundary_frac"] >= 0.9
    assert same["adc_mismatch_rate"] < 1e-3
    assert t["charges"]["sipms_with_different_charges_frac"] < 1e-3
    # the FP32-mixed waveform stage alone, on the FP64 run's own charges: mismatches are one-count flips at a
    # quantisation boundary, but for the rare charge whose FP32 offset from the cluster start lands on the other side
    # of a 0.5 ns template step (1e-5 of the samples at 65,536 events, 2 % of the mismatches there, at most two counts)
    from crvgpu.accuracy import waveform_only_table
    w = waveform_only_table(e32, r64, e32.wcfg.adc_conversion, e32.wcfg.pedestal)
    print(json.dumps(w))
    assert w["matched_frac"] == 1.0 and w["fp32"] == w["fp64"]
    assert w["adc_mismatch_max_abs"] <= 2 and w["adc_mismatch_at_boundary_frac"] >= 0.9
    assert w["adc_mismatch_rate"] < 1e-4
    assert t["clusters"]["same_members_frac"] > 0.98
