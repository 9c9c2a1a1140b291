"""Host-side configuration: validation rules (crv/crvfastsim/response/contract.py:5-29 semantics: invalid settings are
refused before any work) and the reference-config converter.  CPU only."""
import types

import numpy as np
import pytest

from crvgpu import config as C
from crvgpu.chain import from_reference
from crvgpu.params import make_params, validate_sipm, validate_window


def test_thermal_noise_is_refused():
    with pytest.raises(ValueError, match="thermal_rate"):
        validate_sipm(C.SiPMConfig(thermal_rate=1e-3))


@pytest.mark.parametrize("kw", [dict(pixel_id="square"), dict(n_pixels_x=30)])
def test_unsupported_pixel_layouts_are_refused(kw):
    with pytest.raises(ValueError):
        validate_sipm(C.SiPMConfig(**kw))


@pytest.mark.parametrize("pid, flag", [("truncate", 0), ("lrint", 1)])
def test_both_reference_pixel_id_rules_are_accepted(pid, flag):
    """crv/crvfastsim/response/sipm.py:23 PIXEL_IDS; the rule reaches the kernels as CrvParams.pixel_lrint."""
    sc = C.SiPMConfig(pixel_id=pid)
    validate_sipm(sc)
    assert make_params(C.ChainConfig(sipm=sc), 1).pixel_lrint == flag
    assert set(C.PIXEL_IDS) == {"lrint", "truncate"}


@pytest.mark.parametrize("w", [(10.0, 5.0), (0.0, float("inf")), (0.0,), (float("nan"), 1.0)])
def test_bad_windows_are_refused(w):
    with pytest.raises(ValueError):
        validate_window(w)


def test_defaults_are_the_workload_values():
    P = make_params(C.ChainConfig(), 7)
    assert P.seed == 7
    assert C.WaveformConfig().period == 12.55 and C.RecoConfig().period == 12.55
    assert C.WaveformConfig().min_voltage == pytest.approx(5 * 0.0055)
    assert C.WORKLOAD_CUTS.coincidence_layers == 3 and C.WORKLOAD_CUTS.max_dt == 10
    assert C.SiPMConfig().cross_talk == 0.05 and C.SiPMConfig().trap0_prob == 0.02


def test_from_reference_carries_same_named_fields():
    ref = types.SimpleNamespace(
        sipm=types.SimpleNamespace(cross_talk=0.1, time_constant=12.0, jax_only=1),
        window=(0.0, 1e5), noise=False, jax=True, rounds=3, feb_phase_width=12.5, feb_phase_key="feb",
        waveform=types.SimpleNamespace(noise=1e-3, samples_zs=10),
        pulse_reco=types.SimpleNamespace(max_pulses=4, min_beta=4.0),
        finder=None,
        response=types.SimpleNamespace(photon_yield_scale=1.2, tables="v6"))
    c = from_reference(ref, precision="fp32")
    assert c.sipm.cross_talk == 0.1 and c.sipm.time_constant == 12.0 and c.sipm.trap0_prob == 0.02
    assert c.window == (0.0, 1e5) and c.noise is False and c.feb_phase_key == "feb"
    assert c.waveform.noise == 1e-3 and c.waveform.samples_zs == 10 and c.waveform.period == 12.55
    assert c.pulse_reco.max_pulses == 4 and c.pulse_reco.min_beta == 4.0
    assert c.finder is None and c.response.photon_yield_scale == 1.2 and c.precision == "fp32"


def test_from_reference_carries_the_pixel_id_rule():
    """The reference's SiPMConfig defaults to "lrint" (crv/crvfastsim/response/sipm.py:42): carried over, accepted,
    and passed to the kernels."""
    ref = types.SimpleNamespace(sipm=types.SimpleNamespace(pixel_id="lrint", cross_talk=0.05), window=(0.0, 1e5))
    c = from_reference(ref)
    assert c.sipm.pixel_id == "lrint"
    validate_sipm(c.sipm)
    assert make_params(c, 3).pixel_lrint == 1
    assert make_params(from_reference(types.SimpleNamespace(window=(0.0, 1e5))), 3).pixel_lrint == 0


@pytest.mark.parametrize("kw, match", [(dict(feb_phase_key="roc"), "phase key"),
                                       (dict(feb_phase_width=13.0), "phase width"),
                                       (dict(feb_phase_width=-0.1), "phase width"),
                                       (dict(feb_phase_width=float("nan")), "phase width")])
def test_bad_feb_phase_settings_are_refused(kw, match):
    """crv/crvfastsim/chain.py:223-226: an unknown phase key or a width outside [0, period] is a ValueError."""
    with pytest.raises(ValueError, match=match):
        make_params(C.ChainConfig(**kw), 1)
    assert make_params(C.ChainConfig(feb_phase_key="feb", feb_phase_width=0.0), 1).feb_key_mode == 1
    assert make_params(C.ChainConfig(), 1).feb_phase_width == C.WaveformConfig().period


@pytest.mark.parametrize("weights", [np.zeros((40, 40)), np.ones((41, 41)), -np.ones((40, 40)),
                                     np.full((40, 40), np.nan), np.full((40, 40), np.inf)])
def test_photon_maps_outside_the_capability_are_refused(weights):
    """crv/crvfastsim/response_config.py:288-290: finite, non-negative 40 x 40 weights with a positive sum."""
    from crvgpu.response import check_photon_map
    with pytest.raises(ValueError, match="photon_map"):
        check_photon_map(weights)
    check_photon_map(np.ones((40, 40)))
    one = np.zeros((40, 40))
    one[39, 39] = 1.0
    check_photon_map(one)


def test_knobs_follow_the_reference_table_and_semantics():
    """apply_knobs (crv/crvfastsim/chain.py:91-144): the reference's knob names; each sets its block's field; yield
    knobs change the lookup-table block's sectors (yield_TAG every tagger M1..M8); propagation ratios must be positive;
    unknown names raise KeyError."""
    from types import SimpleNamespace
    from crvgpu import config as CF
    prop = ("EX", "T1", "T2", "TAG", "EX0", "EX1", "EX2", "EX3", "T10", "T11", "T20", "T21") + \
        tuple(f"M{i}" for i in range(1, 9))
    names = {"photon_yield_scale", "time_constant", "cross_talk", "min_voltage", "wf_noise", "pe_stretch",
             "background_scale", "yield_EX", "yield_T1", "yield_T2", "yield_TAG"} | \
        {f"{q}_{n}" for q in ("speed", "atten") for n in prop}
    assert set(CF.KNOBS) == names
    sec = lambda y: SimpleNamespace(table="t", reflector=0, yield_per_mev=y)  # noqa: E731
    lk = SimpleNamespace(sectors={"EX": sec(1.0), "T1": sec(2.0), **{f"M{i}": sec(3.0) for i in range(1, 9)}},
                         photon_yield_scale=1.0, speed_ratio={}, atten_ratio={"EX": 0.5})
    base = CF.ChainConfig(lookup=lk)
    cfg = CF.apply_knobs(base, {"photon_yield_scale": 1.2, "time_constant": 11.0, "cross_talk": 0.03,
                                "min_voltage": 0.01, "wf_noise": 5e-4, "pe_stretch": 1.1, "background_scale": 2.0,
                                "yield_TAG": 4.0, "yield_EX": 5.0, "speed_EX1": 0.9, "atten_EX": 1.1})
    assert cfg.response.photon_yield_scale == 1.2 and cfg.lookup.photon_yield_scale == 1.2
    assert cfg.sipm.time_constant == 11.0 and cfg.sipm.cross_talk == 0.03
    assert (cfg.waveform.min_voltage, cfg.waveform.noise, cfg.waveform.single_pe_stretch) == (0.01, 5e-4, 1.1)
    assert cfg.background_scale == 2.0
    assert all(cfg.lookup.sectors[f"M{i}"].yield_per_mev == 4.0 for i in range(1, 9))
    assert cfg.lookup.sectors["EX"].yield_per_mev == 5.0 and cfg.lookup.sectors["T1"].yield_per_mev == 2.0
    assert cfg.lookup.speed_ratio == {"EX1": 0.9} and cfg.lookup.atten_ratio == {"EX": 1.1}
    assert lk.sectors["EX"].yield_per_mev == 1.0 and base.sipm.time_constant != 11.0   # inputs untouched
    with pytest.raises(KeyError, match="unknown knob"):
        CF.apply_knobs(base, {"nope": 1})
    with pytest.raises(ValueError):
        CF.apply_knobs(base, {"speed_EX": 0.0})
    with pytest.raises(ValueError):
        CF.apply_knobs(CF.ChainConfig(), {"yield_EX": 3.0})
    assert CF.apply_knobs(CF.ChainConfig(), {}).waveform == CF.WaveformConfig()
