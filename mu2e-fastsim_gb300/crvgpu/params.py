"""Pack the configuration dataclasses into the C ABI's CrvParams (every physics knob is runtime data)."""
from __future__ import annotations

import numpy as np

from . import _capi
from .config import (FEB_PHASE_KEYS, PERIOD, PIXEL_IDS, ChainConfig, FinderConfig, RecoConfig, ResponseConfig, SiPMConfig, WaveformConfig)


def p_fire(sc, v):
    return sc.p1 * (1.0 - np.exp(-v / sc.p2))


def validate_sipm(sc):
    """The engine implements cross-talk and both trap afterpulses; dark noise is not part of this chain
    (the reference's contract refuses it as well, crv/crvfastsim/response/contract.py:5-12)."""
    if sc.thermal_rate != 0:
        raise ValueError("CRV response: unsupported SiPM processes: ['thermal_rate']")
    if getattr(sc, "pixel_id", "truncate") not in PIXEL_IDS:
        raise ValueError(f"CRV response: SiPM pixel_id must be one of {PIXEL_IDS}, got {sc.pixel_id!r}")
    if sc.n_pixels_x != 40 or sc.n_pixels_y != 40:
        raise ValueError("CRV response: the pixel grid is 40 x 40")


def validate_feb_phase(width, key, period):
    """The TDC0 phase settings (crv/crvfastsim/chain.py:223-226): width finite in [0, period], a known key."""
    if not np.isfinite(width) or not 0 <= width <= period:
        raise ValueError(f"FEB phase width must be finite and in [0, {period}] ns, got {width}")
    if key not in FEB_PHASE_KEYS:
        raise ValueError(f"FEB phase key must be one of {FEB_PHASE_KEYS}, got {key!r}")


def validate_window(window):
    w = np.asarray(window, dtype=float)
    if w.shape != (2,) or not np.isfinite(w).all() or w[1] <= w[0]:
        raise ValueError("CRV response: window must contain finite, increasing bounds")


def make_params(cfg: ChainConfig = None, seed: int = 0, *, response: ResponseConfig = None, sipm: SiPMConfig = None,
                waveform: WaveformConfig = None, reco: RecoConfig = None, finder: FinderConfig = None,
                window=None, precision=None, t_end=None, template_len=0, uniform_map=True, charge_factor=1):
    cfg = cfg or ChainConfig()
    rc = response or cfg.response
    sc = sipm or cfg.sipm
    wc = waveform or cfg.waveform or WaveformConfig()
    pc = reco or cfg.pulse_reco or RecoConfig()
    fc = finder or cfg.finder or FinderConfig()
    win = window if window is not None else cfg.window
    prec = precision if precision is not None else cfg.precision
    if prec not in ("fp64", "fp32"):
        raise ValueError(f"precision must be 'fp64' or 'fp32', got {prec!r}")
    P = _capi.CrvParams()
    P.seed = int(seed) & 0xFFFFFFFF
    P.precision = 1 if prec == "fp32" else 0
    P.yield_per_mev = rc.yield_per_mev
    P.frac_short = rc.frac_short
    P.frac_long = 1.0 - rc.frac_short
    P.lambda_short = rc.lambda_short
    P.lambda_long = rc.lambda_long
    P.signal_speed = rc.signal_speed
    P.decay_time = rc.decay_time
    pf = float(p_fire(sc, sc.overvoltage))
    P.overvoltage, P.time_constant, P.capacitance, P.p1, P.p2 = (sc.overvoltage, sc.time_constant, sc.capacitance,
                                                                 sc.p1, sc.p2)
    P.q_ct = (1.0 - (1.0 - sc.cross_talk) ** 0.25) / pf
    P.q_t0 = sc.trap0_prob / pf
    P.q_t1 = sc.trap1_prob / pf
    P.trap0_lifetime, P.trap1_lifetime = sc.trap0_lifetime, sc.trap1_lifetime
    P.t_end = float(t_end if t_end is not None else win[1])
    P.n_pixels_x, P.n_pixels_y = sc.n_pixels_x, sc.n_pixels_y
    P.uniform_map = 1 if uniform_map else 0
    P.pixel_lrint = 1 if getattr(sc, "pixel_id", "truncate") == "lrint" else 0
    P.charge_factor = int(charge_factor)
    period = getattr(wc, "period", PERIOD)
    P.period = period
    P.spe_precision = wc.single_pe_precision
    P.spe_max_time = wc.single_pe_max_time
    P.spe_ref_charge = wc.single_pe_reference_charge
    P.min_voltage = wc.min_voltage
    P.noise_sigma = wc.noise
    P.adc_conversion = wc.adc_conversion
    P.window_lo, P.window_hi = float(win[0]), float(win[1])
    P.feb_phase_width = period if cfg.feb_phase_width is None else float(cfg.feb_phase_width)
    validate_feb_phase(P.feb_phase_width, cfg.feb_phase_key, period)
    P.samples_zs, P.adc_pedestal, P.min_adc, P.max_adc = wc.samples_zs, wc.pedestal, wc.min_adc, wc.max_adc
    P.template_len = int(template_len)
    P.feb_key_mode = 1 if cfg.feb_phase_key == "feb" else 0
    P.noise_on = 1 if cfg.noise else 0
    P.min_adc_difference, P.default_beta, P.min_beta, P.max_beta = (pc.min_adc_difference, pc.default_beta,
                                                                    pc.min_beta, pc.max_beta)
    P.max_time_difference, P.min_height_ratio, P.max_height_ratio = (pc.max_time_difference,
                                                                     pc.min_pulse_height_ratio,
                                                                     pc.max_pulse_height_ratio)
    P.le_time_factor, P.pedestal_undershoot, P.time_offset_scale = (pc.le_time_factor,
                                                                    pc.pedestal_undershoot_threshold,
                                                                    pc.time_offset_scale)
    P.limit_tolerance, P.knife_edge_adc = pc.limit_tolerance, pc.knife_edge_adc
    P.samples_before, P.samples_after, P.max_pulses, P.lm_iterations = (pc.samples_before, pc.samples_after,
                                                                        pc.max_pulses, pc.lm_iterations)
    P.use_time_offset_db = 1 if pc.use_time_offset_db else 0
    P.ignore_channels = 1 if pc.ignore_channels else 0
    P.fiber_signal_speed, P.max_time_interval, P.time_offset = (fc.fiber_signal_speed, fc.max_time_interval,
                                                                fc.time_offset)
    P.compensate_mask = sum(1 << b for b in fc.compensate_status_bits)
    P.ignore_secondary = 1 if fc.ignore_secondary_pulses else 0
    P.big_cluster_threshold = fc.big_cluster_threshold
    P.add_opposite = 1 if fc.add_opposite_side_pulses else 0
    return P
