"""Configuration of the CRV response engine.

The dataclasses keep the field names and meanings of the reference stage configurations so that a caller's
existing objects and knob overrides carry over:

  SiPMConfig      crv/crvfastsim/response/sipm.py:26-47
  WaveformConfig  crv/crvfastsim/reco/waveform.py:29-43
  RecoConfig      crv/crvfastsim/reco/pulsefit.py:26-46
  SectorCuts, FinderConfig, SectorGeom   crv/crvfastsim/reco/coinc.py:29-79
  ChainConfig, Conditions                crv/crvfastsim/chain.py:29-84

ResponseConfig replaces the reference's lookup-table photon model (crv/crvfastsim/response/photons.py:45-53) by the
analytic one of the workload: a photon yield per MeV per SiPM and a two-exponential fibre attenuation
frac_short e^(-d/lambda_short) + (1 - frac_short) e^(-d/lambda_long), d the distance from the step to the SiPM's
bar end; arrival time = step time + d / signal_speed + an exponential emission delay (decay_time).

Defaults are the workload's values where it names one (12.55 ns sampling, 40 PE/MeV, attenuation 100/500 cm with
fractions 0.3/0.7, cross-talk 0.05, afterpulses 0.02, 5 PE threshold, 3 of 4 layers within 10 ns) and the
reference's stock values otherwise.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import Optional

import numpy as np

CHAN_MULT = 32768          # SiPM label = event key * CHAN_MULT + channel (crv/crvfastsim/chain.py:25)
PERIOD = 12.55             # digitisation period [ns] of the workload (the reference module constant is 12.5)
NPIX = 41                  # pixels per side of the SiPM pixel state (crv/crvfastsim/response/sipm.py:22): ids
                           # x * 41 + y; the 40 x 40 grid minus the inactive 4 x 4 centre leaves 1,584 live pixels,
                           # the 41st row and column are reached by the "lrint" rule only
SPE_PEAK_VOLT = 0.0055     # single-PE peak voltage of the Gumbel template [V]


@dataclass
class ResponseConfig:
    yield_per_mev: float = 40.0          # PE per MeV deposited, per SiPM, at zero attenuation
    frac_short: float = 0.3
    lambda_short: float = 1000.0         # mm
    lambda_long: float = 5000.0          # mm
    signal_speed: float = 140.0          # mm/ns along the fibre
    decay_time: float = 7.4              # ns, exponential emission delay per photon
    photon_yield_scale: float = 1.0
    photon_yield_variation_scale: float = 1.0


# TDC0 phase per (event, ROC, FEB) or per (event, FEB number) across ROCs (crv/crvfastsim/chain.py:216-231)
FEB_PHASE_KEYS = ("roc_feb", "feb")
PIXEL_IDS = ("lrint", "truncate")          # crv/crvfastsim/response/sipm.py:23


@dataclass
class SiPMConfig:
    n_pixels_x: int = 40
    n_pixels_y: int = 40
    overvoltage: float = 3.0
    time_constant: float = 13.3
    capacitance: float = 8.84e-14
    p1: float = 0.607
    p2: float = 2.7
    cross_talk: float = 0.05
    thermal_rate: float = 0.0
    trap0_prob: float = 0.02
    trap1_prob: float = 0.0
    trap0_lifetime: float = 5.0
    trap1_lifetime: float = 50.0
    inactive: tuple = field(default_factory=lambda: tuple((x, y) for x in range(18, 22) for y in range(18, 22)))
    pixel_id: str = "truncate"

    def p_fire(self, v):
        return self.p1 * (1.0 - np.exp(-np.asarray(v) / self.p2))


@dataclass(frozen=True)
class WaveformConfig:
    single_pe_file: Optional[str] = None      # (t, v) text file; None = Gumbel single-PE shape below
    single_pe_precision: float = 0.5
    single_pe_stretch: float = 1.0
    single_pe_max_time: float = 100.0
    single_pe_reference_charge: float = 2.652e-13
    min_voltage: float = 5 * SPE_PEAK_VOLT    # readout threshold: 5 PE
    noise: float = 4.0e-4
    samples_zs: int = 12
    adc_conversion: float = 2300.0
    pedestal: int = 100
    min_adc: int = 0
    max_adc: int = 4095
    gumbel_peak: float = SPE_PEAK_VOLT
    gumbel_mu: float = 15.0
    gumbel_beta: float = 10.0
    period: float = PERIOD


@dataclass(frozen=True)
class RecoConfig:
    min_adc_difference: float = 40.0
    default_beta: float = 19.0
    min_beta: float = 5.0
    max_beta: float = 40.0
    max_time_difference: float = 15.0
    min_pulse_height_ratio: float = 0.7
    max_pulse_height_ratio: float = 1.5
    le_time_factor: float = 0.985
    samples_before: int = 4
    samples_after: int = 3
    pedestal_undershoot_threshold: float = 6.0
    use_time_offset_db: bool = True
    time_offset_scale: float = 1.0
    ignore_channels: bool = True
    max_pulses: int = 8
    lm_iterations: int = 40
    limit_tolerance: float = 0.01
    knife_edge_adc: float = 1.0
    period: float = PERIOD


@dataclass(frozen=True)
class SectorCuts:
    pe_threshold: float
    max_dt_adjacent: float
    max_dt: float
    min_slope: float
    max_slope: float
    max_slope_diff: float
    coincidence_layers: int
    min_cluster_pes: float
    initial_max_distance: float
    final_max_distance: float


# the workload's coincidence: >= 3 of 4 layers within 10 ns; other cuts as the reference's extracted-v04 EX sector
WORKLOAD_CUTS = SectorCuts(8, 10, 10, -6, 6, 3, 3, 0, 250, 0)


@dataclass(frozen=True)
class FinderConfig:
    fiber_signal_speed: float = 140.0
    max_time_interval: float = 20.0
    time_offset: float = 34.5
    compensate_status_bits: tuple = (0, 1, 2)
    ignore_secondary_pulses: bool = True
    big_cluster_threshold: int = 50000
    cuts: dict = field(default_factory=lambda: {"EX": WORKLOAD_CUTS})
    add_opposite_side_pulses: bool = True


@dataclass
class SectorGeom:
    sector: np.ndarray
    layer: np.ndarray
    counter_in_type: np.ndarray
    x: np.ndarray
    y: np.ndarray
    pos: np.ndarray
    length_dir: np.ndarray
    sector_type: np.ndarray
    sector_names: list
    pos_side0: np.ndarray
    pos_side1: np.ndarray
    sipms_side0: np.ndarray
    sipms_side1: np.ndarray


@dataclass
class Conditions:
    pedestal: np.ndarray
    pulsearea: np.ndarray
    pulseheight: np.ndarray
    timeoffset: np.ndarray
    status: np.ndarray
    roc: np.ndarray
    feb: np.ndarray
    deviation: np.ndarray
    readout_mask: Optional[np.ndarray] = None

    @staticmethod
    def from_csv(calib_csv, photon_csv=None):
        """Conditions.from_csv (crv/crvfastsim/chain.py:42-51): per-channel CSV rows channel, pedestal, pulsearea,
        pulseheight, timeoffset, status, roc, feb[, febch] (e.g. dumped from crvdump/calib), dense by channel;
        yield deviations from an optional channel, deviation CSV."""
        a = np.loadtxt(calib_csv, delimiter=",", comments="#", ndmin=2)
        n = int(a[:, 0].max()) + 1 if a.size else 0

        def col(j, dt=float):
            out = np.zeros(n, dt)
            if a.size:
                out[a[:, 0].astype(int)] = a[:, j]
            return out
        dev = np.zeros(n)
        if photon_csv:
            p = np.loadtxt(photon_csv, delimiter=",", comments="#", ndmin=2)
            dev[p[:, 0].astype(int)] = p[:, 1]
        return Conditions(col(1), col(2), col(3), col(4), col(5, np.int64), col(6, np.int64), col(7, np.int64), dev)


PRECISIONS = ("fp64", "fp32")


@dataclass
class ChainConfig:
    response: ResponseConfig = field(default_factory=ResponseConfig)
    finder: object = None
    sipm: SiPMConfig = field(default_factory=SiPMConfig)
    window: tuple = (0.0, 128 * PERIOD)
    noise: bool = True
    waveform: object = None
    pulse_reco: object = None
    feb_phase_width: Optional[float] = None    # None = one digitisation period
    feb_phase_key: str = "roc_feb"            # FEB_PHASE_KEYS
    backend: str = "cuda"
    precision: str = "fp64"                     # "fp64" plain, or "fp32" mixed (float-float LM solve, FP64 times)
    # the reference's lookup-table response block (sectors {name: (table, reflector, yield_per_mev)}, yield scales,
    # speed / attenuation ratios): charges() runs the lookup-table photon model with it when given lookup tables
    lookup: object = None
    # the background model's rate factor (the reference's knob); inert: this engine takes no background overlays
    background_scale: float = 1.0


# light-propagation keys of the reference's knobs (crv/crvfastsim/chain.py:88-89): sectors, TAG = every muon tagger,
# and modules
PROP_KEYS = (("EX", "T1", "T2", "TAG") + tuple(f"EX{i}" for i in range(4)) + ("T10", "T11", "T20", "T21")
             + tuple(f"M{i}" for i in range(1, 9)))
# the reference's design-point knobs (crv/crvfastsim/chain.py:91-97): name -> (block, field) of this engine's config;
# "response" sets the analytic model's field and the lookup-table block's; sector yields and light-propagation ratios
# live in the lookup-table block
KNOBS = {"photon_yield_scale": ("response", "photon_yield_scale"), "time_constant": ("sipm", "time_constant"),
         "cross_talk": ("sipm", "cross_talk"), "min_voltage": ("waveform", "min_voltage"),
         "wf_noise": ("waveform", "noise"), "pe_stretch": ("waveform", "single_pe_stretch"),
         "background_scale": (None, "background_scale"),
         **{f"yield_{n}": ("sector_yield", n) for n in ("EX", "T1", "T2", "TAG")},
         **{f"speed_{n}": ("speed_ratio", n) for n in PROP_KEYS},
         **{f"atten_{n}": ("atten_ratio", n) for n in PROP_KEYS}}


def _with(obj, **kw):
    """A copy of a dataclass or plain-attribute object with fields replaced."""
    import dataclasses
    import types
    if dataclasses.is_dataclass(obj):
        return dataclasses.replace(obj, **kw)
    return types.SimpleNamespace(**{**vars(obj), **kw})


def apply_knobs(cfg: "ChainConfig", knobs) -> "ChainConfig":
    """ChainConfig with knob overrides {name: value} (KNOBS), as the reference's apply_knobs
    (crv/crvfastsim/chain.py:117-144): unknown names raise KeyError, non-positive propagation ratios ValueError.  A
    sector-yield or propagation knob needs the lookup-table response block (cfg.lookup), whose sectors they change
    (yield_TAG: every muon tagger M1..M8)."""
    if cfg.waveform is None:
        cfg = replace(cfg, waveform=WaveformConfig())
    for k, v in (knobs or {}).items():
        if k not in KNOBS:
            raise KeyError(f"unknown knob {k}; known: {sorted(KNOBS)}")
        blk, fld = KNOBS[k]
        if blk in ("sector_yield", "speed_ratio", "atten_ratio"):
            if cfg.lookup is None:
                raise ValueError(f"knob {k} acts on the lookup-table response block (ChainConfig.lookup): unset")
            if blk == "sector_yield":
                names = [f"M{i}" for i in range(1, 9)] if fld == "TAG" else [fld]
                secs = dict(cfg.lookup.sectors)
                for nm in names:
                    secs[nm] = _with(secs[nm], yield_per_mev=float(v))
                cfg = replace(cfg, lookup=_with(cfg.lookup, sectors=secs))
            else:
                if not float(v) > 0:
                    raise ValueError(f"knob {k} must be positive, got {v}")
                d = {**(getattr(cfg.lookup, blk, None) or {}), fld: float(v)}
                cfg = replace(cfg, lookup=_with(cfg.lookup, **{blk: d}))
            continue
        if blk is None:
            cfg = replace(cfg, **{fld: float(v)})
        elif blk == "response":
            cfg = replace(cfg, response=replace(cfg.response, **{fld: float(v)}),
                          lookup=_with(cfg.lookup, **{fld: float(v)}) if cfg.lookup is not None else None)
        else:
            cfg = replace(cfg, **{blk: replace(getattr(cfg, blk), **{fld: float(v)})})
    return cfg


def _fields_of(cls, obj, **over):
    """cls(**{same-named attributes of obj that cls has}) with overrides; obj None -> None."""
    if obj is None:
        return None
    from dataclasses import fields
    kw = {f.name: getattr(obj, f.name) for f in fields(cls) if hasattr(obj, f.name)}
    kw.update(over)
    return cls(**kw)


def from_reference(cfg, precision="fp64"):
    """ChainConfig of this engine from a reference ChainConfig (crv/crvfastsim/chain.py:62-84) or any object with its
    field names: same-named fields of the chain, SiPM (pixel-id rule included), waveform, reco and finder blocks are
    carried over; the reference's lookup-table response block (sectors with table, reflector and yield) is kept as
    `lookup` and selects the lookup-table photon model when tables are passed, its yield scales also set the analytic
    model's; JAX switches have no meaning here and are dropped."""
    resp = getattr(cfg, "response", None)
    rc = ResponseConfig(**{k: getattr(resp, k) for k in ("photon_yield_scale", "photon_yield_variation_scale")
                           if hasattr(resp, k)})
    kw = dict(response=rc, precision=precision, lookup=resp if hasattr(resp, "sectors") else None,
              sipm=_fields_of(SiPMConfig, getattr(cfg, "sipm", None)) or SiPMConfig(),
              waveform=_fields_of(WaveformConfig, getattr(cfg, "waveform", None)),
              pulse_reco=_fields_of(RecoConfig, getattr(cfg, "pulse_reco", None)),
              finder=_fields_of(FinderConfig, getattr(cfg, "finder", None)))
    for k in ("window", "noise", "feb_phase_width", "feb_phase_key", "background_scale"):
        if hasattr(cfg, k):
            kw[k] = getattr(cfg, k)
    return ChainConfig(**kw)


def workload_finder(sector_names, base: FinderConfig = None) -> FinderConfig:
    """FinderConfig with the workload's coincidence cuts (3 of 4 layers within 10 ns) for every sector name."""
    base = base or FinderConfig()
    return replace(base, cuts={str(n): WORKLOAD_CUTS for n in sector_names})
