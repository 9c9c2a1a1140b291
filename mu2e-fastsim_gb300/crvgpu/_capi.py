"""ctypes binding of libcrvgpu.so (include/crvgpu.h).

The library is the only compute path of this package: if it is missing, cannot be loaded, or no CUDA device is
present, every entry point raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

c_i32, c_i64, c_u32, c_f64, c_p = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32, ctypes.c_double, ctypes.c_void_p

CRV_OK, CRV_ERR_ARG, CRV_ERR_CUDA, CRV_ERR_TOO_LARGE = 0, 1, 2, 3
PULSES_STATIC_MAX_BYTES = 64 << 20
ST_CAPACITY, ST_LIMIT, ST_NONFINITE, ST_ORDER, ST_BOUNDS = 1, 2, 4, 8, 16
NEED = dict(STEPS_PER_EVENT=0, PHOTONS_PER_SIPM=1, CHARGE_FACTOR=2, DIGIS=3, SAMPLES=4, PULSES=5, HITS_PER_EVENT=6,
            CLUSTERS=7, PHOTONS_TOTAL=8, SLOTS_TOTAL=9, CHARGES_OUT=10, DIGIS_OUT=11, WAVEFORMS=12, PULSES_OUT=13,
            MEMBERS=14, PHOTONS_OUT=15)


class CrvStatus(ctypes.Structure):
    _fields_ = [("flags", c_i32), ("pad", c_i32), ("need", c_i64 * 16)]


_PARAM_FIELDS = [
    ("seed", c_u32), ("precision", c_i32),
    *[(n, c_f64) for n in ("yield_per_mev", "frac_short", "frac_long", "lambda_short", "lambda_long", "signal_speed",
                           "decay_time")],
    *[(n, c_f64) for n in ("overvoltage", "time_constant", "capacitance", "p1", "p2", "q_ct", "q_t0", "q_t1",
                           "trap0_lifetime", "trap1_lifetime", "t_end")],
    ("n_pixels_x", c_i32), ("n_pixels_y", c_i32), ("uniform_map", c_i32), ("charge_factor", c_i32),
    *[(n, c_f64) for n in ("period", "spe_precision", "spe_max_time", "spe_ref_charge", "min_voltage", "noise_sigma",
                           "adc_conversion", "window_lo", "window_hi", "feb_phase_width")],
    *[(n, c_i32) for n in ("samples_zs", "adc_pedestal", "min_adc", "max_adc", "template_len", "feb_key_mode",
                           "noise_on", "pixel_lrint")],
    *[(n, c_f64) for n in ("min_adc_difference", "default_beta", "min_beta", "max_beta", "max_time_difference",
                           "min_height_ratio", "max_height_ratio", "le_time_factor", "pedestal_undershoot",
                           "time_offset_scale", "limit_tolerance", "knife_edge_adc")],
    *[(n, c_i32) for n in ("samples_before", "samples_after", "max_pulses", "lm_iterations", "use_time_offset_db",
                           "ignore_channels")],
    *[(n, c_f64) for n in ("fiber_signal_speed", "max_time_interval", "time_offset")],
    *[(n, c_i32) for n in ("compensate_mask", "ignore_secondary", "big_cluster_threshold", "add_opposite")],
]


class CrvParams(ctypes.Structure):
    _fields_ = _PARAM_FIELDS


class CrvEvents(ctypes.Structure):
    _fields_ = [("event", c_p), ("subrun", c_p), ("run", c_p), ("first_step", c_p), ("nsteps", c_p)]


class CrvSteps(ctypes.Structure):
    _fields_ = [("x", c_p), ("y", c_p), ("z", c_p), ("t", c_p), ("edep", c_p), ("bar", c_p), ("real_bytes", c_i32),
                ("pad", c_i32)]


class CrvBars(ctypes.Structure):
    _fields_ = [("length_axis", c_p), ("center_l", c_p), ("half_l", c_p), ("nbars", c_i32), ("pad", c_i32)]


class CrvChannels(ctypes.Structure):
    _fields_ = [("yield_factor", c_p), ("status", c_p), ("roc", c_p), ("feb", c_p), ("pedestal", c_p),
                ("pulsearea", c_p), ("pulseheight", c_p), ("timeoffset", c_p), ("nchan", c_i32), ("pad", c_i32)]


class CrvPixels(ctypes.Structure):
    _fields_ = [("cum", c_p), ("dead_bits", c_p)]


class CrvCharges(ctypes.Structure):
    _fields_ = [("label", c_p), ("time", c_p), ("charge", c_p), ("pe", c_p), ("photon", c_p)]


class CrvDigis(ctypes.Structure):
    _fields_ = [("chan", c_p), ("start", c_p), ("tdc0", c_p), ("starttdc", c_p), ("volt", c_p), ("adc", c_p)]


PULSE_INT = ("wf", "seq")
PULSE_FLOAT = ("pe", "peph", "time", "height", "beta", "chi2", "letime", "ped", "fit_A", "fit_mu", "fit_b")
PULSE_BOOL = ("failed", "zerondf", "pedfromdb")


class CrvPulses(ctypes.Structure):
    _fields_ = [(k, c_p) for k in PULSE_INT + PULSE_FLOAT + PULSE_BOOL]


class CrvFinderGeom(ctypes.Structure):
    _fields_ = [(k, c_p) for k in ("bar_sector", "bar_layer", "bar_counter", "bar_x", "bar_y", "bar_pos", "sec_type",
                                   "sec_cut", "sec_length_dir", "sec_pos0", "sec_pos1", "cuts", "type_id", "type_p0",
                                   "type_p1", "type_half", "type_maxdt", "type_side0", "type_side1")] + \
        [("ntypes", c_i32), ("pad", c_i32)]


class CrvClusters(ctypes.Structure):
    _fields_ = [(k, c_p) for k in ("event", "type", "pe", "start", "end", "slope", "avgtime", "poscalc", "pos",
                                   "sidepe", "sidetime", "sidehits", "nlayers")]


class CrvMembers(ctypes.Structure):
    _fields_ = [("cl", c_p), ("idx", c_p), ("event", c_p)]


class CrvLookupTable(ctypes.Structure):
    _fields_ = [(k, c_p) for k in ("prob", "delays", "delay_sum", "emis", "emis_sum")] + \
        [(k, c_i32) for k in ("nbins", "ndelay", "nemis", "pad")]


class CrvLookup(ctypes.Structure):
    _fields_ = [(k, c_f64) for k in ("half_thickness", "half_width", "half_length", "fiber_separation", "hole_radius_x",
                                     "hole_radius_y", "fiber_radius", "corner_radius", "fiber_decay_time")] + \
        [("edges", c_p * 7), ("nedges", c_i32 * 7), ("precision", c_i32), ("cos_phi_edges", c_p),
         ("table", CrvLookupTable * 3), ("cos_theta_edges", c_p)]


class CrvSubstepRows(ctypes.Structure):
    _fields_ = [(k, c_p) for k in ("s", "d", "t0", "t1", "beta", "theta", "dev", "mu", "nsub", "step", "chan",
                                   "n_scint", "n_ck_s", "n_ck_f", "cos_theta")]


LOOKUP_STEP_COLS = ("x0", "y0", "z0", "x1", "y1", "z1", "px0", "py0", "pz0", "p1", "t0", "t1", "edep", "len")
LOOKUP_ROW_COLS = ("s", "d", "t0", "t1", "beta", "cos_theta", "dev", "mu", "nsub", "step", "chan", "n_scint", "n_ck_s",
                   "n_ck_f")


class CrvLookupSteps(ctypes.Structure):
    _fields_ = [(k, c_p) for k in LOOKUP_STEP_COLS + ("bar", "pdg")]


class CrvLookupGroup(ctypes.Structure):
    _fields_ = [(k, c_p) for k in ("center", "l2w", "in_group", "yield_", "speed_k", "mu", "dev", "ck_scint",
                                   "ck_fiber", "pdg_code", "pdg_mass", "pdg_charge")] + \
        [("half_length", c_f64)] + [(k, c_i32) for k in ("reflector", "nbars", "nck_scint", "nck_fiber", "npdg", "pad")]


class CrvSubstepRowsOut(ctypes.Structure):
    _fields_ = [(k, c_p) for k in LOOKUP_ROW_COLS]


LOOKUP_CHAIN_GROUPS = 8


class CrvLookupChain(ctypes.Structure):
    _fields_ = [("steps", CrvLookupSteps), ("ngroups", c_i32), ("pad", c_i32),
                ("group", CrvLookupGroup * LOOKUP_CHAIN_GROUPS), ("table", CrvLookup * LOOKUP_CHAIN_GROUPS)]


# lookup-table file reader (host memory)
LUTF_VERSION, LUTF_BIN_NUMBER, LUTF_TRAILING, LUTF_TRUNCATED, LUTF_SIZE = 1, 2, 3, 4, 5


class CrvLookupFileInfo(ctypes.Structure):
    _fields_ = [("version_major", c_i32), ("version_minor", c_i32), ("reflector", c_i32), ("error", c_i32),
                ("error_a", c_i64), ("error_b", c_i64), ("constants", c_f64 * 10), ("n_ck", c_i64 * 2),
                ("n_edges", c_i64 * 7), ("n_bins", c_i64 * 3), ("delay_width", c_i64 * 3), ("emis_width", c_i64 * 3)]


class CrvLookupFileTable(ctypes.Structure):
    _fields_ = [(k, c_p) for k in ("prob", "delays", "delay_sum", "emis", "emis_sum")]


class CrvLookupFileOut(ctypes.Structure):
    _fields_ = [("ck", c_p * 2), ("edges", c_p * 7), ("tables", CrvLookupFileTable * 3)]


CHAIN_CAPS = ("events", "steps", "photons", "charges", "slots", "digis", "pulses", "max_steps_per_event")
CHAIN_COUNTS = ("charges", "digis", "waveforms", "pulses", "events", "hits", "clusters", "members", "photons",
                "slots")


class CrvChainCaps(ctypes.Structure):
    _fields_ = [(k, c_i64) for k in CHAIN_CAPS[:-1]] + [("max_steps_per_event", c_i32), ("pad", c_i32)]


P = ctypes.POINTER

_SIGS = {
    "crv_version": (c_i32, []),
    "crv_status_string": (ctypes.c_char_p, [c_i32]),
    "crv_launch_count": (ctypes.c_longlong, []),
    "crv_profile": (None, [c_i32]),
    "crv_profile_read": (c_i32, [c_i32, ctypes.c_char_p, P(ctypes.c_float)]),
    "crv_response_workspace": (c_i64, [P(CrvParams), c_i64, c_i64, c_i64, c_i32]),
    "crv_response": (c_i32, [P(CrvParams), P(CrvEvents), c_i64, P(CrvSteps), c_i64, c_i32, P(CrvBars), P(CrvChannels),
                             P(CrvPixels), c_i64, P(CrvCharges), c_i64, c_p, c_p, c_p, c_p, c_i64, c_p, c_p, c_i64,
                             c_p, c_p]),
    "crv_photon_counts": (c_i32, [P(CrvParams), P(CrvEvents), c_i64, P(CrvSteps), c_i64, P(CrvBars), P(CrvChannels),
                                  c_p, c_p, c_p, c_p]),
    "crv_photons": (c_i32, [P(CrvParams), P(CrvEvents), c_i64, P(CrvSteps), c_i64, P(CrvBars), c_p, c_p, c_p, c_p,
                            c_p, c_p, c_p, c_p, c_p]),
    "crv_sipm_workspace": (c_i64, [P(CrvParams), c_i64, c_i64]),
    "crv_digis_workspace": (c_i64, [P(CrvParams), c_i64, c_i64]),
    "crv_digis": (c_i32, [P(CrvParams), P(CrvChannels), c_i64, c_p, c_p, c_p, c_p, c_i32, c_p, c_p, c_i64, c_i64,
                          P(CrvDigis), c_i64, c_p, c_p, c_i64, c_p, c_p]),
    "crv_synthesize": (c_i32, [P(CrvParams), P(CrvChannels), c_i64, c_p, c_p, c_p, c_p, c_p, c_i32, c_i64, P(CrvDigis),
                               c_i64, c_p, c_p, c_i64, c_p, c_p]),
    "crv_tdc0_per_feb": (c_i32, [P(CrvParams), P(CrvChannels), c_i64, c_p, c_p, c_p, c_i64, c_p, c_p, c_p]),
    "crv_pulses_workspace": (c_i64, [P(CrvParams), c_i64, c_i64]),
    "crv_pulses": (c_i32, [P(CrvParams), c_i64, c_i64, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_i32, P(CrvPulses),
                           c_i64, c_p, c_p, c_p, c_i64, c_p, c_p]),
    "crv_pulses_shape": (c_i32, [c_i32, c_i32, c_i32]),
    "crv_pulses_static": (c_i32, [P(CrvParams), c_i64, c_i64, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_i32,
                                  P(CrvPulses), c_i64, c_p, c_p, c_p, c_p]),
    "crv_coincidences_workspace": (c_i64, [c_i64, c_i64]),
    "crv_coincidences": (c_i32, [P(CrvParams), P(CrvFinderGeom), c_i64, c_p, c_p, c_p, c_i64, c_p, c_p, c_p, c_p, c_p,
                                 c_p, P(CrvClusters), c_i64, c_p, P(CrvMembers), c_i64, c_p, c_p, c_i64, c_p, c_p]),
    "crv_reco_waveforms_workspace": (c_i64, [c_i64]),
    "crv_reco_waveforms": (c_i32, [P(CrvParams), P(CrvChannels), c_i64, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_p,
                                   c_p, c_p, c_p, c_i64, c_p, c_p]),
    "crv_pulse_hits_workspace": (c_i64, [c_i64]),
    "crv_pulse_hits": (c_i32, [P(CrvParams), c_p, c_i64, c_p, c_p, c_p, c_i64, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_p,
                               c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_i64, c_p, c_p]),
    "crv_sipm": (c_i32, [P(CrvParams), P(CrvPixels), c_i64, c_i64, c_p, c_p, c_p, c_p, c_p, c_p, c_p, P(CrvCharges),
                         c_i64, c_p, c_p, c_p, c_p, c_i64, c_p, c_p]),
    "crv_chain_workspace": (c_i64, [P(CrvParams), P(CrvChainCaps)]),
    "crv_substeps_workspace": (c_i64, [c_i64]),
    "crv_lookup_rows_workspace": (c_i64, [c_i64]),
    "crv_lookup_rows": (c_i32, [P(CrvLookupGroup), c_u32, P(CrvLookupSteps), c_i64, P(CrvSubstepRowsOut), c_i64, c_p,
                                c_p, c_i64, c_p, c_p]),
    "crv_substep_photons": (c_i32, [P(CrvLookup), c_u32, P(CrvSubstepRows), c_i64, c_p, c_p, c_p, c_i64, c_p, c_p,
                                    c_i64, c_p, c_p]),
    "crv_lookup_file_info": (c_i32, [c_p, c_i64, P(CrvLookupFileInfo)]),
    "crv_lookup_file_read": (c_i32, [c_p, c_i64, P(CrvLookupFileInfo), P(CrvLookupFileOut)]),
    "crv_lz4_block_decompress": (c_i64, [c_p, c_i64, c_p, c_i64]),
    "crv_xxh64": (ctypes.c_uint64, [c_p, c_i64, ctypes.c_uint64]),
    "crv_chain": (c_i32, [P(CrvParams), P(CrvChainCaps), P(CrvEvents), c_p, c_p, P(CrvSteps), c_p, P(CrvBars),
                          P(CrvChannels), P(CrvPixels), c_p, c_i32, P(CrvFinderGeom), P(CrvClusters), P(CrvMembers),
                          c_p, c_p, c_i64, c_p, c_p]),
    "crv_chain_graph_create": (c_i32, [P(CrvParams), P(CrvChainCaps), P(CrvEvents), c_p, c_p, P(CrvSteps), c_p,
                                       P(CrvBars), P(CrvChannels), P(CrvPixels), c_p, c_i32, P(CrvFinderGeom),
                                       P(CrvClusters), P(CrvMembers), c_p, c_p, c_i64, c_p, c_p, P(c_p)]),
    "crv_chain_lookup_workspace": (c_i64, [P(CrvParams), P(CrvChainCaps)]),
    "crv_chain_lookup": (c_i32, [P(CrvParams), P(CrvChainCaps), P(CrvEvents), c_p, c_p, P(CrvSteps), c_p, P(CrvBars),
                                 P(CrvChannels), P(CrvPixels), c_p, c_i32, P(CrvFinderGeom), P(CrvClusters),
                                 P(CrvMembers), c_p, c_p, c_i64, c_p, c_p, P(CrvLookupChain)]),
    "crv_chain_graph_create_lookup": (c_i32, [P(CrvParams), P(CrvChainCaps), P(CrvEvents), c_p, c_p, P(CrvSteps), c_p,
                                              P(CrvBars), P(CrvChannels), P(CrvPixels), c_p, c_i32, P(CrvFinderGeom),
                                              P(CrvClusters), P(CrvMembers), c_p, c_p, c_i64, c_p, c_p,
                                              P(CrvLookupChain), P(c_p)]),
    "crv_chain_graph_launch": (c_i32, [c_p, c_p]),
    "crv_chain_graph_set_params": (c_i32, [c_p, P(CrvParams)]),
    "crv_chain_graph_destroy": (None, [c_p]),
}

# symbols declared in include/crvgpu.h (the load test checks every one is exported)
DECLARED = tuple(_SIGS)

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libcrvgpu.so (building it first if needed) and declare the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"CRV engine library missing: {path}")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc, what):
    if rc == CRV_ERR_ARG:
        raise ValueError(f"{what}: invalid arguments")
    if rc == CRV_ERR_TOO_LARGE:
        raise ValueError(f"{what}: the call needs more scratch than the static maximum ({PULSES_STATIC_MAX_BYTES} bytes)")
    if rc != CRV_OK:
        raise RuntimeError(f"{what}: CUDA launch failed (code {rc})")


def ptr(t):
    """Device pointer of a torch tensor (None -> NULL)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def status_string(flags):
    return load().crv_status_string(int(flags)).decode()


class DeviceStatus:
    """A device status block (CrvStatus) held in a torch tensor; read() copies it to the host."""

    def __init__(self, device):
        import torch
        self.t = torch.zeros(ctypes.sizeof(CrvStatus) // 8, dtype=torch.int64, device=device)

    def reset(self):
        self.t.zero_()

    @property
    def ptr(self):
        return ctypes.c_void_p(self.t.data_ptr())

    def read(self):
        a = self.t.cpu().numpy()
        flags = int(np.int64(a[0]) & 0xFFFFFFFF)
        return flags, a[1:17].copy()


def launch_count():
    return int(load().crv_launch_count())


def profile(on):
    load().crv_profile(1 if on else 0)


def profile_read(cap=100000):
    """[(kernel name, ms)] of the launches recorded since profile(True) (synchronises on their events)."""
    L = load()
    names = ctypes.create_string_buffer(64 * cap)
    ms = (ctypes.c_float * cap)()
    n = L.crv_profile_read(cap, names, ms)
    raw = names.raw
    return [(raw[64 * i:64 * i + 64].split(b"\0", 1)[0].decode(), float(ms[i])) for i in range(min(n, cap))]
