"""Physical SiPM presence for the chain's status masking (crv/crvfastsim/readout.py:9-72): a channel 4 * bar + SiPM is
read out iff its bar's sector has SiPMs on side SiPM % 2 (Offline CrvSiPMChargeGenerator's hasCMB), independent of
calibration status.  sensor_mask builds the dense mask from a counters configuration, apply returns conditions that
carry it, effective_status ORs status bit 0 into the absent channels (the chain drops SiPMs with bit 0 or 2).

Host code (NumPy): the mask is prepared once per geometry and enters the device tables as status bits.  Invalid
inputs raise ValueError with the reference's messages, before any work.
"""
from __future__ import annotations

from collections.abc import Mapping
from dataclasses import replace

import numpy as np


def _is_name_list(names):
    if isinstance(names, np.ndarray):
        return names.ndim == 1
    return isinstance(names, (list, tuple))


def _sector_names(geom):
    names = getattr(geom, "sector_names", None)
    if not _is_name_list(names) or len(names) == 0:
        raise ValueError("readout geometry requires nonempty sector_names")
    names = list(names)
    valid = all(isinstance(n, str) and len(n) > 0 for n in names)
    if not valid or len(set(names)) != len(names):
        raise ValueError("readout geometry sector_names must be unique nonempty strings")
    return names


def _bar_sectors(geom, n_sectors):
    sector = np.asarray(getattr(geom, "sector", None))
    if sector.ndim != 1 or sector.dtype.kind not in "iu":
        raise ValueError("readout geometry sector must be a one-dimensional integer array")
    nbars = getattr(geom, "nbars", None)
    is_count = isinstance(nbars, (int, np.integer)) and not isinstance(nbars, (bool, np.bool_))
    if not is_count or nbars < 0 or sector.shape != (nbars,):
        raise ValueError("readout geometry sector size must equal nbars")
    if sector.size and (sector.min() < 0 or sector.max() >= n_sectors):
        raise ValueError("readout geometry contains an unknown sector index")
    return sector


def _side_flags(names, counters_cfg):
    """[sectors, 2] presence of SiPMs on side 0 / 1 from crs.sipmsAtSide<side><sector> (booleans only)."""
    if not isinstance(counters_cfg, Mapping):
        raise ValueError("readout counters_cfg must be a mapping")
    if "crs.sectorNames" in counters_cfg:
        listed = counters_cfg["crs.sectorNames"]
        if not _is_name_list(listed) or list(listed) != names:
            raise ValueError("readout geometry sector_names disagree with crs.sectorNames")
    flags = np.zeros((len(names), 2), bool)
    for s, name in enumerate(names):
        for side in (0, 1):
            key = f"crs.sipmsAtSide{side}{name}"
            if key not in counters_cfg:
                raise ValueError(f"readout counters missing {key}")
            v = counters_cfg[key]
            if not isinstance(v, (bool, np.bool_)):
                raise ValueError(f"readout counters {key} must be boolean, got {v!r}")
            flags[s, side] = bool(v)
    return flags


def sensor_mask(geom, counters_cfg):
    """Dense bool mask over channels 4 * bar + SiPM: present iff the bar's sector has SiPMs on side SiPM % 2."""
    names = _sector_names(geom)
    sector = _bar_sectors(geom, len(names))
    flags = _side_flags(names, counters_cfg)
    side_of_sipm = np.array([0, 1, 0, 1])
    return flags[sector][:, side_of_sipm].reshape(-1)


def effective_status(cond):
    """cond.status with bit 0 set on the channels readout_mask marks absent (cond.status itself without a mask)."""
    mask = getattr(cond, "readout_mask", None)
    if mask is None:
        return cond.status
    status = np.asarray(cond.status)
    if status.ndim != 1 or status.dtype.kind not in "iu":
        raise ValueError("readout status must be a one-dimensional integer array")
    if not isinstance(mask, np.ndarray) or mask.dtype != np.dtype(bool):
        raise ValueError("readout_mask must be a boolean numpy array")
    if mask.shape != status.shape:
        raise ValueError("readout_mask must be one-dimensional with exactly one entry per status channel")
    out = status.copy()
    out[~mask] |= 1
    return out


def apply(cond, geom, counters_cfg):
    """Conditions carrying the physical mask (a new object; cond is not modified).  Channels beyond the geometry's bars
    stay present."""
    mask = sensor_mask(geom, counters_cfg)
    n = len(np.asarray(cond.status))
    if n < mask.size:
        raise ValueError(f"readout: conditions cover {n} channels, the geometry has {mask.size}")
    full = np.ones(n, bool)
    full[:mask.size] = mask
    masked = replace(cond, readout_mask=full)
    effective_status(masked)
    return masked
