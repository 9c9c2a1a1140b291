"""Reader of the CRV photon lookup tables (format version 6, Offline CRVResponse MakeCrvPhotons) into the reference's
LookupTable fields (crv/crvfastsim/response/lookup.py:70-98), so a table read here drives LookupModel directly.

The parse is native (crv_lookup_file_info / crv_lookup_file_read in libcrvgpu.so, host memory): one linear pass
validates the image and sizes the arrays, a second fills them; delay and emission weights are kept as the reference
keeps them (uint8, zero-padded to the longest vector of each table, at least one column, with int32 per-bin sums).
load(name, directory) mirrors the reference's load (crv/crvfastsim/response/lookup.py:149-179): the same file names,
lookup directory (CRVFS_LOOKUP_DIR) and ValueError messages; its pinning and provenance records (the reference's
library bookkeeping) are not part of this engine.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import _capi

DEFAULT_DIR = "/cvmfs/mu2e.opensciencegrid.org/DataFiles/CRVConditions/v6_0"   # the reference's default
EDGES = ("x", "y", "z", "beta", "theta", "phi", "r")
TABLES = ("scint", "ckscint", "ckfiber")
CONSTANTS = ("half_thickness", "half_width", "half_length", "fiber_separation", "hole_radius_x", "hole_radius_y",
             "fiber_radius", "corner_radius", "birks", "fiber_decay_time")


def lookup_dir():
    return os.environ.get("CRVFS_LOOKUP_DIR", DEFAULT_DIR)


@dataclass
class Table:
    """One of a file's three tables, one row per table bin (field names as the reference's decoded table)."""
    prob: np.ndarray        # float32 per bin: chance that a photon made in the bin reaches the first SiPM
    delays: np.ndarray      # uint8, bins x longest delay vector: arrival-delay histogram (1 ns bins), zero padded
    delay_sum: np.ndarray   # int32 per bin: total of the bin's delay weights
    emis: np.ndarray        # uint8, bins x longest emission vector: fibre re-emission count histogram, zero padded
    emis_sum: np.ndarray    # int32 per bin: total of the bin's emission weights


@dataclass
class LookupTable:
    """A decoded version-6 table file: the counter and fibre geometry, the Cherenkov yield curves, the bin edges of
    every table axis and the three tables (field names as the reference's decoded object)."""
    name: str
    version: tuple
    reflector: int
    half_thickness: float
    half_width: float
    half_length: float
    fiber_separation: float
    hole_radius_x: float
    hole_radius_y: float
    fiber_radius: float
    corner_radius: float
    birks: float
    fiber_decay_time: float
    ck_scint: np.ndarray    # Cherenkov yield in the scintillator: rows of (beta, photons per mm)
    ck_fiber: np.ndarray    # the same in the fibre
    edges: dict             # axis name (x, y, z, beta, theta, phi, r) -> float64 bin edges
    tables: dict            # table name (scint, ckscint, ckfiber) -> Table


def _error(info, where):
    e, a, b = info.error, info.error_a, info.error_b
    if e == _capi.LUTF_VERSION:
        return ValueError(f"{where}: lookup table version {a}.{b}, expected 6.x")
    if e == _capi.LUTF_BIN_NUMBER:
        return ValueError(f"corrupt lookup table: bin {a} at position {b}")
    if e == _capi.LUTF_TRAILING:
        return ValueError(f"{where}: {a} trailing bytes")
    if e == _capi.LUTF_TRUNCATED:
        return ValueError(f"{where}: lookup table truncated inside the record at byte {a}")
    if e == _capi.LUTF_SIZE:
        return ValueError(f"{where}: empty bin-edge vector {EDGES[a]!r}" if a >= 0 else
                          f"{where}: table sizes beyond the file")
    return ValueError(f"{where}: malformed lookup table")


def parse(image, name="", where=None):
    """A LookupTable from the bytes of a version-6 table file."""
    L = _capi.load()
    buf = np.frombuffer(memoryview(image), np.uint8) if len(image) else np.zeros(0, np.uint8)
    where = where or name or "lookup table"
    info = _capi.CrvLookupFileInfo()
    ptr = ctypes.c_void_p(buf.ctypes.data) if len(buf) else None
    if L.crv_lookup_file_info(ptr, len(buf), ctypes.byref(info)) != _capi.CRV_OK:
        raise _error(info, where)
    ck = [np.empty((info.n_ck[m], 2), np.float64) for m in range(2)]
    edges = [np.empty(info.n_edges[e], np.float64) for e in range(7)]
    tabs = []
    for t in range(3):
        n, dw, ew = info.n_bins[t], info.delay_width[t], info.emis_width[t]
        tabs.append(Table(np.empty(n, np.float32), np.empty((n, dw), np.uint8), np.empty(n, np.int32),
                          np.empty((n, ew), np.uint8), np.empty(n, np.int32)))
    out = _capi.CrvLookupFileOut()
    p = lambda a: a.ctypes.data if a.size else None                                    # noqa: E731
    for m in range(2):
        out.ck[m] = p(ck[m])
    for e in range(7):
        out.edges[e] = p(edges[e])
    for t, T in enumerate(tabs):
        out.tables[t] = _capi.CrvLookupFileTable(p(T.prob), p(T.delays), p(T.delay_sum), p(T.emis), p(T.emis_sum))
    if L.crv_lookup_file_read(ptr, len(buf), ctypes.byref(info), ctypes.byref(out)) != _capi.CRV_OK:
        raise ValueError(f"{where}: lookup table changed between the size and the read pass")
    return LookupTable(name, (int(info.version_major), int(info.version_minor)), int(info.reflector),
                       *(float(info.constants[i]) for i in range(10)), ck[0], ck[1], dict(zip(EDGES, edges)),
                       dict(zip(TABLES, tabs)))


def load(name, directory=None):
    """Read LookupTable_<name> (e.g. '6000_0') from the lookup directory (crv/crvfastsim/response/lookup.py:149-179)."""
    path = os.path.join(directory or lookup_dir(), f"LookupTable_{name}" if not name.startswith("LookupTable") else name)
    with open(path, "rb") as fh:
        image = fh.read()
    return parse(image, os.path.basename(path), path)


def arrays(L):
    """The decoded content of a table as named arrays (the reference's lookup.arrays naming, lookup.py:182-192)."""
    out = {"version": np.array(L.version, np.int64), "reflector": np.int64(L.reflector),
           "constants": np.array([getattr(L, k) for k in CONSTANTS]), "ck_scint": L.ck_scint, "ck_fiber": L.ck_fiber}
    out.update({f"edges_{k}": v for k, v in L.edges.items()})
    for t, T in L.tables.items():
        out.update({f"{t}_prob": T.prob, f"{t}_delays": T.delays, f"{t}_delay_sum": T.delay_sum,
                    f"{t}_emis": T.emis, f"{t}_emis_sum": T.emis_sum})
    return out
