"""The step-table interchange format: flat TTrees in the TFileService directory ``dump/`` keyed by (run, subrun,
event) — the reference's core/mu2efastsim/tables.py (KEY, DIR, expand, read, read_many, livetime, primary_muons,
all_primary_muons, write: :12-72) and crv/crvfastsim/tables.py (primary_muon_crossings :13-26, write :29-31).

The reference returns pandas DataFrames read through uproot; uproot is not a dependency here, and pandas is optional:
read returns a DataFrame where pandas is importable (library="pd"), else a `Table` (library="np"): a dict of NumPy
columns with the row count as len() and attribute access to columns (``t.bar``); the ``steps`` tree then comes back as
a StepTable.  The engine's entry points (chain.charges, upload_steps) take either as they are.  Files are
read and written by crvgpu.rootio (TTrees; the reference's writer makes RNTuples unless as_ttree=True, this one makes
TTrees either way).
"""
from __future__ import annotations

import glob

import numpy as np

from . import rootio
from .geometry import StepTable

KEY = ["run", "subrun", "event"]
DIR = "dump"
PRIMARY_MUON_PDG = 13


class Table(dict):
    """Column table: {name: array}, len() = rows, columns also as attributes."""

    def __len__(self):
        for v in self.values():
            return len(v)
        return 0

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError:
            raise AttributeError(k) from None

    def rows(self, sel):
        return type(self)({k: np.asarray(v)[sel] for k, v in self.items()})

    @property
    def columns(self):
        return list(self.keys())


class StepRows(StepTable):
    """The ``steps`` tree: a StepTable (midpoint aliases for the engine) with Table's attribute access."""

    __getattr__ = Table.__getattr__
    rows = Table.rows
    columns = Table.columns


def _table(tree, cols, library="np"):
    if library == "pd":
        import pandas as pd
        return pd.DataFrame(dict(cols))
    return StepRows(cols) if tree == "steps" else Table(cols)


def _library(library):
    """The reference returns pandas DataFrames: library None means "pd" where pandas is importable, else "np"."""
    if library is None:
        try:
            import pandas  # noqa: F401
            return "pd"
        except ImportError:
            return "np"
    if library not in ("np", "pd"):
        raise ValueError(f"library must be 'np' or 'pd', got {library!r}")
    return library


def expand(inputs):
    """Glob patterns -> sorted file lists (a pattern that matches nothing is kept as a path)."""
    out = []
    for p in inputs:
        out += sorted(glob.glob(p)) or [p]
    return out


def read(path, tree, columns=None, library=None):
    """Tree `tree` of directory dump/ in `path` -> a pandas DataFrame, as the reference returns (library "pd", the
    default where pandas is importable), or a Table (StepRows for ``steps``; library "np", the default otherwise)."""
    lib = _library(library)
    with rootio.RootFile(path) as f:
        return _table(tree, f[f"{DIR}/{tree}"].arrays(columns), lib)


def read_many(paths, tree, columns=None, library=None):
    """Rows of `tree` from every file (patterns expanded), concatenated in file order (library as in read)."""
    lib = _library(library)
    parts = [read(p, tree, columns, "np") for p in expand(paths)]
    if not parts:
        return _table(tree, {}, lib)
    return _table(tree, {k: np.concatenate([t[k] for t in parts]) for k in parts[0]}, lib)


def _first_of_groups(cols):
    """Indices of the first row of each distinct key tuple, in row order (drop_duplicates(keep='first'))."""
    n = len(cols[0])
    if n == 0:
        return np.zeros(0, np.int64)
    a = np.stack([np.asarray(c).astype(np.int64) for c in cols], 1)
    _, first = np.unique(a, axis=0, return_index=True)
    return np.sort(first)


def livetime(paths):
    """Total CosmicLivetime [s] over the subruns of the given files (each (run, subrun) counted once)."""
    s = read_many(paths, "subruns", library="np")
    if len(s) == 0:
        return 0.0
    keep = _first_of_groups([s["run"], s["subrun"]])
    return float(np.asarray(s["livetime"], float)[keep].sum())


def primary_muons(gen):
    """The generated primary muon of each event: one row per event (events with no muon are dropped)."""
    m = np.abs(np.asarray(gen["pdg"])) == PRIMARY_MUON_PDG
    mu = Table({k: np.asarray(v)[m] for k, v in gen.items()})
    if len(mu) == 0:
        return mu
    return mu.rows(_first_of_groups([mu[k] for k in KEY]))


def all_primary_muons(gen):
    """Every generated muon ordered by event and gen index, with `mukey` = 1, 2, ... per event (the SimParticle key of
    the event's first, second, ... muon)."""
    m = np.abs(np.asarray(gen["pdg"])) == PRIMARY_MUON_PDG
    mu = Table({k: np.asarray(v)[m] for k, v in gen.items()})
    order_cols = [c for c in KEY + ["idx"] if c in mu]
    if len(mu):
        mu = mu.rows(np.lexsort([np.asarray(mu[c]) for c in reversed(order_cols)]))
    a = np.stack([np.asarray(mu[k]).astype(np.int64) for k in KEY], 1) if len(mu) else np.zeros((0, 3), np.int64)
    new = np.ones(len(mu), bool)
    if len(mu) > 1:
        new[1:] = np.any(a[1:] != a[:-1], axis=1)
    start = np.flatnonzero(new)
    cnt = np.diff(np.r_[start, len(mu)])
    mu["mukey"] = (np.arange(len(mu)) - np.repeat(start, cnt) + 1).astype(np.int64)
    return mu


def primary_muon_crossings(steps, parts, sector_of_bar):
    """The CrvSteps of each event's primary muon summed per bar: one row per (event, bar) crossing, in order of first
    appearance (edep and len summed, earliest t0, nsteps = steps merged), plus the bar's sector.  The primary muon is
    the SimParticle with isprim == 1 and |pdg| == 13 (truth identity, never time or distance)."""
    pm = (np.asarray(parts["isprim"]) == 1) & (np.abs(np.asarray(parts["pdg"])) == PRIMARY_MUON_PDG)
    pk = np.stack([np.asarray(parts[k])[pm].astype(np.int64) for k in KEY] +
                  [np.asarray(parts["key"])[pm].astype(np.int64)], 1)
    sk = np.stack([np.asarray(steps[k]).astype(np.int64) for k in KEY] + [np.asarray(steps["sp"]).astype(np.int64)], 1)
    _, inv = np.unique(np.concatenate([pk, sk]), axis=0, return_inverse=True)
    inv = inv.ravel()
    sel = np.flatnonzero(np.isin(inv[len(pk):], inv[:len(pk)]))
    g = np.stack([np.asarray(steps[k])[sel].astype(np.int64) for k in KEY] +
                 [np.asarray(steps["bar"])[sel].astype(np.int64)], 1)
    out = Table()
    if len(sel) == 0:
        for k in KEY + ["bar", "edep", "len", "t0", "nsteps", "sector"]:
            out[k] = np.zeros(0)
        return out
    _, first, gid = np.unique(g, axis=0, return_index=True, return_inverse=True)
    gid = gid.ravel()
    rank = np.empty(len(first), np.int64)
    rank[np.argsort(first, kind="stable")] = np.arange(len(first))
    gid = rank[gid]
    first = np.sort(first)
    G = len(first)
    for k in KEY + ["bar"]:
        out[k] = np.asarray(steps[k])[sel][first]
    for k in ("edep", "len"):
        v = np.asarray(steps[k])[sel]
        out[k] = np.bincount(gid, weights=v.astype(float), minlength=G).astype(v.dtype)
    t0 = np.asarray(steps["t0"])[sel]
    tmin = np.full(G, np.inf)
    np.minimum.at(tmin, gid, t0.astype(float))
    out["t0"] = tmin.astype(t0.dtype)
    out["nsteps"] = np.bincount(gid, minlength=G).astype(np.int64)
    out["sector"] = np.asarray(sector_of_bar)[np.asarray(out["bar"], np.int64)]
    return out


def write(path, trees, particles=None, gen=None, subruns=None, as_ttree=False):
    """Write tables into directory dump/ of a new ROOT file, zlib level 1 (ROOT's default setting); empty or None
    tables are skipped.  Either form of the reference's write: write(path, {tree name: table}, as_ttree=...)
    (core/mu2efastsim/tables.py:52) or write(path, steps, particles, gen=None, subruns=None, as_ttree=...), the
    CrvStepTableDumper layout (crv/crvfastsim/tables.py:29-31)."""
    if not (isinstance(trees, dict) and trees and all(v is None or hasattr(v, "keys") for v in trees.values())):
        trees = {"steps": trees, "particles": particles, "gen": gen, "subruns": subruns}
    rootio.write(path, {f"{DIR}/{k}": (None if v is None else {c: np.asarray(v[c]) for c in v.keys()})
                        for k, v in trees.items()})
    print(f"wrote {path}")
