"""CRV geometry, conditions and synthetic CrvSteps for the engine.

CRVGeometry keeps the reference's bar-geometry fields (crv/crvfastsim/geometry.py:104-119); SectorGeom the
coincidence finder's per-bar lookups (crv/crvfastsim/reco/coinc.py:64-109).  The Offline counters file the reference
builds them from is not available here, so the workload's geometries are built directly:

  * one module of 4 layers x 16 counters, counters 5.0 x 1.98 x 450 cm (lengths along z, widths along x,
    thickness along y), sector "EX";
  * the full-scale layout: 86 modules of 4 x 16 side by side, bar lengths from {230, 300, 450, 560, 660} cm; one
    sector (and sector type) per length class.

Synthetic steps follow the workload: Poisson(mean) steps per event, counter uniform, position uniform in the bar,
step length U(0.5, 2.5) cm, edep Moyal(3.6 MeV, 0.3 MeV) x length / 1.98 cm (Moyal sampled as loc - scale ln z^2,
z ~ N(0, 1)), time U(0, 1700) ns; optional uniform-time noise steps per counter per event.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .config import CHAN_MULT, Conditions, SectorGeom

WIDTH = 50.0            # mm
THICK = 19.8            # mm
PITCH = 51.3            # mm between counter centres in a layer
LAYER_PITCH = 21.1      # mm between layers
STAGGER = 12.8          # mm offset of odd layers
MODULE_GAP = 20.0       # mm between modules
LENGTHS = (2300.0, 3000.0, 4500.0, 5600.0, 6600.0)
CALIB_HEIGHT = 0.0055 * 2300.0          # ADC per PE at the single-PE peak
CALIB_AREA = np.e * CALIB_HEIGHT * 10.0  # ADC ns per PE of a Gumbel pulse of beta 10 ns


@dataclass
class CRVGeometry:
    sector_names: list
    sector: np.ndarray
    module: np.ndarray
    layer: np.ndarray
    counter: np.ndarray
    center: np.ndarray
    halflen: np.ndarray
    local_to_world: np.ndarray

    @property
    def nbars(self) -> int:
        return len(self.sector)


def module_geometry(n_modules=1, lengths=None, seed=0, n_layers=4, n_counters=16):
    """Modules of n_layers x n_counters side by side along x.  lengths: per-module bar length (mm); default 4500 for one
    module, else uniform over LENGTHS (seeded).  Modules of one length share a sector named L<length in cm>."""
    if lengths is None:
        lengths = ([4500.0] if n_modules == 1 else
                   list(np.random.default_rng(seed).choice(LENGTHS, n_modules)))
    lengths = [float(v) for v in lengths]
    names = ["EX"] if n_modules == 1 else [f"L{int(round(v / 10))}" for v in sorted(set(lengths))]
    sec_of = {v: (0 if n_modules == 1 else sorted(set(lengths)).index(v)) for v in lengths}
    rows = {k: [] for k in ("sector", "module", "layer", "counter", "center", "halflen")}
    mod_in_sec = {}
    width_mod = n_counters * PITCH + MODULE_GAP
    for m, L in enumerate(lengths):
        s = sec_of[L]
        mi = mod_in_sec.get(s, 0)
        mod_in_sec[s] = mi + 1
        for layer in range(n_layers):
            for c in range(n_counters):
                x = m * width_mod + (c - (n_counters - 1) / 2) * PITCH + STAGGER * (layer % 2)
                y = (layer - (n_layers - 1) / 2) * LAYER_PITCH
                rows["sector"].append(s); rows["module"].append(mi); rows["layer"].append(layer)
                rows["counter"].append(c); rows["center"].append((x, y, 0.0))
                rows["halflen"].append((WIDTH / 2, THICK / 2, L / 2))
    nb = len(rows["sector"])
    return CRVGeometry(sector_names=names, sector=np.array(rows["sector"]), module=np.array(rows["module"]),
                       layer=np.array(rows["layer"]), counter=np.array(rows["counter"]),
                       center=np.array(rows["center"], float), halflen=np.array(rows["halflen"], float),
                       local_to_world=np.tile([1, 0, 2], (nb, 1)))


def sector_geom(geom, n_counters=16):
    """SectorGeom of a module geometry: one sector type per sector, both readout ends instrumented."""
    ns = len(geom.sector_names)
    nmod = np.zeros(ns, np.int64)
    np.maximum.at(nmod, geom.sector, geom.module + 1)
    preceding = np.r_[0, np.cumsum(nmod * n_counters)[:-1]]
    cit = preceding[geom.sector] + n_counters * geom.module + geom.counter
    dt, dw, dl = geom.local_to_world[:, 0], geom.local_to_world[:, 1], geom.local_to_world[:, 2]
    b = np.arange(geom.nbars)
    first = np.array([np.flatnonzero(geom.sector == s)[0] for s in range(ns)])
    length_dir = dl[first]
    half = geom.halflen[first, length_dir]
    centre_l = geom.center[first, length_dir]
    return SectorGeom(sector=geom.sector, layer=geom.layer, counter_in_type=cit, x=geom.center[b, dw],
                      y=geom.center[b, dt], pos=geom.center, length_dir=length_dir,
                      sector_type=np.arange(1, ns + 1), sector_names=list(geom.sector_names),
                      pos_side0=centre_l - half, pos_side1=centre_l + half, sipms_side0=np.ones(ns, bool),
                      sipms_side1=np.ones(ns, bool))


def default_conditions(geom, pedestal=100.0):
    """Uniform calibration: pedestal, pulse area/height of the Gumbel single-PE shape, no time offsets, all channels
    good; FEB = 64 consecutive channels, ROC = 24 FEBs."""
    n = 4 * geom.nbars
    ch = np.arange(n)
    z = np.zeros(n)
    return Conditions(pedestal=z + pedestal, pulsearea=z + CALIB_AREA, pulseheight=z + CALIB_HEIGHT, timeoffset=z.copy(),
                      status=np.zeros(n, np.int64), roc=(ch // (64 * 24)).astype(np.int64),
                      feb=((ch // 64) % 24).astype(np.int64), deviation=z.copy())


class StepTable(dict):
    """Column table of CrvSteps (dict of equal-length arrays).  Columns: run, subrun, event, bar, x, y, z, t, edep,
    len; the reference's start/end columns (x0, x1, ..., t0, t1) map to the midpoints."""

    ALIASES = {"x0": "x", "x1": "x", "y0": "y", "y1": "y", "z0": "z", "z1": "z", "t0": "t", "t1": "t"}

    def __getitem__(self, k):
        if not dict.__contains__(self, k) and k in self.ALIASES:
            k = self.ALIASES[k]
        return dict.__getitem__(self, k)

    def __contains__(self, k):
        return dict.__contains__(self, k) or (k in self.ALIASES and dict.__contains__(self, self.ALIASES[k]))

    def __len__(self):
        return len(dict.__getitem__(self, "bar"))

    def rows(self, sel):
        return StepTable({k: v[sel] for k, v in self.items()})


def synthetic_steps(n_events, geom, seed=0, mean_steps=40.0, noise_per_counter=0.0, t_max=1700.0, run=1, subrun=1,
                    first_event=0, dtype=np.float32):
    """Synthetic CrvSteps of the workload, grouped by event in increasing event number (see module docstring)."""
    rng = np.random.default_rng([seed, first_event])
    nb = geom.nbars
    n_sig = rng.poisson(mean_steps, n_events)
    n_noise = rng.poisson(noise_per_counter * nb, n_events) if noise_per_counter > 0 else np.zeros(n_events, np.int64)
    per = n_sig + n_noise
    N = int(per.sum())
    ev = np.repeat(np.arange(first_event, first_event + n_events, dtype=np.int64), per)
    bar = rng.integers(0, nb, N)
    ax = geom.local_to_world[bar]
    half = geom.halflen[bar]
    c = geom.center[bar]
    loc = rng.uniform(-1.0, 1.0, (N, 3))
    pos = c.copy()
    r = np.arange(N)
    for k in range(3):
        pos[r, ax[:, k]] += loc[:, k] * half[r, ax[:, k]]
    ln = rng.uniform(5.0, 25.0, N)                                   # mm
    zz = rng.standard_normal(N)
    edep = (3.6 - 0.3 * np.log(zz * zz)) * ln / 19.8
    t = rng.uniform(0.0, t_max, N)
    return StepTable(run=np.full(N, run, np.int64), subrun=np.full(N, subrun, np.int64), event=ev,
                     bar=bar.astype(np.int32), x=pos[:, 0].astype(dtype), y=pos[:, 1].astype(dtype),
                     z=pos[:, 2].astype(dtype), t=t.astype(dtype), edep=edep.astype(dtype), len=ln.astype(dtype))


def event_key(steps):
    return (np.asarray(steps["subrun"], np.int64) << 20) | np.asarray(steps["event"], np.int64)


def label_of(evkey, chan):
    return np.asarray(evkey, np.int64) * CHAN_MULT + np.asarray(chan, np.int64)
