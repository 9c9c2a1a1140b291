"""Lookup-table photon model on the device: the substep kernel of crvfastsim.response.photons._substep_photons
(crv/crvfastsim/response/photons.py:163-224) behind crv_substep_photons.

DeviceLookup uploads a lookup table with the reference's fields (crv/crvfastsim/response/lookup.py:70-98: geometry,
bin edges, and the scint / ckscint / ckfiber tables of arrival probabilities, delay and emission weights) once;
substep_photons(L, rows, seed) takes the reference's per-(step, SiPM) rows and returns the photons (step index,
channel, arrival time).  The reference draws from a sequential generator (rng); here every draw is keyed by (seed,
step, channel, substep, table, arrival), so rows give the same photons alone and in any batch.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from .response import _stream, _torch, raise_status

EDGES = ("x", "y", "z", "beta", "theta", "phi", "r")
TABLES = ("scint", "ckscint", "ckfiber")
GEOMETRY = ("half_thickness", "half_width", "half_length", "fiber_separation", "hole_radius_x", "hole_radius_y",
            "fiber_radius", "corner_radius", "fiber_decay_time")
ROW_REAL = ("t0", "t1", "beta", "dev")
ROW_INT = ("nsub", "step", "chan", "n_scint", "n_ck_s", "n_ck_f")


def _precision_code(precision):
    if precision not in ("fp64", "fp32"):
        raise ValueError(f"precision must be 'fp64' or 'fp32', got {precision!r}")
    return 0 if precision == "fp64" else 1


class DeviceLookup:
    """A lookup table on the device (CrvLookup)."""

    def __init__(self, L, device="cuda"):
        torch = _torch()
        self.device = device
        self.name = getattr(L, "name", "lookup")
        self.geometry = {k: float(getattr(L, k)) for k in GEOMETRY}
        f64 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(device)  # noqa: E731
        self.edges = []
        for k in EDGES:
            e = np.asarray(L.edges[k], np.float64)
            if e.ndim != 1 or len(e) < 2 or np.any(np.diff(e) < 0):
                raise ValueError(f"lookup edges {k}: at least two ascending values required")
            self.edges.append(f64(e))
        phi = np.asarray(L.edges["phi"], np.float64)
        if phi[0] < 0 or phi[-1] > np.pi:
            raise ValueError("lookup phi edges must lie in [0, pi] (phi bins are found on cos phi)")
        self.cos_phi = f64(np.cos(phi))
        theta = np.asarray(L.edges["theta"], np.float64)
        self.cos_theta = f64(np.cos(theta)) if theta[0] >= 0 and theta[-1] <= np.pi else None
        self.half_length = float(L.half_length)
        self.reflector = int(getattr(L, "reflector", 0))
        self.ck_scint = np.asarray(getattr(L, "ck_scint", np.zeros((0, 2))), np.float64).reshape(-1, 2)
        self.ck_fiber = np.asarray(getattr(L, "ck_fiber", np.zeros((0, 2))), np.float64).reshape(-1, 2)
        nb = {k: len(L.edges[k]) - 1 for k in EDGES}
        need = {"scint": nb["x"] * nb["y"] * nb["z"], "ckscint": nb["x"] * nb["y"] * nb["z"] * nb["beta"],
                "ckfiber": nb["beta"] * nb["theta"] * nb["phi"] * nb["r"] * nb["z"]}
        self.tables = []
        for k in TABLES:
            T = L.tables[k]
            d, e = np.asarray(T.delays, np.uint8), np.asarray(T.emis, np.uint8)
            prob = np.asarray(T.prob, np.float32)
            if len(prob) < need[k] or d.shape[0] != len(prob) or e.shape[0] != len(prob):
                raise ValueError(f"lookup table {k}: {len(prob)} bins, the edges need {need[k]}")
            t = dict(prob=torch.from_numpy(np.ascontiguousarray(prob)).to(device),
                     delays=torch.from_numpy(np.ascontiguousarray(d)).to(device),
                     delay_sum=torch.from_numpy(np.ascontiguousarray(T.delay_sum, np.int32)).to(device),
                     emis=torch.from_numpy(np.ascontiguousarray(e)).to(device),
                     emis_sum=torch.from_numpy(np.ascontiguousarray(T.emis_sum, np.int32)).to(device),
                     shape=(len(prob), d.shape[1], e.shape[1]))
            self.tables.append(t)
        self.nbytes = sum(int(v.numel() * v.element_size()) for t in self.tables for k, v in t.items() if k != "shape")

    def c(self, precision="fp64"):
        S = _capi.CrvLookup(*[self.geometry[k] for k in GEOMETRY])
        S.precision = _precision_code(precision)
        for i, e in enumerate(self.edges):
            S.edges[i] = e.data_ptr()
            S.nedges[i] = int(e.numel())
        S.cos_phi_edges = self.cos_phi.data_ptr()
        S.cos_theta_edges = self.cos_theta.data_ptr() if self.cos_theta is not None else None
        for i, t in enumerate(self.tables):
            n, nd, ne = t["shape"]
            S.table[i] = _capi.CrvLookupTable(t["prob"].data_ptr(), t["delays"].data_ptr(), t["delay_sum"].data_ptr(),
                                              t["emis"].data_ptr(), t["emis_sum"].data_ptr(), n, nd, ne, 0)
        return S


class DeviceRows:
    """(step, SiPM) substep rows on the device (CrvSubstepRows): from the reference's host row dict (theta), or from
    device columns built by crv_lookup_rows (cos theta)."""

    def __init__(self, rows=None, device="cuda"):
        if rows is None:
            return
        torch = _torch()
        n = len(rows["nsub"])
        f64 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(device)  # noqa: E731
        i64 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.int64)).to(device)    # noqa: E731
        chan = np.asarray(rows["chan"], np.int64)
        if n and (chan.min() < 0 or chan.max() >= 32768):
            raise ValueError("substep rows: channels must lie in [0, 32768)")
        self.n = n
        self.s, self.d = f64(np.reshape(rows["s"], (n, 3))), f64(np.reshape(rows["d"], (n, 3)))
        self.real = {k: f64(rows[k]) for k in ROW_REAL}
        self.theta = f64(rows["theta"]) if "theta" in rows else None
        self.cos_theta = f64(rows["cos_theta"]) if self.theta is None else None
        mu = rows.get("mu")
        self.mu = f64(mu) if mu is not None else None
        self.ints = {k: i64(rows[k]) for k in ROW_INT}

    @classmethod
    def from_columns(cls, cols, n):
        """Rows [0, n) of device columns (LOOKUP_ROW_COLS of crv_lookup_rows)."""
        R = cls()
        R.n = int(n)
        R.s, R.d = cols["s"][:n], cols["d"][:n]
        R.real = {k: cols[k][:n] for k in ROW_REAL}
        R.theta, R.cos_theta = None, cols["cos_theta"][:n]
        R.mu = cols["mu"][:n]
        R.ints = {k: cols[k][:n] for k in ROW_INT}
        return R

    def c(self):
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        r = self.real
        return _capi.CrvSubstepRows(p(self.s), p(self.d), p(r["t0"]), p(r["t1"]), p(r["beta"]), p(self.theta),
                                    p(r["dev"]), p(self.mu), *[p(self.ints[k]) for k in ROW_INT], p(self.cos_theta))


class SubstepEngine:
    """Workspace and launcher of crv_substep_photons (output capacity grows on demand)."""

    def __init__(self, device="cuda"):
        self.device = device
        self.ws = None
        self.per_row = 64.0
        self.status = _capi.DeviceStatus(device)

    def run(self, DL: DeviceLookup, R: DeviceRows, seed, max_tries=3, precision="fp64"):
        """precision "fp64": bit-exact with the oracle; "fp32": FP32-mixed (same statistics, absolute times FP64)."""
        torch = _torch()
        L = _capi.load()
        dev = self.device
        wsb = L.crv_substeps_workspace(R.n)
        if self.ws is None or self.ws.numel() < wsb:
            self.ws = torch.empty(int(wsb) + 1024, dtype=torch.uint8, device=dev)
        S, C = DL.c(precision), R.c()
        for _ in range(max_tries):
            cap = int(max(1024, self.per_row * R.n))
            o_step = torch.empty(cap, dtype=torch.int64, device=dev)
            o_chan = torch.empty(cap, dtype=torch.int64, device=dev)
            o_time = torch.empty(cap, dtype=torch.float64, device=dev)
            n_out = torch.zeros(1, dtype=torch.int64, device=dev)
            self.status.reset()
            _capi.check(L.crv_substep_photons(ctypes.byref(S), ctypes.c_uint32(int(seed) & 0xFFFFFFFF),
                                              ctypes.byref(C), R.n, _capi.ptr(o_step), _capi.ptr(o_chan),
                                              _capi.ptr(o_time), cap, _capi.ptr(n_out), _capi.ptr(self.ws),
                                              self.ws.numel(), _stream(), self.status.ptr), "crv_substep_photons")
            flags, need = self.status.read()
            npo = need[_capi.NEED["PHOTONS_OUT"]]
            if flags == _capi.ST_CAPACITY and npo:
                self.per_row = 1.2 * npo / max(R.n, 1)
                continue
            raise_status(flags, need, "crv_substep_photons")
            m = int(n_out.item())
            return o_step[:m], o_chan[:m], o_time[:m]
        raise RuntimeError("crv_substep_photons: capacities did not converge")


_ENGINE = {}


def substep_photons(L, rows, seed, device="cuda", precision="fp64"):
    """photons._substep_photons(L, rows, rng) with keyed draws: (step index, channel, arrival time) host arrays in
    (row, substep, table, arrival) order.  L: a lookup table object (or a DeviceLookup); rows: the reference's row
    dict (s, d, t0, t1, nsub, beta, theta, dev, optional mu, step, chan, n_scint, n_ck_s, n_ck_f)."""
    DL = L if isinstance(L, DeviceLookup) else DeviceLookup(L, device)
    if device not in _ENGINE:
        _ENGINE[device] = SubstepEngine(device)
    st, ch, tm = _ENGINE[device].run(DL, DeviceRows(rows, device), seed, precision=precision)
    return st.cpu().numpy(), ch.cpu().numpy(), tm.cpu().numpy()


# ---- row preparation and make_photons ------------------------------------------------------------------------------

PRECISION_MM = 0.1
# particle code -> (mass [MeV], charge [e]) of the stock generator's particles (PDG values); ions 100ZZZAAAI are
# decoded on the device (mass A x 931.49410242 MeV, charge Z), unknown codes are neutral and massless
PARTICLES = {11: (0.51099895, -1), -11: (0.51099895, 1), 13: (105.6583755, -1), -13: (105.6583755, 1), 22: (0.0, 0),
             211: (139.57039, 1), -211: (139.57039, -1), 111: (134.9768, 0), 321: (493.677, 1),
             -321: (493.677, -1), 130: (497.611, 0), 310: (497.611, 0), 2212: (938.272088, 1),
             -2212: (938.272088, -1), 2112: (939.565420, 0), -2112: (939.565420, 0), 12: (0.0, 0), -12: (0.0, 0),
             14: (0.0, 0), -14: (0.0, 0), 3122: (1115.683, 0), 3222: (1189.37, 1), 3112: (1197.449, -1)}
_PROPAGATION = {}


def table_propagation(L):
    """(inverse signal speed [ns/mm], attenuation length [mm]) of a lookup table, as the reference derives them
    (photons.table_propagation, crv/crvfastsim/response/photons.py:230-254, after MakeCrvPhotons): the slope of the 10 %
    quantile of the probability-weighted scintillation delays against the distance d to the SiPM end, and -1 / the
    slope of log(summed arrival probability) against d over 0.2 < d / half length < 1.8."""
    key = (getattr(L, "name", id(L)), float(L.half_length))
    if key in _PROPAGATION:
        return _PROPAGATION[key]
    E, T = L.edges, L.tables["scint"]
    nx, ny, nz = len(E["x"]) - 1, len(E["y"]) - 1, len(E["z"]) - 1
    p = np.asarray(T.prob, np.float64)[:nx * ny * nz].reshape(nx, ny, nz)
    ds = np.asarray(T.delay_sum, np.float64)[:nx * ny * nz].reshape(nx, ny, nz)
    w = np.where(ds > 0, p / np.where(ds > 0, ds, 1.0), 0.0)
    hist = np.einsum("xyz,xyzj->zj", w, np.asarray(T.delays, np.float64)[:nx * ny * nz].reshape(nx, ny, nz, -1))
    d = 0.5 * (np.asarray(E["z"])[1:] + np.asarray(E["z"])[:-1]) + float(L.half_length)
    tot = hist.sum(1)
    ok = tot > 0
    q10 = np.argmax(np.cumsum(hist, 1) >= 0.1 * tot[:, None], axis=1)
    inv_v = np.polyfit(d[ok], q10[ok].astype(float), 1)[0]
    P = p.sum((0, 1))
    a = (P > 0) & (d > 0.2 * float(L.half_length)) & (d < 1.8 * float(L.half_length))
    slope = np.polyfit(d[a], np.log(P[a]), 1)[0]
    if not slope < 0:
        raise ValueError(f"cannot determine the attenuation length of lookup table {key[0]}")
    _PROPAGATION[key] = (float(inv_v), float(-1.0 / slope))
    return _PROPAGATION[key]


def bar_keys(geom):
    """Per bar: (sector key, module key), the module key being the sector name + module index when the sector has
    several modules (photons.bar_keys, photons.py:257-264)."""
    names = np.array(geom.sector_names, dtype=object)
    sector, module = np.asarray(geom.sector), np.asarray(geom.module)
    nmod = np.zeros(len(names), np.int64)
    np.maximum.at(nmod, sector, module + 1)
    sk = names[sector]
    return sk, np.where(nmod[sector] > 1, sk + module.astype(str).astype(object), sk)


def bar_ratios(values, geom):
    """Per-bar propagation ratios from {key: ratio} (photons.bar_ratios, photons.py:267-289): key = sector name, "TAG"
    (every sector whose name starts with M) or sector name + module index for sectors with several modules; a module
    key wins over its sector, a sector over TAG; unlisted bars 1."""
    out = np.ones(geom.nbars)
    if not values:
        return out
    sk, mk = bar_keys(geom)
    sset, mset = set(sk), set(mk)
    bad = sorted(set(values) - sset - mset - {"TAG"})
    if bad:
        raise KeyError(f"unknown propagation keys {bad}; known: {sorted(sset | mset | {'TAG'})}")
    tag = np.array([str(n).startswith("M") for n in sk])
    if "TAG" in values:
        out[tag] = values["TAG"]
    for k, v in values.items():
        if k != "TAG" and k in sset:
            out[sk == k] = v
    for k, v in values.items():
        if k in mset and k not in sset:
            out[mk == k] = v
    if not np.all(out > 0):
        raise ValueError("propagation ratios must be positive")
    return out


class LookupModel:
    """The lookup-table photon model of a geometry and response configuration (the reference's ResponseConfig fields:
    sectors {name: (table, reflector, yield_per_mev)}, photon_yield_scale, photon_yield_variation_scale, speed_ratio,
    atten_ratio) with its tables on the device: one (table, reflector) group per combination the sectors use, as
    photons.iter_rows iterates them (table names sorted, reflectors sorted)."""

    def __init__(self, geom, cfg, tables, deviation, device="cuda", precision="fp64"):
        torch = _torch()
        self.device = device
        _precision_code(precision)
        self.precision = precision
        names = list(geom.sector_names)
        sec = np.asarray(geom.sector)
        nb = int(geom.nbars)
        l2w = np.asarray(geom.local_to_world, np.int8).reshape(nb, 3)
        if not np.all(np.sort(l2w, axis=1) == np.arange(3)):
            raise ValueError("geometry local_to_world: every bar needs a permutation of the axes 0, 1, 2")
        center = np.asarray(geom.center, np.float64).reshape(nb, 3)
        r_speed, r_atten = bar_ratios(getattr(cfg, "speed_ratio", {}), geom), bar_ratios(getattr(cfg, "atten_ratio", {}),
                                                                                           geom)
        dev = (np.asarray(deviation, np.float64) * cfg.photon_yield_variation_scale + 1.0) * cfg.photon_yield_scale
        if len(dev) < 4 * nb:
            raise ValueError(f"photon-yield deviations cover {len(dev)} channels, the geometry has {4 * nb}")
        f64 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(device)  # noqa: E731
        codes = np.array(sorted(PARTICLES), np.int64)
        self.pdg_code = torch.from_numpy(codes).to(device)
        self.pdg_mass = f64([PARTICLES[c][0] for c in codes])
        self.pdg_charge = f64([PARTICLES[c][1] for c in codes])
        self.center, self.l2w = f64(center), torch.from_numpy(np.ascontiguousarray(l2w)).to(device)
        self.dev = f64(dev)
        self.tables, self.groups = {}, []
        yields = np.array([float(cfg.sectors[n].yield_per_mev) for n in names])
        for tname in sorted({cfg.sectors[n].table for n in names}):
            L = tables[tname]
            inv_v, att = table_propagation(L)
            for refl in sorted({int(cfg.sectors[n].reflector) for n in names if cfg.sectors[n].table == tname}):
                sids = [i for i, n in enumerate(names) if cfg.sectors[n].table == tname
                        and int(cfg.sectors[n].reflector) == refl]
                if abs(refl) != int(getattr(L, "reflector", 0)):
                    raise ValueError(f"reflector {refl} does not match lookup table {tname} ({L.reflector})")
                if tname not in self.tables:
                    self.tables[tname] = DeviceLookup(L, device)
                DL = self.tables[tname]
                if DL.cos_theta is None:
                    raise ValueError(f"lookup table {tname}: theta edges outside [0, pi]")
                in_g = np.isin(sec, sids)
                g = dict(table=tname, reflector=refl, DL=DL,
                         in_group=torch.from_numpy(in_g.astype(np.int32)).to(device),
                         yield_=f64(yields[sec]), speed_k=f64(inv_v * (1.0 / r_speed - 1.0)),
                         mu=f64((1.0 / r_atten - 1.0) / att), ck_scint=f64(DL.ck_scint), ck_fiber=f64(DL.ck_fiber),
                         nck=(len(DL.ck_scint), len(DL.ck_fiber)))
                self.groups.append(g)
        self.nbars = nb
        self.ws = None
        self.status = _capi.DeviceStatus(device)
        self.substeps = SubstepEngine(device)

    def _group_c(self, g):
        return _capi.CrvLookupGroup(self.center.data_ptr(), self.l2w.data_ptr(), g["in_group"].data_ptr(),
                                    g["yield_"].data_ptr(), g["speed_k"].data_ptr(), g["mu"].data_ptr(),
                                    self.dev.data_ptr(), g["ck_scint"].data_ptr(), g["ck_fiber"].data_ptr(),
                                    self.pdg_code.data_ptr(), self.pdg_mass.data_ptr(), self.pdg_charge.data_ptr(),
                                    g["DL"].half_length, g["reflector"], self.nbars, g["nck"][0], g["nck"][1],
                                    int(self.pdg_code.numel()), 0)

    def upload_steps(self, steps, pdg):
        """Device step columns (float64; bar int32; pdg int64) of a step table with the reference's column names."""
        torch = _torch()
        col = lambda k: np.asarray(steps[k].to_numpy() if hasattr(steps[k], "to_numpy") else steps[k])  # noqa: E731
        cols = {k: torch.from_numpy(np.ascontiguousarray(col(k), np.float64)).to(self.device)
                for k in _capi.LOOKUP_STEP_COLS}
        bar = col("bar").astype(np.int64)
        if len(bar) and (bar.min() < 0 or bar.max() >= self.nbars):
            raise ValueError(f"CRV steps: bar index outside [0, {self.nbars})")
        cols["bar"] = torch.from_numpy(bar.astype(np.int32)).to(self.device)
        cols["pdg"] = torch.from_numpy(np.ascontiguousarray(pdg, np.int64)).to(self.device)
        return cols

    def rows(self, g, cols, n, seed):
        """Rows of group g (device columns) for n uploaded steps: (row columns, row count)."""
        torch = _torch()
        L = _capi.load()
        dev = self.device
        cap = (4 if g["reflector"] == 0 else 2) * n
        out = {k: torch.empty((max(cap, 1), 3) if k in ("s", "d") else max(cap, 1),
                              dtype=torch.int64 if k in ROW_INT else torch.float64, device=dev)
               for k in _capi.LOOKUP_ROW_COLS}
        wsb = L.crv_lookup_rows_workspace(n)
        if self.ws is None or self.ws.numel() < wsb:
            self.ws = torch.empty(int(wsb) + 1024, dtype=torch.uint8, device=dev)
        n_rows = torch.zeros(1, dtype=torch.int64, device=dev)
        S = _capi.CrvLookupSteps(*[cols[k].data_ptr() for k in _capi.LOOKUP_STEP_COLS + ("bar", "pdg")])
        O = _capi.CrvSubstepRowsOut(*[out[k].data_ptr() for k in _capi.LOOKUP_ROW_COLS])
        self.status.reset()
        _capi.check(L.crv_lookup_rows(ctypes.byref(self._group_c(g)), ctypes.c_uint32(int(seed) & 0xFFFFFFFF),
                                      ctypes.byref(S), n, ctypes.byref(O), cap, _capi.ptr(n_rows), _capi.ptr(self.ws),
                                      self.ws.numel(), _stream(), self.status.ptr), "crv_lookup_rows")
        return out, int(n_rows.item())

    def make_photons(self, steps, pdg, seed):
        """photons.make_photons with lookup tables: (step index, channel, arrival time) device tensors, groups in the
        reference's order, rows of a group in (SiPM, step) order and their photons in (row, substep, table, arrival)
        order.  Steps with a non-finite start or end time are skipped, as the reference does."""
        torch = _torch()
        n = len(pdg)
        cols = self.upload_steps(steps, pdg)
        parts = []
        for g in self.groups:
            out, m = self.rows(g, cols, n, seed)
            if m == 0:
                continue
            st, ch, tm = self.substeps.run(g["DL"], DeviceRows.from_columns(out, m), seed, precision=self.precision)
            parts.append((st, ch, tm))
        if not parts:
            z = torch.zeros(0, dtype=torch.int64, device=self.device)
            return z, z.clone(), torch.zeros(0, dtype=torch.float64, device=self.device)
        return tuple(torch.cat([p[i] for p in parts]) for i in range(3))


def make_photons(steps, pdg, geom, cfg, tables, deviation, seed, device="cuda", precision="fp64"):
    """photons.make_photons(steps, pdg, geom, cfg, tables, deviation, rng) with the lookup-table model on the device and
    keyed draws (seed in place of rng): (step index, channel = 4 bar + SiPM, arrival time) host arrays."""
    st, ch, tm = LookupModel(geom, cfg, tables, deviation, device, precision).make_photons(steps, pdg, seed)
    return st.cpu().numpy(), ch.cpu().numpy(), tm.cpu().numpy()


def synthetic_module_lookup(n_events, seed=0, yield_per_mev=20000.0):
    """The workload's one-module geometry with a synthetic lookup table of its bars (450 cm long, 19.8 mm thick, 50 mm
    wide; 10 x 10 x 45 position bins, arrival probability falling with the distance to the SiPM as the workload's
    two-exponential attenuation, delay weights peaked at distance / 140 mm/ns, fibre decay 5 ns) and `n_events`
    synthetic events of muons crossing the thickness (the workload's steps: bar, position along the bar and across
    its width, time and energy; start and end on the two faces).  Returns (geom, cond, tables, lookup config,
    steps, pdg)."""
    from types import SimpleNamespace
    from . import geometry as GM
    rng = np.random.default_rng(1000 + seed)
    geom = GM.module_geometry()
    cond = GM.default_conditions(geom)
    hl = 2250.0
    edges = {"x": np.linspace(-9.9, 9.9, 11), "y": np.linspace(-25.0, 25.0, 11), "z": np.linspace(-hl, hl, 46),
             "beta": np.linspace(0.455, 1.0, 6), "theta": np.linspace(0, np.pi, 12), "phi": np.linspace(0, np.pi, 6),
             "r": np.linspace(0, 0.616, 6)}
    nb = {k: len(v) - 1 for k, v in edges.items()}
    zc = 0.5 * (edges["z"][1:] + edges["z"][:-1])
    d = zc + hl                                              # distance to the SiPM end at -half length

    def table(n_per_z, z_of, scale):
        zi = z_of(np.arange(n_per_z * nb["z"]))
        dist = d[zi]
        prob = (scale * (0.3 * np.exp(-dist / 1000.0) + 0.7 * np.exp(-dist / 5000.0))).astype(np.float32)
        j = np.arange(150)[None, :]
        peak = 3.0 + dist[:, None] / 140.0
        delays = np.rint(12.0 * np.exp(-0.5 * ((j - peak) / 2.5) ** 2)).astype(np.uint8)
        delays[:, 0] |= (delays.sum(1) == 0).astype(np.uint8)
        emis = rng.integers(1, 20, (len(prob), 8)).astype(np.uint8)
        return SimpleNamespace(prob=prob, delays=delays, delay_sum=delays.sum(1, dtype=np.int32), emis=emis,
                               emis_sum=emis.sum(1, dtype=np.int32))

    # bin index layouts: scint (x, y, z) and ckscint (x, y, z, beta) with z before beta; ckfiber z last
    nxy = nb["x"] * nb["y"]
    L = SimpleNamespace(name="module450", reflector=0, half_thickness=9.9, half_width=25.0, half_length=hl,
                        fiber_separation=26.0, hole_radius_x=2.0, hole_radius_y=1.0, fiber_radius=0.7,
                        corner_radius=1.75, fiber_decay_time=5.0, edges=edges,
                        ck_scint=np.array([[0.6, 0.0], [1.0, 12.0]]), ck_fiber=np.array([[0.6, 0.0], [1.0, 6.0]]),
                        tables={"scint": table(nxy, lambda i: i % nb["z"], 2.5e-3),
                                "ckscint": table(nxy * nb["beta"], lambda i: (i // nb["beta"]) % nb["z"], 1e-3),
                                "ckfiber": table(nb["beta"] * nb["theta"] * nb["phi"] * nb["r"],
                                                 lambda i: i % nb["z"], 1e-3)})
    lcfg = SimpleNamespace(sectors={"EX": SimpleNamespace(table="module450", reflector=0, yield_per_mev=yield_per_mev)},
                           photon_yield_scale=1.0, photon_yield_variation_scale=1.0, speed_ratio={}, atten_ratio={})
    st = GM.synthetic_steps(n_events, geom, seed=seed, dtype=np.float64)
    bar = np.asarray(st["bar"])
    n = len(bar)
    cy = geom.center[bar, 1]
    half = geom.halflen[bar, 1]
    x, z, t = (np.asarray(st[k], np.float64) for k in ("x", "z", "t"))
    steps = {"x0": x, "x1": x.copy(), "y0": cy - half, "y1": cy + half, "z0": z, "z1": z.copy(),
             "px0": np.zeros(n), "py0": np.full(n, 1000.0), "pz0": np.zeros(n), "p1": np.full(n, 999.0),
             "t0": t, "t1": t + 0.08, "edep": np.asarray(st["edep"], np.float64), "len": 2.0 * half, "bar": bar,
             "event": np.asarray(st["event"]), "subrun": np.asarray(st["subrun"]), "run": np.asarray(st["run"])}
    return geom, cond, {"module450": L}, lcfg, steps, np.full(n, 13, np.int64)
