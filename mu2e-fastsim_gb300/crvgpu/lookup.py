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
ROW_REAL = ("t0", "t1", "beta", "theta", "dev")
ROW_INT = ("nsub", "step", "chan", "n_scint", "n_ck_s", "n_ck_f")


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

    def c(self):
        S = _capi.CrvLookup(*[self.geometry[k] for k in GEOMETRY])
        for i, e in enumerate(self.edges):
            S.edges[i] = e.data_ptr()
            S.nedges[i] = int(e.numel())
        S.cos_phi_edges = self.cos_phi.data_ptr()
        for i, t in enumerate(self.tables):
            n, nd, ne = t["shape"]
            S.table[i] = _capi.CrvLookupTable(t["prob"].data_ptr(), t["delays"].data_ptr(), t["delay_sum"].data_ptr(),
                                              t["emis"].data_ptr(), t["emis_sum"].data_ptr(), n, nd, ne, 0)
        return S


class DeviceRows:
    """(step, SiPM) substep rows on the device (CrvSubstepRows)."""

    def __init__(self, rows, device="cuda"):
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
        mu = rows.get("mu")
        self.mu = f64(mu) if mu is not None else None
        self.ints = {k: i64(rows[k]) for k in ROW_INT}

    def c(self):
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        return _capi.CrvSubstepRows(p(self.s), p(self.d), *[p(self.real[k]) for k in ROW_REAL], p(self.mu),
                                    *[p(self.ints[k]) for k in ROW_INT])


class SubstepEngine:
    """Workspace and launcher of crv_substep_photons (output capacity grows on demand)."""

    def __init__(self, device="cuda"):
        self.device = device
        self.ws = None
        self.per_row = 64.0
        self.status = _capi.DeviceStatus(device)

    def run(self, DL: DeviceLookup, R: DeviceRows, seed, max_tries=3):
        torch = _torch()
        L = _capi.load()
        dev = self.device
        wsb = L.crv_substeps_workspace(R.n)
        if self.ws is None or self.ws.numel() < wsb:
            self.ws = torch.empty(int(wsb) + 1024, dtype=torch.uint8, device=dev)
        S, C = DL.c(), R.c()
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


def substep_photons(L, rows, seed, device="cuda"):
    """photons._substep_photons(L, rows, rng) with keyed draws: (step index, channel, arrival time) host arrays in
    (row, substep, table, arrival) order.  L: a lookup table object (or a DeviceLookup); rows: the reference's row
    dict (s, d, t0, t1, nsub, beta, theta, dev, optional mu, step, chan, n_scint, n_ck_s, n_ck_f)."""
    DL = L if isinstance(L, DeviceLookup) else DeviceLookup(L, device)
    if device not in _ENGINE:
        _ENGINE[device] = SubstepEngine(device)
    st, ch, tm = _ENGINE[device].run(DL, DeviceRows(rows, device), seed)
    return st.cpu().numpy(), ch.cpu().numpy(), tm.cpu().numpy()
