"""Response stages on the GPU: CrvSteps -> photons -> SiPM charges.

Drop-in counterparts of the reference stage functions (same signatures, same flat outputs):
  make_photons(steps, pdg, geom, cfg, tables, deviation, rng)            crv/crvfastsim/response/photons.py:359
  simulate(chan, time, photon, pmap, cfg, rng, t_end, t_start, ...)      crv/crvfastsim/response/sipm.py:102
  charges(steps, parts, geom, cond, cfg, rng, key, ...)                  crv/crvfastsim/chain.py:151

Random numbers come from keyed Philox streams (seed, run, subrun, event, channel, step, photon), so results do not
depend on batching or on the order events are processed in.  The seed is `key` when given, else one draw of the
caller's numpy Generator `rng` (the reference's JAX paths take their seed the same way).
"""
from __future__ import annotations

import ctypes
import time as _time
from dataclasses import dataclass

import numpy as np

from . import _capi, readout
from .config import CHAN_MULT, ChainConfig
from .params import make_params, validate_sipm, validate_window


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the CRV engine needs a CUDA device (no CPU fallback)")
    return torch


def seed_of(rng, key):
    if key is not None:
        return int(key) & 0xFFFFFFFF
    if rng is None:
        return 0
    return int(rng.integers(2 ** 32))


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass
class DeviceSteps:
    """A step table on the device, grouped by event: SoA x, y, z, t, edep (float32 or float64), bar (int32), and the
    event table (event, subrun, run as 32-bit words; first step row, step count)."""
    x: object
    y: object
    z: object
    t: object
    edep: object
    bar: object
    ev_event: object
    ev_subrun: object
    ev_run: object
    ev_first: object
    ev_nsteps: object
    nsteps: int
    nevents: int
    max_steps: int
    order: np.ndarray | None = None     # host permutation applied to the caller's rows (None = identity)

    def c_steps(self):
        rb = 4 if self.x.dtype.itemsize == 4 else 8
        return _capi.CrvSteps(_capi.ptr(self.x), _capi.ptr(self.y), _capi.ptr(self.z), _capi.ptr(self.t),
                              _capi.ptr(self.edep), _capi.ptr(self.bar), rb, 0)

    def c_events(self):
        return _capi.CrvEvents(_capi.ptr(self.ev_event), _capi.ptr(self.ev_subrun), _capi.ptr(self.ev_run),
                               _capi.ptr(self.ev_first), _capi.ptr(self.ev_nsteps))


def _col(steps, a):
    """Midpoint column a (x, y, z or t) of a step table with midpoint or start/end columns."""
    if f"{a}0" in steps and f"{a}1" in steps:
        s0, s1 = steps[f"{a}0"], steps[f"{a}1"]
        if s0 is s1:
            return np.asarray(s0)
        return 0.5 * (np.asarray(s0, float) + np.asarray(s1, float))
    return np.asarray(steps[a])


def upload_steps(steps, device="cuda", dtype=None, nbars=None):
    """Host step table -> DeviceSteps.  Events must be contiguous; they are reordered by increasing event key when they
    are not (the permutation is kept so photon ids refer to the caller's rows)."""
    torch = _torch()
    n = len(np.asarray(steps["bar"]))
    if nbars is not None and n and (np.min(steps["bar"]) < 0 or np.max(steps["bar"]) >= nbars):
        raise ValueError(f"CRV steps: bar index outside [0, {nbars})")
    run = np.asarray(steps["run"], np.int64) if "run" in steps else np.zeros(n, np.int64)
    sub = np.asarray(steps["subrun"], np.int64)
    ev = np.asarray(steps["event"], np.int64)
    evkey = (sub << 20) | ev
    order = None
    if n > 1 and (np.any(np.diff(evkey) < 0) or np.any((np.diff(evkey) == 0) & (np.diff(run) != 0))):
        order = np.lexsort((np.arange(n), run, evkey))
        run, sub, ev, evkey = run[order], sub[order], ev[order], evkey[order]
    new = np.ones(n, bool)
    if n > 1:
        new[1:] = (evkey[1:] != evkey[:-1]) | (run[1:] != run[:-1])
    first = np.flatnonzero(new)
    cnt = np.diff(np.r_[first, n])
    if len(np.unique(evkey[first])) != len(first):
        raise ValueError("CRV steps: an event key appears in more than one run (labels would collide)")
    x = {a: _col(steps, a) for a in "xyzt"}
    x["edep"] = np.asarray(steps["edep"])
    dt = dtype or (np.float32 if all(np.asarray(x[k]).dtype == np.float32 for k in x) else np.float64)
    cols = {}
    for k, v in x.items():
        v = np.asarray(v, dt)
        cols[k] = torch.from_numpy(np.ascontiguousarray(v if order is None else v[order])).to(device)
    bar = np.asarray(steps["bar"], np.int32)
    bar = bar if order is None else bar[order]
    u32 = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.int64).astype(np.uint32).view(np.int32))).to(device)  # noqa: E731
    return DeviceSteps(x=cols["x"], y=cols["y"], z=cols["z"], t=cols["t"], edep=cols["edep"],
                       bar=torch.from_numpy(np.ascontiguousarray(bar)).to(device),
                       ev_event=u32(ev[first]), ev_subrun=u32(sub[first]), ev_run=u32(run[first]),
                       ev_first=torch.from_numpy(first.astype(np.int64)).to(device),
                       ev_nsteps=torch.from_numpy(cnt.astype(np.int32)).to(device), nsteps=n, nevents=len(first),
                       max_steps=int(cnt.max()) if len(cnt) else 0, order=order)


@dataclass
class PinnedSteps:
    """A step table staged in pinned host memory with its event table (see pin_steps); to_device copies it with
    asynchronous copies on the current stream."""
    cols: dict
    nsteps: int
    nevents: int
    max_steps: int

    def to_device(self, device="cuda") -> DeviceSteps:
        c = {k: v.to(device, non_blocking=True) for k, v in self.cols.items()}
        return DeviceSteps(x=c["x"], y=c["y"], z=c["z"], t=c["t"], edep=c["edep"], bar=c["bar"],
                           ev_event=c["ev_event"], ev_subrun=c["ev_subrun"], ev_run=c["ev_run"],
                           ev_first=c["ev_first"], ev_nsteps=c["ev_nsteps"], nsteps=self.nsteps,
                           nevents=self.nevents, max_steps=self.max_steps)

    @property
    def nbytes(self):
        return sum(v.numel() * v.element_size() for v in self.cols.values())


def pin_steps(steps, nbars=None) -> PinnedSteps:
    """Host step table -> the device layout of upload_steps, in pinned host memory (events grouped and keyed once
    on the host, so a later transfer is a set of plain copies)."""
    torch = _torch()
    ds = upload_steps(steps, device="cpu", nbars=nbars)
    if ds.order is not None:
        raise ValueError("pin_steps: events must be contiguous and in increasing key order")
    cols = {k: getattr(ds, k).pin_memory() for k in ("x", "y", "z", "t", "edep", "bar", "ev_event", "ev_subrun",
                                                       "ev_run", "ev_first", "ev_nsteps")}
    return PinnedSteps(cols, ds.nsteps, ds.nevents, ds.max_steps)


def check_photon_map(pm):
    """The photon map's capability rule (crv/crvfastsim/response_config.py:288-290): finite, non-negative 40 x 40
    weights with a positive, finite sum (the pixel draw samples bins by their running sums)."""
    p = np.asarray(pm, float)
    if p.shape != (40, 40) or not np.isfinite(p).all() or np.any(p < 0) or not np.isfinite(p.sum()) or p.sum() <= 0:
        raise ValueError("photon_map: require finite nonnegative 40x40 weights with positive sum")


class PixelTables:
    """Photon-map running sums and dead-pixel bitmap of a SiPM configuration on the device."""

    def __init__(self, sc, pmap=None, device="cuda"):
        torch = _torch()
        pm = np.ones((40, 40)) if pmap is None else np.asarray(pmap, float)
        check_photon_map(pm)
        self.uniform_map = bool(np.all(pm == pm.flat[0]))
        self.cum = torch.from_numpy(np.cumsum(pm.ravel())).to(device)
        words = np.zeros(64, np.uint32)                  # pixel ids x * 41 + y over the 41 x 41 state (53 words used)
        for x, y in sc.inactive:
            if not (0 <= x < 41 and 0 <= y < 41):
                raise ValueError(f"SiPM inactive pixel ({x}, {y}) is outside the 41 x 41 pixel state")
            q = x * 41 + y
            words[q >> 5] |= np.uint32(1) << np.uint32(q & 31)
        self.dead_bits = torch.from_numpy(words.view(np.int32)).to(device)

    def c_pixels(self):
        return _capi.CrvPixels(_capi.ptr(self.cum), _capi.ptr(self.dead_bits))


class DeviceTables:
    """Per-bar geometry, per-channel conditions and SiPM pixel tables on the device."""

    def __init__(self, geom, cond, cfg: ChainConfig, device="cuda", pmap=None):
        torch = _torch()
        self.device = device
        nb = geom.nbars
        ax = np.asarray(geom.local_to_world)[:, 2].astype(np.int8)
        r = np.arange(nb)
        self.length_axis = torch.from_numpy(ax).to(device)
        self.center_l = torch.from_numpy(np.asarray(geom.center, float)[r, ax].copy()).to(device)
        self.half_l = torch.from_numpy(np.asarray(geom.halflen, float)[r, ax].copy()).to(device)
        self.nbars = nb
        rc = cfg.response
        status = effective_status(cond)
        check_readout_mask(cond, nb)
        dev = (np.asarray(cond.deviation, float) * rc.photon_yield_variation_scale + 1.0) * rc.photon_yield_scale
        f64 = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float64))).to(device)  # noqa: E731
        i32 = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.int32))).to(device)    # noqa: E731
        self.yield_factor = f64(dev)
        self.status = i32(status)
        self.roc = i32(cond.roc)
        self.feb = i32(cond.feb)
        self.pedestal, self.pulsearea = f64(cond.pedestal), f64(cond.pulsearea)
        self.pulseheight, self.timeoffset = f64(cond.pulseheight), f64(cond.timeoffset)
        self.nchan = len(status)
        if self.nchan < 4 * nb:
            raise ValueError(f"conditions cover {self.nchan} channels, the geometry has {4 * nb}")
        self.pixels = PixelTables(cfg.sipm, pmap, device)
        self.uniform_map = self.pixels.uniform_map

    def c_bars(self):
        return _capi.CrvBars(_capi.ptr(self.length_axis), _capi.ptr(self.center_l), _capi.ptr(self.half_l),
                             self.nbars, 0)

    def c_channels(self):
        return _capi.CrvChannels(_capi.ptr(self.yield_factor), _capi.ptr(self.status), _capi.ptr(self.roc),
                                 _capi.ptr(self.feb), _capi.ptr(self.pedestal), _capi.ptr(self.pulsearea),
                                 _capi.ptr(self.pulseheight), _capi.ptr(self.timeoffset), self.nchan, 0)

    def c_pixels(self):
        return self.pixels.c_pixels()


def check_readout_mask(cond, nbars):
    """The engine keeps one status table per channel: the readout-masked status (readout.effective_status), which the
    response needs to drop absent SiPMs.  The reference's reco stages read the unmasked status, and the finder reads it
    for a pulse's same-side partner SiPM (PE compensation, crv/crvfastsim/reco/coinc.py:312-314).  With masks that
    cover whole bar sides, as readout.sensor_mask builds them, the two agree wherever a pulse can exist; a mask that
    splits a side (SiPM 0 without 2, or 1 without 3) would not, and is refused."""
    mask = getattr(cond, "readout_mask", None)
    if mask is None:
        return
    m = np.asarray(mask, bool)[:4 * nbars].reshape(-1, 4)
    if np.any(m[:, 0] != m[:, 2]) or np.any(m[:, 1] != m[:, 3]):
        raise NotImplementedError("readout masks must cover whole bar sides (SiPMs 0 and 2, 1 and 3 together), "
                                  "as readout.sensor_mask builds them")


def effective_status(cond):
    """Status with bit 0 set for physically absent sensors (crvgpu.readout.effective_status; the reference's
    crv/crvfastsim/readout.py:58-72), as an array."""
    return np.asarray(readout.effective_status(cond))


class EngineError(RuntimeError):
    pass


def raise_status(flags, need, what):
    if flags:
        nd = {k: int(need[v]) for k, v in _capi.NEED.items() if need[v]}
        raise EngineError(f"{what}: {_capi.status_string(flags)} {nd}")


@dataclass
class ResponseResult:
    """Device outputs of the response stage (torch tensors) and sizes."""
    label: object
    time: object
    charge: object
    pe: object
    photon: object
    n: int
    sipm_label: object
    sipm_photons: object
    sipm_fired: object
    nsipm: int


class ResponseEngine:
    """Reusable workspace + launcher for crv_response (capacities grow on demand, fail-closed)."""

    def __init__(self, device="cuda"):
        self.device = device
        self.ws = None
        self.photon_per_step = 300.0
        self.out_factor = 0.6
        self.status = _capi.DeviceStatus(device)

    def run(self, P, ds: DeviceSteps, tabs: DeviceTables, diagnostics=True, max_tries=4):
        torch = _torch()
        L = _capi.load()
        dev = self.device
        for _ in range(max_tries):
            pcap = int(max(1024, self.photon_per_step * ds.nsteps))
            ocap = int(max(1024, self.out_factor * pcap))
            wsb = L.crv_response_workspace(ctypes.byref(P), ds.nevents, ds.nsteps, pcap, ds.max_steps)
            if self.ws is None or self.ws.numel() < wsb:
                self.ws = torch.empty(int(wsb * 1.1) + 1024, dtype=torch.uint8, device=dev)
            out = {k: torch.empty(ocap, dtype=torch.float64, device=dev) for k in ("time", "charge", "pe")}
            out["label"] = torch.empty(ocap, dtype=torch.int64, device=dev)
            out["photon"] = torch.empty(ocap, dtype=torch.int64, device=dev)
            nb = 4 * ds.nsteps
            sl = torch.empty(max(nb, 1), dtype=torch.int64, device=dev) if diagnostics else None
            sp = torch.empty(max(nb, 1), dtype=torch.int32, device=dev) if diagnostics else None
            sf = torch.empty(max(nb, 1), dtype=torch.int32, device=dev) if diagnostics else None
            counts = torch.zeros(2, dtype=torch.int64, device=dev)
            self.status.reset()
            C = _capi.CrvCharges(*[_capi.ptr(out[k]) for k in ("label", "time", "charge", "pe", "photon")])
            rc = L.crv_response(ctypes.byref(P), ctypes.byref(ds.c_events()), ds.nevents, ctypes.byref(ds.c_steps()),
                                ds.nsteps, ds.max_steps, ctypes.byref(tabs.c_bars()),
                                ctypes.byref(tabs.c_channels()), ctypes.byref(tabs.c_pixels()), pcap,
                                ctypes.byref(C), ocap, _capi.ptr(counts[0:1]), _capi.ptr(sl), _capi.ptr(sp),
                                _capi.ptr(sf), nb, _capi.ptr(counts[1:2]), _capi.ptr(self.ws), self.ws.numel(),
                                _stream(), self.status.ptr)
            _capi.check(rc, "crv_response")
            flags, need = self.status.read()
            n, ns = (int(v) for v in counts.cpu().numpy())
            if flags == _capi.ST_CAPACITY and (need[_capi.NEED["PHOTONS_TOTAL"]] or need[_capi.NEED["CHARGES_OUT"]]) \
                    and not need[_capi.NEED["PHOTONS_PER_SIPM"]] and not need[_capi.NEED["STEPS_PER_EVENT"]]:
                npt = need[_capi.NEED["PHOTONS_TOTAL"]]
                if npt:
                    self.photon_per_step = 1.2 * npt / max(ds.nsteps, 1)
                nco = need[_capi.NEED["CHARGES_OUT"]]
                if nco:
                    self.out_factor = 1.2 * nco / max(pcap, 1)
                continue
            raise_status(flags, need, "crv_response")
            return ResponseResult(out["label"][:n], out["time"][:n], out["charge"][:n], out["pe"][:n],
                                  out["photon"][:n], n, sl[:ns] if diagnostics else None,
                                  sp[:ns] if diagnostics else None, sf[:ns] if diagnostics else None, ns)
        raise EngineError("crv_response: capacities did not converge")


_ENGINE = {}


def engine(device="cuda"):
    if device not in _ENGINE:
        _ENGINE[device] = ResponseEngine(device)
    return _ENGINE[device]


def _is_lookup(tabs):
    return isinstance(tabs, dict) and bool(tabs) and all(hasattr(t, "edges") and hasattr(t, "tables")
                                                         for t in tabs.values())


def lookup_charges(steps, pdg, geom, cond, cfg: ChainConfig, tables, seed, pmap=None, timers=None):
    """chain.charges with the lookup-table photon model (crv/crvfastsim/chain.py:197-213): photons of every (step,
    SiPM) row on the device (crvgpu.lookup), SiPMs with status bit 0 or 2 dropped, labels event key * CHAN_MULT +
    channel, then the SiPM stage (simulate) up to the readout window's end.  cfg.lookup: the sector configuration."""
    from . import lookup as LK
    from .geometry import event_key
    timers = timers if timers is not None else {}
    if cfg.lookup is None:
        raise ValueError("the lookup-table photon model needs ChainConfig.lookup (the reference's response block)")
    if pdg is None:
        raise ValueError("the lookup-table photon model needs the particle code of every step (pdg)")
    t0 = _time.perf_counter()
    model = LK.LookupModel(geom, cfg.lookup, tables, cond.deviation, precision=cfg.precision)
    s, c, t = (x.cpu().numpy() for x in model.make_photons(steps, pdg, seed))
    timers["photons_s"] = timers.get("photons_s", 0.0) + _time.perf_counter() - t0
    status = effective_status(cond)
    keep = (status[c] & 0b101) == 0
    s, c, t = s[keep], c[keep], t[keep]
    if len(c) and int(c.max()) >= CHAN_MULT:
        raise ValueError(f"channel {int(c.max())} >= CHAN_MULT {CHAN_MULT}: SiPM labels would overlap the next event")
    col = lambda k: np.asarray(steps[k].to_numpy() if hasattr(steps[k], "to_numpy") else steps[k])  # noqa: E731
    label = event_key({"subrun": col("subrun"), "event": col("event")})[s] * CHAN_MULT + c
    run = col("run")[s] if "run" in getattr(steps, "columns", steps) else None
    t0 = _time.perf_counter()
    Q = simulate(label, t, s, pmap, cfg.sipm, None, t_end=cfg.window[1], key=seed, run=run, precision=cfg.precision)
    timers["sipm_s"] = timers.get("sipm_s", 0.0) + _time.perf_counter() - t0
    timers["photons"] = timers.get("photons", 0) + len(s)
    timers["charges"] = timers.get("charges", 0) + len(Q["time"])
    return {k: Q[k] for k in ("chan", "time", "charge", "pe", "photon")}


def charges(steps, parts, geom, cond, cfg: ChainConfig, rng, key=None, tabs=None, pmap=None, timers=None, pdg=None,
            caps=None):
    """chain.charges: CrvSteps -> SiPM charges (dict chan (label), time, charge, pe, photon; sorted by label, time).
    With lookup tables in `tabs` ({name: lookup table}) and cfg.lookup set, the lookup-table photon model
    (lookup_charges); otherwise the analytic model."""
    if caps is not None:
        raise ValueError("capacities are managed by the engine (fail-closed re-runs)")
    validate_sipm(cfg.sipm)
    validate_window(cfg.window)
    timers = timers if timers is not None else {}
    seed = seed_of(rng, key)
    if _is_lookup(tabs):
        return lookup_charges(steps, pdg, geom, cond, cfg, tabs, seed, pmap=pmap, timers=timers)
    t0 = _time.perf_counter()
    ds = upload_steps(steps, nbars=geom.nbars)
    T = tabs if isinstance(tabs, DeviceTables) else DeviceTables(geom, cond, cfg, pmap=pmap)
    P = make_params(cfg, seed, uniform_map=T.uniform_map)
    R = engine().run(P, ds, T)
    photon = R.photon.cpu().numpy()
    if ds.order is not None:
        photon = ds.order[photon]
    Q = {"chan": R.label.cpu().numpy(), "time": R.time.cpu().numpy(), "charge": R.charge.cpu().numpy(),
         "pe": R.pe.cpu().numpy(), "photon": photon}
    timers["response_s"] = timers.get("response_s", 0.0) + _time.perf_counter() - t0
    timers["photons"] = timers.get("photons", 0) + int(R.sipm_photons.sum().item()) if R.nsipm else 0
    timers["charges"] = timers.get("charges", 0) + R.n
    return Q


def make_photons(steps, pdg, geom, cfg, tables, deviation, rng, key=None, chain_cfg=None):
    """photons.make_photons: (step row, channel = bar*4 + SiPM, arrival time) per photon, in the reference's block
    order (SiPM 0..3, then step, then photon).  cfg: ResponseConfig (analytic model); tables/pdg are not used by it."""
    torch = _torch()
    L = _capi.load()
    ccfg = chain_cfg or ChainConfig(response=cfg)
    seed = seed_of(rng, key)
    ds = upload_steps(steps, nbars=geom.nbars)
    cond_dev = np.zeros(4 * geom.nbars) if deviation is None else deviation
    from .config import Conditions
    n = 4 * geom.nbars
    cond = Conditions(np.zeros(n), np.ones(n), np.ones(n), np.zeros(n), np.zeros(n, np.int64), np.zeros(n, np.int64),
                      np.zeros(n, np.int64), np.asarray(cond_dev, float))
    T = DeviceTables(geom, cond, ccfg)
    P = make_params(ccfg, seed)
    st = _capi.DeviceStatus("cuda")
    step_event = torch.empty(max(ds.nsteps, 1), dtype=torch.int32, device="cuda")
    count = torch.empty(max(4 * ds.nsteps, 1), dtype=torch.int32, device="cuda")
    _capi.check(L.crv_photon_counts(ctypes.byref(P), ctypes.byref(ds.c_events()), ds.nevents,
                                    ctypes.byref(ds.c_steps()), ds.nsteps, ctypes.byref(T.c_bars()),
                                    ctypes.byref(T.c_channels()), _capi.ptr(step_event), _capi.ptr(count),
                                    _stream(), st.ptr), "crv_photon_counts")
    # rows in block order: s * nsteps + i
    c4 = count[:4 * ds.nsteps].view(ds.nsteps, 4).t().contiguous().view(-1).to(torch.int64)
    off = torch.cumsum(c4, 0) - c4
    tot = int(c4.sum().item()) if ds.nsteps else 0
    o = [torch.empty(max(tot, 1), dtype=dt, device="cuda") for dt in (torch.int64, torch.int64, torch.float64,
                                                                       torch.int64)]
    _capi.check(L.crv_photons(ctypes.byref(P), ctypes.byref(ds.c_events()), ds.nevents, ctypes.byref(ds.c_steps()),
                              ds.nsteps, ctypes.byref(T.c_bars()), _capi.ptr(step_event), _capi.ptr(count),
                              _capi.ptr(off), *[_capi.ptr(x) for x in o], _stream(), st.ptr), "crv_photons")
    flags, need = st.read()
    raise_status(flags, need, "make_photons")
    s, c, t, k = (x[:tot].cpu().numpy() for x in o)
    if ds.order is not None:
        s = ds.order[s]
    return s, c, t, k


def simulate(chan, time, photon, pmap, cfg, rng, t_end=1e5, t_start=0.0, thermal_chans=None, chunk=20000, key=None,
             draw_key=None, run=None, precision="fp64"):
    """sipm.simulate: SiPM charges for photon arrivals (dict chan, time, charge, pe, photon), sorted by (chan, time).

    chan: SiPM label per photon (event key * 32768 + channel); draw_key: per-photon draw key (step-in-event << 16 |
    photon; default: index of the photon within its SiPM in input order); run: run number per photon (default 0)."""
    torch = _torch()
    L = _capi.load()
    validate_sipm(cfg)
    chan = np.asarray(chan, np.int64)
    time = np.asarray(time, float)
    photon = np.asarray(photon, np.int64)
    n = len(chan)
    o = np.argsort(chan, kind="stable")
    lab = chan[o]
    u, start, cnt = np.unique(lab, return_index=True, return_counts=True)
    if draw_key is None:
        dk = np.arange(n) - np.repeat(start, cnt)
    else:
        dk = np.asarray(draw_key, np.int64)[o]
    rn = np.zeros(len(u), np.uint32) if run is None else np.asarray(run, np.int64)[o][start].astype(np.uint32)
    ccfg = ChainConfig(sipm=cfg, window=(t_start, t_end), precision=precision)
    P = make_params(ccfg, seed_of(rng, key), t_end=t_end, uniform_map=pmap is None or bool(
        np.all(np.asarray(pmap) == np.asarray(pmap).flat[0])))
    T = PixelTables(cfg, pmap)
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).astype(dt)).to("cuda")  # noqa: E731
    G = len(u)
    gstart, gcount, glabel = d(start, np.int64), d(cnt, np.int32), d(u, np.int64)
    grun = d(rn.view(np.int32), np.int32)
    tt, kk, pp = d(time[o], np.float64), d(dk, np.int64), d(photon[o], np.int64)
    wsb = L.crv_sipm_workspace(ctypes.byref(P), G, n)
    ws = torch.empty(max(int(wsb), 1), dtype=torch.uint8, device="cuda")
    ocap = max(2 * n + 16 * G, 16)
    out = {k: torch.empty(ocap, dtype=torch.float64, device="cuda") for k in ("time", "charge", "pe")}
    out["label"] = torch.empty(ocap, dtype=torch.int64, device="cuda")
    out["photon"] = torch.empty(ocap, dtype=torch.int64, device="cuda")
    nq = torch.zeros(1, dtype=torch.int64, device="cuda")
    gch = torch.empty(max(G, 1), dtype=torch.int32, device="cuda")
    gfi = torch.empty(max(G, 1), dtype=torch.int32, device="cuda")
    st = _capi.DeviceStatus("cuda")
    C = _capi.CrvCharges(*[_capi.ptr(out[k]) for k in ("label", "time", "charge", "pe", "photon")])
    _capi.check(L.crv_sipm(ctypes.byref(P), ctypes.byref(T.c_pixels()), G, n, _capi.ptr(gstart), _capi.ptr(gcount),
                           _capi.ptr(glabel), _capi.ptr(grun), _capi.ptr(tt), _capi.ptr(kk), _capi.ptr(pp),
                           ctypes.byref(C), ocap, _capi.ptr(nq), _capi.ptr(gch), _capi.ptr(gfi), _capi.ptr(ws),
                           ws.numel(), _stream(), st.ptr), "crv_sipm")
    flags, need = st.read()
    raise_status(flags, need, "sipm.simulate")
    m = int(nq.item())
    res = {"chan": out["label"][:m].cpu().numpy(), "time": out["time"][:m].cpu().numpy(),
           "charge": out["charge"][:m].cpu().numpy(), "pe": out["pe"][:m].cpu().numpy(),
           "photon": out["photon"][:m].cpu().numpy()}
    res["_group_labels"] = u
    res["_group_fired"] = gfi[:G].cpu().numpy()
    res["_group_charges"] = gch[:G].cpu().numpy()
    return res
