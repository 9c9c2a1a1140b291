"""Shared workload builders for the tests (the workload's one-module geometry and synthetic steps)."""
import numpy as np

from crvgpu import config as CF
from crvgpu import geometry as GM


def workload(n_events=64, seed=0, mean_steps=40.0, noise_per_counter=0.0, n_modules=1):
    geom = GM.module_geometry(n_modules=n_modules)
    cond = GM.default_conditions(geom)
    cfg = CF.ChainConfig()
    steps = GM.synthetic_steps(n_events, geom, seed=seed, mean_steps=mean_steps, noise_per_counter=noise_per_counter)
    return geom, cond, cfg, steps


def run_of(steps):
    run = np.asarray(steps["run"], np.int64)
    evk = (np.asarray(steps["subrun"], np.int64) << 20) | np.asarray(steps["event"], np.int64)
    tab = dict(zip(evk.tolist(), run.tolist()))
    return lambda keys: np.array([tab[int(k)] for k in np.asarray(keys).ravel()], np.int64)


def gumbel(t, A, mu, b):
    z = (t - mu) / b
    return A * np.exp(-z - np.exp(-z))


def uneven_waveforms(rng, W=120, period=12.55, area=400.0):
    """Waveforms of the uneven batched-fit workload: lengths over {32, 64, 128, 256, 512}, 1-12 pulses of
    log-uniform 5-500 PE and beta U(10, 25) ns, pedestal 100 with N(0, 2) ADC noise, clipped to [0, 4095].
    Returns (adc [W, Lmax], n, start_tdc, pedestal, area, height)."""
    lens = rng.choice([32, 64, 128, 256, 512], W)
    L = int(lens.max())
    adc = np.zeros((W, L), np.int64)
    start = rng.integers(0, 200, W)
    for w in range(W):
        n = lens[w]
        t = (start[w] + np.arange(n)) * period
        y = np.zeros(n)
        for _ in range(rng.integers(1, 13)):
            pe = np.exp(rng.uniform(np.log(5), np.log(500)))
            b = rng.uniform(10, 25)
            mu = t[0] + rng.uniform(0, n * period)
            y += gumbel(t, pe * area / b, mu, b)
        adc[w, :n] = np.clip(np.round(y + 100.0 + rng.normal(0, 2.0, n)), 0, 4095)
    return adc, lens, start, np.full(W, 100.0), np.full(W, area), np.full(W, area / 15.0)


# ---------------------------------------------------------------------------------------------------------------------
# Conditioning of the reference's pulse fit: how far its own results move under last-bit changes of its arithmetic

FIT_KEYS = ("pe", "peph", "time", "height", "beta", "chi2", "letime", "ped", "fit_A", "fit_mu", "fit_b")


def _perturbed_exp(mode, ulps=1):
    """np.exp moved by `ulps` ulps: all up, all down, or up / down by a hash of the value (two hash variants)."""
    def f(x, *a, **k):
        v = np.exp(x)
        up = np.full(np.shape(v), mode == "up")
        if mode.startswith("hash"):
            mult = np.uint64(0x9E3779B97F4A7C15 if mode == "hash" else 0xC2B2AE3D27D4EB4F)
            up = ((np.asarray(v).view(np.uint64) * mult) >> np.uint64(63)).astype(bool)
        for _ in range(ulps):
            v = np.where(up, np.nextafter(v, np.inf), np.nextafter(v, -np.inf))
        return v
    return f


def _perturbed_solve(a, b):
    """np.linalg.solve with the matrix moved by one ulp per element (up / down by a hash of its bits): another
    rounding of the same normal equations, as a different elimination order or a fused multiply-add gives."""
    a = np.asarray(a, float)
    up = ((a.view(np.uint64) * np.uint64(0x9E3779B97F4A7C15)) >> np.uint64(63)).astype(bool)
    return np.linalg.solve(np.where(up, np.nextafter(a, np.inf), np.nextafter(a, -np.inf)), b)


def fit_sensitivity(args, cfg, period, full, ref=None):
    """Per-pulse relative movement of the oracle's pulse fit (the reference's LM schedule, pulsefit.py:125-216) under
    changes that leave the mathematics unchanged: every exp of the fit model one ulp up, one ulp down, or one or two
    ulps up / down by a hash of its value (two hashes); the fit points summed in reverse order; the normal-equation
    matrix moved by one ulp per element before the solve.  These are the differences between NumPy's and CUDA's exp
    (each within about one ulp of the true value, so up to two apart), between two reduction orders and between two
    roundings of the 3x3 solve (LAPACK's elimination with fused multiply-adds against an unfused one).  Returns ({key: per-pulse max relative
    movement}, the unperturbed oracle result); ref (the reference's own outputs) adds |oracle - ref| as one more
    sample, so a platform whose NumPy exp differs from the fixture generator's is covered too.  Perturbations that
    change the pulse list or a failure flag are left out (none do on the committed fixtures)."""
    import types
    from oracle import oracle as O
    fit0 = O.fit_gumbel

    def reverse(t, y, mask, p0, lo, hi, iterations=40):
        return fit0(t[:, ::-1], y[:, ::-1], mask[:, ::-1], p0, lo, hi, iterations)

    def call():
        if full:
            return O.reconstruct_full(*args, cfg, period)
        return O.reconstruct(*args, cfg, period)

    base = call()
    sens = {k: np.zeros(len(base["pe"])) for k in FIT_KEYS}
    variants = []
    modes = [("up", 1), ("down", 1), ("hash", 1), ("hash2", 1), ("hash", 2), ("hash2", 2), ("reverse", 0),
             ("solve", 0)]
    for mode, ulps in modes:
        fake = types.SimpleNamespace(**{k: getattr(np, k) for k in dir(np) if not k.startswith("__")})
        if mode == "reverse":
            O.fit_gumbel = reverse
        else:
            if mode == "solve":
                fake.linalg = types.SimpleNamespace(solve=_perturbed_solve, eigvalsh=np.linalg.eigvalsh,
                                                    LinAlgError=np.linalg.LinAlgError)
            else:
                fake.exp = _perturbed_exp(mode, ulps)
            O.fit_gumbel = types.FunctionType(fit0.__code__, {**fit0.__globals__, "np": fake}, "fit_gumbel",
                                              fit0.__defaults__)
        try:
            variants.append(call())
        finally:
            O.fit_gumbel = fit0
    if ref is not None:
        variants.append(ref)
    ok = ~np.asarray(base["failed"], bool)
    for r in variants:
        if len(r["pe"]) != len(base["pe"]) or not np.array_equal(np.asarray(r["failed"], bool), ~ok):
            continue
        for k in FIT_KEYS:
            a, b = np.asarray(r[k], float), np.asarray(base[k], float)
            rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
            rel[a == b] = 0.0
            sens[k] = np.maximum(sens[k], rel)
    return sens, base


def fit_windows(args, cfg, period, full):
    """The fit window of every pulse of the oracle's reconstruction, in output order: (times, samples, mask) of the
    points the bounded LM fit minimises over (recorded from the oracle's fit calls: one call per round, its rows the
    round's waveforms in increasing order)."""
    from oracle import oracle as O
    fit0 = O.fit_gumbel
    calls = []

    def record(t, y, mask, p0, lo, hi, iterations=40):
        calls.append((t.copy(), y.copy(), mask.copy()))
        return fit0(t, y, mask, p0, lo, hi, iterations)
    O.fit_gumbel = record
    try:
        r = O.reconstruct_full(*args, cfg, period) if full else O.reconstruct(*args, cfg, period)
    finally:
        O.fit_gumbel = fit0
    wf, seq = np.asarray(r["wf"]), np.asarray(r["seq"])
    out = []
    for i in range(len(wf)):
        rows = np.flatnonzero(seq == seq[i])
        k = int(np.searchsorted(wf[rows], wf[i]))
        t, y, m = calls[int(seq[i])]
        out.append((t[k], y[k], m[k]))
    return out


def window_chi2(win, A, mu, b):
    """chi2 of the Gumbel A exp(-z - exp(-z)), z = (t - mu) / b over a fit window (the fit's objective, FP64)."""
    t, y, m = win
    z = (t - mu) / b
    return float((((y - A * np.exp(-z - np.exp(-z))) * m) ** 2).sum())



def module_lookup(n_events, seed=0, yield_per_mev=20000.0):
    """The workload's module with a synthetic lookup table and muon-crossing steps (crvgpu.lookup.synthetic_module_lookup)."""
    from crvgpu.lookup import synthetic_module_lookup
    return synthetic_module_lookup(n_events, seed=seed, yield_per_mev=yield_per_mev)
