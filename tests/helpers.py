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
