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
