"""How well the reference's own pulse fit defines its results (CPU, the oracle against the reference's fixtures).

The fit (crv/crvfastsim/reco/pulsefit.py:125-216) is a bounded Levenberg-Marquardt / Gauss-Newton minimisation whose
chi2 is flat to ~1e-16 relative at the minimum.  Changing every exp of the fit model by one ulp, or summing the fit
points in the other order, changes nothing mathematically, yet moves the fitted PE of the worse-conditioned pulses by
more than 1e-9 relative: on these inputs the reference's result itself is not defined to 1e-9.  CUDA's exp and the
GPU's reduction order differ from NumPy's in exactly these ways, so the GPU tests bound each pulse's deviation from the
reference by this per-pulse movement (tests/helpers.py fit_sensitivity), and by 1e-9 where the fit is well defined.
"""
import numpy as np

from crvgpu import config as CF
from tests.helpers import fit_sensitivity


def _set(golden, tag):
    g = golden("pulsefit.npz")
    period = 12.5 if tag == "p125" else float(g["period"][0])
    args = [g[f"{tag}_{k}"] for k in ("adc", "n", "start", "ped", "area", "height")]
    ref = {k[len(tag) + 5:]: g[k] for k in g.files if k.startswith(f"{tag}_out_")}
    return args, CF.RecoConfig(period=period), period, tag in ("uneven", "edge"), ref


def test_last_bit_changes_move_ill_conditioned_fits_beyond_1e9(golden):
    moved = {}
    for tag in ("single", "kpp", "uneven", "edge", "p125"):
        args, cfg, period, full, ref = _set(golden, tag)
        sens, base = fit_sensitivity(args, cfg, period, full)
        # the unperturbed oracle is the reference bit for bit on this machine
        for k in ("pe", "time", "failed", "seq"):
            assert np.array_equal(base[k], ref[k]), (tag, k)
        moved[tag] = (float(sens["pe"].max()), float((sens["pe"] > 1e-9).mean()), float(sens["time"].max()))
        # a one-ulp change never moves a fit by more than a few parts in 1e8 (the fits converge)
        assert sens["pe"].max() < 5e-8 and sens["time"].max() < 1e-9, (tag, moved[tag])
    # the KPP-like and uneven sets hold pulses whose own PE moves beyond 1e-9 (so 1e-9 is not a property of the
    # reference there), while the median pulse is defined to far better than 1e-9
    assert moved["kpp"][0] > 1e-9 and moved["uneven"][0] > 1e-9, moved
    assert moved["kpp"][1] > 0.01 and moved["uneven"][1] > 0.01, moved
    print({t: f"max {m[0]:.2e}, beyond 1e-9 {m[1]:.3f}, time max {m[2]:.1e}" for t, m in moved.items()})
