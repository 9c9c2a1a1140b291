"""Chain glue with the reference's entry points (crv/crvfastsim/chain.py): charges, digis, reco_waveforms, clusters."""
from __future__ import annotations

from .config import CHAN_MULT, PERIOD, ChainConfig, Conditions  # noqa: F401
from .response import charges  # noqa: F401
