"""GB300 CRV response engine: CrvSteps -> photons -> SiPM charges -> digis -> reco pulses -> coincidences.

Host code is Python over PyTorch device memory; every stage runs in hand-written sm_103a CUDA behind the C ABI in
include/crvgpu.h (libcrvgpu.so, loaded through ctypes).  There is no CPU fallback.
"""
from . import config  # noqa: F401

__version__ = "0.1.0"
