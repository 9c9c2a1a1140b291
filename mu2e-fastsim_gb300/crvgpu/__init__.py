"""GB300 CRV response engine: CrvSteps -> photons -> SiPM charges -> digis -> reco pulses -> coincidences.

Host code is Python over PyTorch device memory; every stage runs in hand-written sm_103a CUDA behind the C ABI in
include/crvgpu.h (libcrvgpu.so, loaded through ctypes).  There is no CPU fallback.

Modules: chain (the reference's chain entry points and ChainEngine, stage by stage), resident (the whole chain in one
call with explicit capacities, replayed as a CUDA graph), serve (continuous batching of design-point jobs), response /
waveform / pulsefit / coinc (the stages), lookup (the lookup-table photon model), lookup_file (the native reader of the
version-6 lookup-table files, host only), readout (the mask of physically present SiPMs), shard (event partition
across ranks),
config / params / geometry (configuration, launch parameters, geometry and synthetic workloads).
"""
from . import config  # noqa: F401

__version__ = "0.1.0"
