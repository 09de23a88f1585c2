"""GB300-native engine for the per-timestep force-and-integrate path of
jhalverson/surfactant_enhanced_spreading (water / surfactant nanodroplets on
graphite): CUDA kernels for sm_103a behind the C ABI of include/sesp.h, with
a ctypes host layer mirroring the reference driver's calls."""
from .system import System, droplet  # noqa: F401

__all__ = ["System", "droplet", "engine"]
