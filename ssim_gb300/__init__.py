"""ssim_gb300 -- GB300-native (sm_103a) FEM backward-Euler time stepping of tetrahedral stable
Neo-Hookean solids, a drop-in for the hot path of ssim (time_step.hpp, stepper/*.hpp).

The compute lives in the CUDA library libssim_gb300.so (C ABI: include/ssim_gb.h); this package
holds its Python binding (``TimeStep``), the reference-shaped ``libssim`` / ``pyssim`` mirrors, the
mesh generators and the benchmark scenes.
"""
from . import mesh
from ._lib import DeviceTimeout, NumericalError, SsimGbError, default_params, launch_count, lib, mesh_csr_pattern
from .timestep import TimeStep

__all__ = ["TimeStep", "mesh", "lib", "default_params", "launch_count", "mesh_csr_pattern", "SsimGbError",
           "NumericalError", "DeviceTimeout"]
__version__ = "0.1.0"
