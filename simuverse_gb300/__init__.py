"""GB300-native D2Q9 lattice-Boltzmann step (simuverse's fluid path) over liblbm.so.

``FluidSimulator`` mirrors simuverse's fluid simulator API; the compute runs in the
hand-written sm_103a kernels of ``csrc/`` behind the C ABI of ``include/lbm.h``.
"""
from ._native import INFO_DTYPE, LbmError, load  # noqa: F401
from .batch import BatchSimulator, generate_domains  # noqa: F401
from .fluid import FluidSimulator  # noqa: F401

__all__ = ["FluidSimulator", "BatchSimulator", "generate_domains", "LbmError", "INFO_DTYPE", "load"]
