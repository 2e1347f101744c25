"""GB300-native auxiliary-mode-expansion (AME) propagation for Zandpack.

The package keeps the reference's names for the propagation path
(``mpi_RK4pars_dev``-style tableau, ``mpi_funcs``/``func_step_forward`` kernels,
the ``zand`` driver) and runs them as sm_103a CUDA through ``libzandgpu.so``.
"""
from .constants import HBAR  # noqa: F401

__version__ = "0.1.0"
