"""Module-name shim: `from MPSClass import MpsOpenBoundaryClass` resolves to the GPU implementation."""
from tnalg_gb300.MPSClass import *  # noqa: F401,F403
from tnalg_gb300.MPSClass import MpsBasic, MpsOpenBoundaryClass  # noqa: F401
