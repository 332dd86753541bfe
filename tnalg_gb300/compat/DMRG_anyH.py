"""Module-name shim: `from DMRG_anyH import dmrg_finite_size` resolves to the GPU implementation."""
from tnalg_gb300.DMRG_anyH import *  # noqa: F401,F403
from tnalg_gb300.DMRG_anyH import dmrg_finite_size, get_bond_energies, positions_set2array, sort_positions  # noqa: F401
