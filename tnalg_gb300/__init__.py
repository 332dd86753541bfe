"""GB300-native finite-size DMRG sweep with T-Nalg's Python API.

    import numpy as np
    from tnalg_gb300 import Parameters as pm, dmrg_finite_size
    para = pm.generate_parameters_dmrg('chain')
    np.random.seed(0)
    ob, A, info, para = dmrg_finite_size(para)

The numeric work runs in libtnalg_gb300.so (include/tnalg_gb300.h) on one CUDA
device; build it with ``tnalg_gb300.build.build()``.
"""
from . import HamiltonianModule, Parameters  # noqa: F401
from .DMRG_anyH import dmrg_finite_size, get_bond_energies  # noqa: F401
from .Parameters import generate_parameters_dmrg, make_consistent_parameter_dmrg  # noqa: F401


def __getattr__(name):
    if name == "MpsOpenBoundaryClass":
        from .MPSClass import MpsOpenBoundaryClass
        return MpsOpenBoundaryClass
    raise AttributeError(name)
