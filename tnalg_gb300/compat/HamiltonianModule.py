"""Module-name shim: `import HamiltonianModule as hm` resolves to the GPU implementation's operators."""
from tnalg_gb300.HamiltonianModule import *  # noqa: F401,F403
