"""Module-name shim: `import Parameters as pm` resolves to the GPU implementation's parameter builder."""
from tnalg_gb300.Parameters import *  # noqa: F401,F403
