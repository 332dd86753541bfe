"""Module-name shim: `from BasicFunctionsSJR import save_pr, load_pr` resolves to tnalg_gb300's result files."""
from tnalg_gb300.BasicFunctionsSJR import *  # noqa: F401,F403
from tnalg_gb300.BasicFunctionsSJR import load_pr, mkdir, save_pr  # noqa: F401
