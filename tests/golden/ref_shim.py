"""Import shim for running the unmodified T-Nalg reference in this container.

Used ONLY by ``make_golden.py`` (fixture generation, run by hand where the
reference sources are mounted). Nothing under ``tests/`` that runs in the test
suite imports this module, and the GPU machine never needs it.

The reference targets numpy 1.x / 2018 scipy and needs four compatibility
patches to import and run; none of them changes its arithmetic:

1. stub modules for ``termcolor``, ``ipdb`` and ``matplotlib`` (not installed);
2. ``np.mat`` / ``np.complex`` aliases removed in numpy 2
   (used at Parameters.py:175 and HamiltonianModule.py:13);
3. ``observe_bond_energy`` / ``observe_magnetization`` results ravelled so the
   ``'%g' % ob['e_per_site']`` print at DMRG_anyH.py:86 gets a scalar;
4. ``eigs`` receives ``v0`` ravelled: scipy's ARPACK restart path rejects the
   (n, 1) start vector passed at MPSClass.py:804.
"""
import os
import sys
import types

import numpy as np

REF_ROOT = os.environ.get("TNALG_REFERENCE")
if not REF_ROOT:
    raise RuntimeError("set TNALG_REFERENCE to the directory of the T-Nalg sources")


def install():
    tc = types.ModuleType("termcolor")
    tc.cprint = lambda *a, **k: None
    tc.colored = lambda s, *a, **k: s
    sys.modules["termcolor"] = tc
    ip = types.ModuleType("ipdb")
    ip.set_trace = lambda *a, **k: None
    sys.modules["ipdb"] = ip
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt
    if not hasattr(np, "mat"):
        np.mat = np.asmatrix
    if not hasattr(np, "complex"):
        np.complex = complex
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    import MPSClass

    C = MPSClass.MpsOpenBoundaryClass
    if not getattr(C, "_shimmed", False):
        ob, om = C.observe_bond_energy, C.observe_magnetization
        C.observe_bond_energy = lambda self, *a, **k: np.ravel(ob(self, *a, **k))
        C.observe_magnetization = lambda self, *a, **k: np.ravel(om(self, *a, **k))
        e = MPSClass.eigs
        counter = {"matvec": 0, "solves": 0}

        def eigs1(A, k=6, **kw):
            if kw.get("v0") is not None:
                kw["v0"] = np.ravel(kw["v0"])
            counter["solves"] += 1
            return e(A, k=k, **kw)

        MPSClass.eigs = eigs1
        MPSClass._shim_counter = counter
        C._shimmed = True
    return MPSClass


def install_package_layout():
    """Also make the package layout (``library.*``) importable: it imports matplotlib.cm and
    mpl_toolkits.mplot3d for plotting helpers, stubbed here (nothing plots)."""
    install()
    for name in ("matplotlib.cm", "mpl_toolkits", "mpl_toolkits.mplot3d"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["matplotlib"].cm = sys.modules["matplotlib.cm"]
    sys.modules["matplotlib.cm"].coolwarm = None
    sys.modules["mpl_toolkits.mplot3d"].Axes3D = object
