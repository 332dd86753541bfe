"""Result files: ``save_pr`` / ``load_pr`` (drop-in for T-Nalg's BasicFunctionsSJR.py:25-89).

A result file is a pickled dict {name: value}, e.g. ``(ob, A, info, para)`` of a DMRG run.
``load_pr`` also reads files written by the reference: its ``MpsOpenBoundaryClass``
instances (pickled under the module names ``MPSClass`` / ``library.MPSClass``) are restored
as this package's class, with the tensors uploaded to the device given by ``device``.
Files written here hold host (numpy) tensors in the reference layout.
"""
import os
import pickle

from . import MPSClass as _mps

# reference module -> this package's module, for classes found in reference result files
_MODULES = {
    "MPSClass": "tnalg_gb300.MPSClass",
    "library.MPSClass": "tnalg_gb300.MPSClass",
    "Parameters": "tnalg_gb300.Parameters",
    "library.Parameters": "tnalg_gb300.Parameters",
}


class _Unpickler(pickle.Unpickler):
    def find_class(self, module, name):
        return super().find_class(_MODULES.get(module, module), name)


def mkdir(path):
    """Create the folder (and its parents) if it does not exist; returns whether it existed
    (BasicFunctionsSJR.py:92-104)."""
    path = path.strip().rstrip("\\")
    existed = os.path.exists(path) if path else True
    if not existed:
        os.makedirs(path)
    return existed


def save_pr(path, file, data, names):
    """Save data[k] under names[k] as one pickled dict in path/file (BasicFunctionsSJR.py:25-50)."""
    mkdir(path)
    tmp = {names[i]: data[i] for i in range(len(names))}
    with open(os.path.join(path, file), "wb") as s:
        pickle.dump(tmp, s)


def load_pr(path_file, names=None, *, device=None):
    """Load a file written by save_pr (BasicFunctionsSJR.py:53-89).

    names None: the whole dict; a string: that entry; a list/tuple: a tuple of those entries.
    Returns False when the file does not exist, as the reference does. ``device`` (default
    'cuda') is where MPS objects read from the file are placed. (The reference wraps a single
    string name's value in tuple(), which splits strings and fails for objects; here it is
    returned as is.)
    """
    if not os.path.isfile(path_file):
        return False
    token = _mps.LOAD_DEVICE.set(device or "cuda")
    try:
        with open(path_file, "rb") as s:
            tmp = _Unpickler(s).load()
    finally:
        _mps.LOAD_DEVICE.reset(token)
    if names is None:
        return tmp
    if isinstance(names, str):
        return tmp[names]
    return tuple(tmp[n] for n in names)
