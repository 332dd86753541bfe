"""Coupling tables of the reference's 'husimi' lattice (library/Parameters.py, package layout).

Run by hand where the T-Nalg sources are mounted, with ``TNALG_REFERENCE`` set to their directory
(required)::

    TNALG_REFERENCE=<path to T-Nalg> python tests/golden/make_husimi_tables.py

The package layout's plotting imports are stubbed by ``ref_shim.install_package_layout``. Writes ``husimi_tables.npz`` for depths 2 and 3.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_shim  # noqa: E402

ref_shim.install_package_layout()
from library import Parameters as LP  # noqa: E402


def main():
    out = {}
    for depth in (2, 3):
        p = LP.generate_parameters_dmrg("husimi")
        p["depth"] = depth
        p = LP.make_consistent_parameter_dmrg(p)
        for k in ("index1", "index2", "coeff1", "coeff2", "positions_h2"):
            out["d%d_%s" % (depth, k)] = np.asarray(p[k])
        out["d%d_l" % depth] = np.asarray(p["l"])
        out["d%d_op" % depth] = np.stack([np.real(np.asarray(o)) for o in p["op"]])
    np.savez_compressed(os.path.join(HERE, "husimi_tables.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
