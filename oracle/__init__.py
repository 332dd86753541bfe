"""CPU oracle for the finite-size DMRG sweep — TEST INFRASTRUCTURE ONLY.

This package restates, in plain numpy/scipy, the arithmetic of T-Nalg's
finite-size DMRG hot path (``dmrg_finite_size`` in DMRG_anyH.py:18-101 and the
``MpsOpenBoundaryClass`` methods in MPSClass.py it calls). It is the checker for
the CUDA implementation in ``tnalg_gb300``: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of
``bench.py`` may import it. The product path never calls it and has no CPU
fallback.

Parity pin: the oracle is checked against golden vectors produced by running
the unmodified reference (``tests/golden/make_golden.py``): twelve DMRG runs
(spin-1/2 chains with and without fields, periodic, started mid-chain and
stopped early by the convergence test; a spin-1 chain; a 2x4 ladder; a spin-1
jigsaw chain; all-to-all long-range and fully connected chains; the 'square'
lattice; a J1-J2 square lattice in snake order), the two result pickles shipped
with the reference, a dense effective Hamiltonian, the docstring examples of the
contraction primitives and the reference's exact diagonalisation.
"""
