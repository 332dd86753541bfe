"""MpsOpenBoundaryClass on one GB300 (drop-in for T-Nalg's MPSClass.MpsOpenBoundaryClass).

Constructor signature, attribute names and the methods used by the finite-size
DMRG (MPSClass.py:53-1098) are kept; the tensors live on the GPU and every
numeric step runs in libtnalg_gb300.so. ``mps`` returns host (numpy) copies in
the reference layout, so user code and pickling see the same objects as with
the reference.

Differences a user can observe:
  * ``is_parallel`` / ``is_env_parallel_lmr`` / ``par_pool`` / ``eig_way`` /
    ``is_save_op`` are accepted and ignored: there is one device path, equivalent
    to the reference's eig_way=1 matrix-free local solve with cached operators.
  * Two-body rows with i > j are oriented to i < j (the reference applies the
    wrong site operator for such rows in classify_and_update_env, MPSClass.py:717-728).
  * observe_correlators_from_middle never reads stale cached operators (with
    is_save_op=True the reference's corr_z after calculate_entanglement_spectrum
    does; its is_save_op=False values are what this class returns).
  * Operators must be real (spin 'sy' enters only through complex-free products
    in the Heisenberg expansion).
  * full_coefficients_mps works for any length (the reference's drops a reshape,
    MPSClass.py:983); reduced_density_matrix_one_body (from the package layout,
    library/MPSClass.py:994-999) also works at the orthogonality centre.
"""
import contextvars
import functools

import numpy as np
import torch

from . import _lib as L
from . import engine as E
from .HamiltonianModule import spin_operators

# device for MPS objects restored from a reference result file (set by BasicFunctionsSJR.load_pr)
LOAD_DEVICE = contextvars.ContextVar("tnalg_load_device", default="cuda")


def on_device(fn):
    """Run a method with the MPS's device current. Every C-ABI call works on the current device
    and launches on its current stream, so an MPS on cuda:1 used while cuda:0 is current would
    otherwise queue kernels on a cuda:0 stream with cuda:1 pointers."""
    @functools.wraps(fn)
    def wrapper(self, *args, **kwargs):
        dev = self._dev.device
        if dev.type == "cuda" and dev.index is not None and not L._host_test and \
                dev.index != torch.cuda.current_device():
            with torch.cuda.device(dev):
                return fn(self, *args, **kwargs)
        return fn(self, *args, **kwargs)
    return wrapper


def random_open_mps(l, d, chi):
    """Global numpy RNG, draw order of TensorBasicModule.py:181-186 (site 0, site l-1, then 1..l-2)."""
    mps = [None] * l
    mps[0] = np.random.randn(1, d, chi)
    mps[l - 1] = np.random.randn(chi, d, 1)
    for n in range(1, l - 1):
        mps[n] = np.random.randn(chi, d, chi)
    return mps


def ones_open_mps(l, d, chi):
    """TensorBasicModule.py ones_open_mps: all-ones tensors."""
    return [np.ones((1, d, chi))] + [np.ones((chi, d, chi)) for _ in range(l - 2)] + [np.ones((chi, d, 1))]


def entanglement_entropy(lm, tol=1e-20):
    """TensorBasicModule.py:786-801: -2 sum lm^2 ln lm over lm > tol."""
    lm = np.sort(np.reshape(lm, -1))[::-1]
    lm = lm[lm > tol]
    return float(-2.0 * np.dot(lm ** 2, np.log(lm)))


class MpsBasic:
    def __init__(self):
        self.version = "gb300-1"
        self.operators = list()


class MpsOpenBoundaryClass(MpsBasic):
    """Open-boundary MPS (MPSClass.py:26-106) resident on a CUDA device."""

    def __init__(self, length, d, chi, spin="half", way="qr", ini_way="r", operators=None, debug=False,
                 is_parallel=False, is_save_op=False, eig_way=0, par_pool=None, is_env_parallel_lmr=True,
                 device="cuda", precision="fp64", tensors=None):
        MpsBasic.__init__(self)
        self.spin = spin
        self.phys_dim = d
        self.decomp_way = way
        self.length = length
        self.lm = [np.zeros(0) for _ in range(length - 1)]
        self.ent = np.zeros((length - 1, 1))
        if tensors is None:
            if ini_way == "r":
                tensors = random_open_mps(length, d, chi)
            elif ini_way == "1":
                tensors = ones_open_mps(length, d, chi)
            else:
                raise ValueError("ini_way must be 'r' or '1'")
        if operators is None:
            op = spin_operators(spin)
            operators = [op["id"], op["sx"], op["sy"], op["sz"], op["su"], op["sd"]]
        self.operators = operators
        self._is_save_op = is_save_op
        self._is_parallel = is_parallel
        self._is_env_parallel_lmr = is_env_parallel_lmr
        self._debug = debug
        self.eig_way = eig_way
        self.pool = None
        # refine: None = FP64 Rayleigh quotient after every mixed-precision solve, 0/1 = never/always,
        # "last" = only for solves flagged with refine_next_solve() (dmrg_finite_size flags the last
        # solve of every sweep)
        self.lanczos = {"max_krylov": 40, "max_restarts": 50, "check_every": 3, "tol_cap": 0.0,
                        "mixed_floor": 2e-6, "refine": "last", "refine_cycles": 4}
        self._refine_next = False
        # split-TF32 path: when set, every local solve refines its vector to the FP64 tolerance
        # (restart cycles opened by an FP64 matvec, refine == 2 of tn_lanczos); dmrg_finite_size
        # sets it for the final sweeps, whose local solves fix the accuracy of the returned state
        self.refine_vectors = False
        self.last_solve = None
        # two-body couplings: False carries one operator per open (site, op) as the reference does;
        # True carries rank-compressed combinations (engine.CompressedModel); "auto" picks the
        # compressed model when it saves at least a quarter of the carried operators
        self.coupling_compress = False
        self.coupling_tol = 1e-14
        self._model_key = None
        self._dev = E.DeviceMPS(tensors, d, device, precision=precision)
        self.solve_energies = []

    # -- reference attributes ---------------------------------------------------
    @property
    def mps(self):
        return self._dev.numpy_tensors()

    @property
    def mps_device(self):
        return self._dev.mps

    @property
    def virtual_dim(self):
        return self._dev.virtual_dim

    @property
    def center(self):
        return self._dev.center

    @center.setter
    def center(self, value):
        self._dev.center = value

    @property
    def orthogonality(self):
        return self._dev.orthogonality.reshape(-1, 1)

    @property
    def precision(self):
        return {v: k for k, v in L.PRECISIONS.items() if k in ("fp64", "tf32x3")}[self._dev.precision]

    @on_device
    def set_precision(self, precision):
        self._dev.precision = L.PRECISIONS[precision]
        self._dev.set_model(None)
        self._model_key = None

    @property
    def stats(self):
        return self._dev.stats

    # -- gauge -------------------------------------------------------------------
    @on_device
    def orthogonalize_mps(self, l0, l1):
        """MPSClass.py:143-167 (QR moves; 'svd' moves also record the Schmidt values)."""
        if self.decomp_way == "svd":
            self._svd_moves(l0, l1)
        else:
            self._dev.orthogonalize_mps(l0, l1)

    @on_device
    def central_orthogonalization(self, lc, l0=0, l1=-1):
        """MPSClass.py:170-185."""
        if l1 == -1:
            l1 = self.length - 1
        self.orthogonalize_mps(l0, lc)
        self.orthogonalize_mps(l1, lc)
        self._dev.center = lc

    @on_device
    def correct_orthogonal_center(self, p=-1):
        """MPSClass.py:188-198."""
        if p < -0.5 and self.center < -0.5:
            p = self.check_orthogonal_center(if_print=False)
        elif p < -0.5:
            p = self.center
        if self.center < -0.5:
            self.central_orthogonalization(p)
        elif self.center != p:
            self.orthogonalize_mps(self.center, p)
        self._dev.center = p

    def check_orthogonal_center(self, expected_center=-2, if_print=True):
        """Centre implied by the orthogonality flags (MPSClass.py:989-1022, without prints)."""
        if self.center > -0.5:
            return self.center
        o = self._dev.orthogonality
        left = np.nonzero(o == -1)[0]
        right = np.nonzero(o == 1)[0]
        lpos = left[-1] if left.size else -1
        if right.size and lpos + 2 == right[0]:
            return lpos + 1
        return lpos + 1

    def _svd_moves(self, l0, l1):
        """QR moves plus the singular values of each R factor (the reference's 'svd' decomposition
        stores lm at MPSClass.py:154-155,163-164; the Schmidt values of a bond are the singular
        values of R). Each R is kept and all of them go through one batched Jacobi call at the
        end: along a sweep of moves the left sites of a bond are left-canonical and the right sites
        right-canonical when its R is formed, so the bonds' spectra are independent."""
        dev = self._dev
        step = 1 if l0 < l1 else -1
        collected = []
        for n in range(l0, l1, step):
            if step > 0:
                dev.qr_left(n)
                bond = n
            else:
                dev.qr_right(n)
                bond = n - 1
            if self.center > -1:
                collected.append((bond, dev._last_r))
        if collected:
            spectra = L.singular_values_batched([R for _, R in collected], ws=dev.ws2)
            for (bond, R), s in zip(collected, spectra):
                self.lm[bond] = s[: min(R.shape)]
        if l0 < l1:
            dev.orthogonality[l0:l1] = -1
            dev.orthogonality[l1] = 0
        elif l0 > l1:
            dev.orthogonality[l1 + 1:l0 + 1] = 1
            dev.orthogonality[l1] = 0

    @on_device
    def grow_bond_dimension(self, chi_new, noise=1e-3, seed=0, method="noise", model=None):
        """Enlarge all bonds to chi_new (capped by d^b) and re-centre the MPS at its previous centre
        (or 0). method 'expand': subspace expansion with a truncated SVD of the Hamiltonian's open
        channels (DeviceMPS.expand_bonds; needs the run's coupling lists, model = (index1, index2,
        coeff1, coeff2, tol)); 'noise': seeded Gaussian noise in the new entries. Not in the
        reference, whose chi is fixed; used by para['chi_schedule']."""
        c = self.center if self.center >= 0 else 0
        if method == "expand":
            self._model(*model)
            # the expansion's gauge moves, like the re-centring after it, may use the
            # mixed-precision QR: the grown state is re-optimised by the next sweep
            self._dev.fast_gauge = True
            try:
                if self._dev.expand_bonds(chi_new, seed=seed):
                    self.lm = [np.zeros(0) for _ in range(self.length - 1)]
                    self.correct_orthogonal_center(c)
            finally:
                self._dev.fast_gauge = False
            return
        if method != "noise":
            raise ValueError("method must be 'expand' or 'noise'")
        if self._dev.grow_bonds(chi_new, noise=noise, seed=seed):
            self.lm = [np.zeros(0) for _ in range(self.length - 1)]
            # the grown state is re-optimised by the next sweep: its gauge moves may use the
            # mixed-precision QR
            self._dev.fast_gauge = True
            try:
                self.correct_orthogonal_center(c)
            finally:
                self._dev.fast_gauge = False

    # -- local update ------------------------------------------------------------
    def _model(self, index1, index2, coeff1, coeff2, tol):
        key = (id(index1), id(index2), id(coeff1), id(coeff2), float(tol), str(self.coupling_compress),
               float(self.coupling_tol),
               np.asarray(index2).tobytes(), np.asarray(coeff2, dtype=float).tobytes(),
               np.asarray(index1).tobytes(), np.asarray(coeff1, dtype=float).tobytes())
        if key != self._model_key:
            one, two = E.canonical_terms(index1, coeff1, index2, coeff2, self.operators, tol)
            used = {sn for _, sn, _ in one} | {a for *_, a, b, c in two} | {b for *_, b, c in two}
            for k in used:
                if np.any(np.abs(np.imag(np.asarray(self.operators[k], dtype=complex))) > 0):
                    raise ValueError("operator %d is complex; the GPU path is real FP64" % k)
            model = E.make_model(self.length, self.phys_dim, self.operators, one, two, self._dev.device,
                                 compress=self.coupling_compress, tol=self.coupling_tol)
            self._dev.set_model(model)
            self._model_key = key
        return self._dev.model

    @on_device
    def update_tensor_eigs(self, p, index1, index2, coeff1, coeff2, tau, is_real, tol=1e-16):
        """MPSClass.py:778-809: move the centre to p and replace site p by the lowest eigenvector
        of its effective Hamiltonian. Returns the eigenvalue of H_eff."""
        self._model(index1, index2, coeff1, coeff2, tol)
        if self.decomp_way == "svd":
            self.correct_orthogonal_center(p)
        else:
            self._dev.move_center_for_solve(p)
        o = self.lanczos
        refine = o["refine"]
        if refine == "last":  # FP64 Rayleigh quotient only when the caller marks the solve
            refine = 1 if self._refine_next else 0
        if self.refine_vectors and self._dev.precision == L.PREC_TF32X3:
            refine = 2
        self._refine_next = False
        res = self._dev.solve(p, tol, tau, tol_cap=o["tol_cap"], max_krylov=o["max_krylov"],
                              max_restarts=o["max_restarts"], check_every=o["check_every"], refine=refine,
                              mixed_floor=o["mixed_floor"], refine_cycles=o.get("refine_cycles", 4))
        self.last_solve = res
        e = res.energy_fp64 if res.energy_fp64 != 0.0 or res.energy == 0.0 else res.energy
        self.solve_energies.append(e)
        return e

    def refine_next_solve(self):
        """Have the next update_tensor_eigs end with an FP64 residual and Rayleigh quotient."""
        self._refine_next = True

    @on_device
    def effective_hamiltonian_dmrg(self, p, index1, index2, coeff1, coeff2, tol=1e-12):
        """Dense H_eff at the centre p (MPSClass.py:532-580), built column by column with
        tn_matvec; only for small bond dimensions."""
        self._model(index1, index2, coeff1, coeff2, tol)
        self.correct_orthogonal_center(p)
        s = [int(x) for x in self._dev.mps[p].shape]
        n = int(np.prod(s))
        eye = torch.eye(n, dtype=torch.float64, device=self._dev.device)
        cols = [self._dev.apply_heff(p, eye[k].reshape(s), precision=L.PREC_FP64) for k in range(n)]
        h = torch.stack([c.reshape(-1) for c in cols], dim=1)
        return h.cpu().numpy(), s

    # -- observables ---------------------------------------------------------------
    def _ensure_obs_model(self):
        if self._dev.model is None:
            self._dev.set_model(E.Model(self.length, self.phys_dim, self.operators, [], [], self._dev.device))

    @on_device
    def observe_magnetization(self, sn):
        """MPSClass.py:911-921: <operators[sn]> on every site, shape (length, 1)."""
        self._ensure_obs_model()
        v1, _ = E.observe(self._dev, [(i, sn) for i in range(self.length)], [])
        return v1.reshape(-1, 1)

    @on_device
    def observe_bond_energy(self, index2, coeff2):
        """MPSClass.py:923-934: coeff * <op_i op_j> for every row of index2, shape (nh, 1)."""
        self._ensure_obs_model()
        idx = np.asarray(index2).reshape(-1, 4)
        c2 = np.ravel(np.asarray(coeff2, dtype=float))
        _, v2 = E.observe(self._dev, [], [tuple(int(x) for x in r) for r in idx])
        return (c2 * v2).reshape(-1, 1)

    @on_device
    def observation_s1(self, inputs):
        sn, position = inputs
        self._ensure_obs_model()
        return float(E.observe(self._dev, [(int(position), int(sn))], [])[0][0])

    @on_device
    def observation_s1_s2(self, inputs):
        ssn, positions = inputs
        self._ensure_obs_model()
        q = (int(positions[0]), int(positions[1]), int(ssn[0]), int(ssn[1]))
        return float(E.observe(self._dev, [], [q])[1][0])

    @on_device
    def observe_correlators_from_middle(self, op1, op2, ob_len=None):
        """MPSClass.py:936-952 (Python round() of length/2 for the middle site)."""
        self._ensure_obs_model()
        if ob_len is None:
            ob_len = self.length
        pairs = []
        pos1 = round(self.length / 2)
        pos2 = pos1 + 1
        n = 0
        while pos1 > -0.1 and pos2 < self.length and ob_len > -0.1:
            pairs.append((pos1, pos2, op1, op2))
            if n % 2 == 0:
                pos1 -= 1
            else:
                pos2 += 1
            n += 1
            ob_len -= 1
        if not pairs:
            return np.zeros(0)
        # O(N^2) transfer steps: the mixed-precision path runs them in split TF32 (~1e-7 of the
        # correlations); energies and one-site observables stay FP64
        return E.observe(self._dev, [], pairs, precision=self._dev.precision)[1]

    @on_device
    def calculate_entanglement_spectrum(self, if_fast=True):
        """MPSClass.py:812-832: moves to the ends and back fill lm. The reference takes an SVD at
        every move of the three passes; the spectra do not depend on the pass, and the middle
        pass crosses every bond that is filled, so only its moves record singular values (one
        batched call). On the mixed-precision path the moves use the mixed-precision QR (the
        state is then kept to ~1e-7)."""
        way, c0 = self.decomp_way, self.center
        self._dev.fast_gauge = True
        try:
            if if_fast and c0 > -0.5:
                p0, p1 = self.length - 1, 0
                for n in range(self.length - 1):
                    if self.lm[n].size == 0:
                        p0 = min(p0, n)
                        p1 = max(p1, n)
                self.correct_orthogonal_center(p0)
                self.decomp_way = "svd"
                self.correct_orthogonal_center(p1 + 1)
                self.decomp_way = way
                self.correct_orthogonal_center(c0)
            else:
                self.correct_orthogonal_center(0)
                self.decomp_way = "svd"
                self.correct_orthogonal_center(self.length - 1)
                self.decomp_way = way
                if c0 > 0:
                    self.correct_orthogonal_center(c0)
        finally:
            self.decomp_way = way
            self._dev.fast_gauge = False

    def calculate_entanglement_entropy(self):
        """MPSClass.py:834-839."""
        for i in range(self.length - 1):
            self.ent[i] = -1 if self.lm[i].size == 0 else entanglement_entropy(self.lm[i])

    @on_device
    def reduced_density_matrix_two_body(self, p1, p2):
        """MPSClass.py:841-855: the (d^2, d^2) reduced density matrix of sites p1, p2 with trace 1,
        rho[(s1 s2), (s1' s2')] = sum_rest psi*(.. s1 .. s2 ..) psi(.. s1' .. s2' ..), computed on the
        device at the current centre. The reference takes p1 < p2; p1 > p2 gives the matrix with
        the sites in the order passed."""
        if p1 == p2:
            raise ValueError("reduced_density_matrix_two_body needs two different sites")
        if self.center < 0:
            raise RuntimeError("reduced_density_matrix_two_body needs a central-orthogonal MPS")
        self._ensure_obs_model()
        q1, q2 = min(p1, p2), max(p1, p2)
        rho = E._Observer(self._dev).two_site_density(q1, q2)
        if p1 > p2:
            d = self.phys_dim
            rho = rho.reshape(d, d, d, d).transpose(1, 0, 3, 2).reshape(d * d, d * d)
        return rho / np.trace(rho)

    def _site_rhos(self, sites):
        if self.center < 0:
            raise RuntimeError("one-site density matrices need a central-orthogonal MPS "
                               "(call correct_orthogonal_center first)")
        self._ensure_obs_model()
        out = []
        for g in E._Observer(self._dev).site_densities(list(sites)):
            rho = g + g.T
            out.append(rho / np.trace(rho))
        return out

    @on_device
    def reduced_density_matrix_one_body(self, p):
        """library/MPSClass.py:994-999: the (d, d) density matrix of site p, symmetrised (rho + rho^T)
        and normalised to trace 1, computed on the device. The reference's version fails when p is
        the orthogonality centre (its transfer from the centre to p is empty); here any site works."""
        return self._site_rhos([p])[0]

    @on_device
    def calculate_onsite_entanglement_entropy(self):
        """library/MPSClass.py:1001-1038: (ent, rho) with rho[n] the one-site density matrix of site n
        (as reduced_density_matrix_one_body) and ent[n] = -sum lm ln lm over its eigenvalues > 1e-25."""
        rho = self._site_rhos(range(self.length))
        ent = np.zeros((self.length,))
        for n, r in enumerate(rho):
            lm = np.linalg.eigvalsh(r)
            lm = lm[lm > 1e-25]
            ent[n] = -np.inner(lm, np.log(lm))
        return ent, rho

    @on_device
    def full_coefficients_mps(self, tol_memory=20):
        """MPSClass.py:968-985: all d^L amplitudes psi[s_0 ... s_(L-1)] (s_0 slowest) as a (d^L, 1)
        array, contracted site by site with tn_gemm. The reference drops the result of its reshape
        (MPSClass.py:983) and fails for three or more sites; it also refuses, as here, when
        L log2(d) - 5 exceeds tol_memory (returns None)."""
        tot_size_log2 = self.length * np.log2(self.phys_dim) - 5
        if tot_size_log2 > tol_memory:
            print("The memory cost of the total coefficients is too large (a lot more than %d Mb). Stop "
                  "calculation; pass a larger tol_memory to compute it anyway" % tot_size_log2)
            return None
        mps = self._dev.mps
        x = mps[0].reshape(-1, mps[0].shape[2])
        for n in range(1, self.length):
            cl, d, cr = (int(v) for v in mps[n].shape)
            y = torch.empty((x.shape[0], d * cr), dtype=torch.float64, device=self._dev.device)
            L.gemm(x, mps[n].contiguous(), y, int(x.shape[0]), d * cr, cl, (cl, 1), (d * cr, 1), (d * cr, 1),
                   ws=self._dev.ws)
            x = y.reshape(-1, cr)
        return x.reshape(-1, 1).cpu().numpy()

    @on_device
    def norm_mps(self):
        """MPSClass.py:954-966 (norm of the centre tensor)."""
        if self.center < -0.5:
            raise RuntimeError("norm_mps needs a central-orthogonal MPS")
        return float(torch.linalg.vector_norm(self._dev.mps[self.center]).item())

    def report_yourself(self):
        print("center: " + str(self.center))
        print("orthogonality:" + str(self.orthogonality.T))
        print("virtual bond dimensions: " + str(self.virtual_dim))

    def clean_to_save(self):
        """MPSClass.py:1090-1098: drop cached environments and the thread pool."""
        self._dev.set_model(None)
        self._model_key = None
        self.pool = None

    # -- pickling: host copies in the reference layout -----------------------------
    def __getstate__(self):
        st = {k: v for k, v in self.__dict__.items() if k != "_dev"}
        st["_mps_host"] = self.mps
        st["_virtual_dim"] = np.array(self.virtual_dim)
        st["_center"] = self.center
        st["_orthogonality"] = np.array(self._dev.orthogonality)
        st["_precision"] = self.precision
        st["_device"] = str(self._dev.device)
        st["last_solve"] = None
        st["_refine_next"] = False
        st["_model_key"] = None
        return st

    def _from_reference_state(self, st):
        """Restore an object pickled by the reference's MpsOpenBoundaryClass (its __dict__, set up at
        MPSClass.py:53-106): tensors, centre, orthogonality flags, spectra and entropies are kept;
        the host operator caches (effect_s / effect_ss and their position tables) are dropped, the
        device environments are rebuilt on first use. Tensors go to LOAD_DEVICE."""
        tensors = [np.asarray(t, dtype=float) for t in st["mps"]]
        d = int(st.get("phys_dim", tensors[0].shape[1]))
        chi = max(int(t.shape[2]) for t in tensors)
        self.__init__(len(tensors), d, chi, spin=st.get("spin", "half"), way=st.get("decomp_way", "qr"),
                      operators=st.get("operators"), debug=bool(st.get("_debug", False)),
                      is_parallel=bool(st.get("_is_parallel", False)), is_save_op=bool(st.get("_is_save_op", False)),
                      eig_way=int(st.get("eig_way", 0)), device=LOAD_DEVICE.get(), tensors=tensors)
        vd = np.ravel(np.asarray(st.get("virtual_dim", self._dev.virtual_dim))).astype(int)
        if vd.shape != self._dev.virtual_dim.shape or (vd != self._dev.virtual_dim).any():
            raise ValueError("pickled virtual_dim %s does not match the tensors %s" % (vd, self._dev.virtual_dim))
        self._dev.center = int(st.get("center", -1))
        if "orthogonality" in st:
            self._dev.orthogonality = np.ravel(np.asarray(st["orthogonality"], dtype=float)).copy()
        if "lm" in st:
            self.lm = [np.ravel(np.asarray(x, dtype=float)) for x in st["lm"]]
        if "ent" in st:
            self.ent = np.asarray(st["ent"], dtype=float).reshape(-1, 1)

    def __setstate__(self, st):
        if "_mps_host" not in st:
            self._from_reference_state(st)
            return
        tensors = st.pop("_mps_host")
        vd = st.pop("_virtual_dim")
        c = st.pop("_center")
        orth = st.pop("_orthogonality")
        prec = st.pop("_precision")
        dev = st.pop("_device")
        self.__dict__.update(st)
        self._dev = E.DeviceMPS(tensors, self.phys_dim, dev, precision=prec)
        self._dev.virtual_dim = vd
        self._dev.center = c
        self._dev.orthogonality = orth
