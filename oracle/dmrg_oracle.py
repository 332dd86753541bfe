"""numpy restatement of T-Nalg's one-site finite-size DMRG (TEST INFRASTRUCTURE ONLY).

Every function cites the reference lines whose arithmetic it restates. The
effective operators are cached per (term, bond) and rebuilt only when a tensor
they pass through changes; the reference keeps a similar cache
(MPSClass.py:202-325) but additionally rebuilds its identity environments at
every site (MPSClass.py:491-502). Both give the same matrices, so the oracle's
results equal the reference's while it runs faster.

Conventions (same as the reference): an MPS tensor is a numpy array of shape
(chi_left, d, chi_right); environments are (chi, chi) matrices indexed
[bra, ket]; the effective Hamiltonian acts on the flattened centre tensor.
"""
import numpy as np
from scipy.sparse.linalg import LinearOperator, eigsh


# ---------------------------------------------------------------------------
# model input


def canonical_terms(index1, coeff1, index2, coeff2, ops, tol):
    """Filter and orient the coupling lists the way the environment builder uses them.

    One-body rows [site, op] are kept when |coeff| > tol and ||op|| > tol, two-body
    rows [i, j, op_i, op_j] when |coeff| > tol (MPSClass.py:643-652). Two-body
    rows are oriented so that i < j (environment_s1_s2 sorts the positions,
    MPSClass.py:345-347).
    """
    one, two = [], []
    index1 = np.asarray(index1).reshape(-1, 2) if np.size(index1) else np.zeros((0, 2), int)
    index2 = np.asarray(index2).reshape(-1, 4) if np.size(index2) else np.zeros((0, 4), int)
    c1 = np.ravel(np.asarray(coeff1, dtype=float)) if np.size(coeff1) else np.zeros(0)
    c2 = np.ravel(np.asarray(coeff2, dtype=float)) if np.size(coeff2) else np.zeros(0)
    for n in range(index1.shape[0]):
        q, sn = int(index1[n, 0]), int(index1[n, 1])
        if abs(c1[n]) > tol and np.linalg.norm(np.reshape(ops[sn], -1)) > tol:
            one.append((q, sn, float(c1[n])))
    for n in range(index2.shape[0]):
        i, j, a, b = (int(x) for x in index2[n])
        if abs(c2[n]) > tol:
            if i > j:
                i, j, a, b = j, i, b, a
            two.append((i, j, a, b, float(c2[n])))
    return one, two


# ---------------------------------------------------------------------------
# tensor primitives (TensorBasicModule.py)


def random_open_mps(l, d, chi):
    """Global-RNG draw order of TensorBasicModule.py:181-186: site 0, site l-1, then 1..l-2."""
    mps = [None] * l
    mps[0] = np.random.randn(1, d, chi)
    mps[l - 1] = np.random.randn(chi, d, 1)
    for n in range(1, l - 1):
        mps[n] = np.random.randn(chi, d, chi)
    return mps


def left2right_decompose(t, way="qr"):
    """TensorBasicModule.py:314-348: reshape (chi_l*d, chi_r), QR or SVD, keep min(rows, cols)."""
    s = t.shape
    dim = min(s[0] * s[1], s[2])
    m = t.reshape(s[0] * s[1], s[2])
    if way == "svd":
        u, lm, v = np.linalg.svd(m, full_matrices=False)
        v = np.diag(lm[:dim]).dot(v[:dim, :])
        q = u
    else:
        q, v = np.linalg.qr(m)
        lm = np.zeros(0)
    return q[:, :dim].reshape(s[0], s[1], dim), v.T, dim, lm


def right2left_decompose(t, way="qr"):
    """TensorBasicModule.py:351-384: QR/SVD of the transpose of (chi_l, d*chi_r)."""
    s = t.shape
    m = t.reshape(s[0], s[1] * s[2])
    dim = min(s[0], s[1] * s[2])
    if way == "svd":
        u, lm, v = np.linalg.svd(m.T, full_matrices=False)
        v = np.dot(np.diag(lm[:dim]), v[:dim, :])
        q = u
    else:
        q, v = np.linalg.qr(m.T)
        lm = np.zeros(0)
    return q[:, :dim].T.reshape(dim, s[1], s[2]), v.T, dim, lm


def absorb_matrix2tensor(t, mat, bond):
    """TensorBasicModule.py:387-424: contract the FIRST index of mat with bond `bond` of t."""
    return np.moveaxis(np.tensordot(t, mat, ([bond], [0])), -1, bond)


def transfer_left(t, op=None, v=None):
    """TensorBasicModule.py:530-573: v'[b', b] = sum conj(t)[a', s', b'] v[a', a] op[s', s] t[a, s, b]."""
    t1 = t if op is None else np.einsum("xs,asb->axb", op, t)
    if v is not None:
        t1 = np.tensordot(v, t1, ([1], [0]))
    s = t.shape
    return t.conj().reshape(s[0] * s[1], s[2]).T.dot(t1.reshape(s[0] * s[1], s[2]))


def transfer_right(t, op=None, v=None):
    """TensorBasicModule.py:576-619: v'[a', a] = sum conj(t)[a', s', b'] op[s', s] t[a, s, b] v[b', b]."""
    t1 = t if op is None else np.einsum("xs,asb->axb", op, t)
    tc = t.conj()
    if v is not None:
        tc = np.tensordot(tc, v, ([2], [0]))
    s = t.shape
    return tc.reshape(s[0], s[1] * s[2]).dot(t1.reshape(s[0], s[1] * s[2]).T)


def entanglement_entropy(lm, tol=1e-20):
    """TensorBasicModule.py:786-801: S = -2 sum lm^2 ln lm over lm > tol (sorted descending)."""
    lm = np.sort(np.reshape(lm, -1))[::-1]
    lm = lm[lm > tol]
    return float(-2.0 * np.dot(lm ** 2, np.log(lm)))


# ---------------------------------------------------------------------------
# MPS with cached effective operators


class OracleMPS:
    """Open-boundary MPS restating MpsOpenBoundaryClass (MPSClass.py:53-1098).

    ``center``/``virtual_dim``/``orthogonality``/``lm``/``ent`` follow the
    reference's meaning (MPSClass.py:57-72).
    """

    def __init__(self, l, d, chi, ops, mps=None):
        self.length = l
        self.phys_dim = d
        self.ops = [np.real_if_close(np.asarray(o)) for o in ops]
        self.mps = random_open_mps(l, d, chi) if mps is None else [np.array(t, dtype=float) for t in mps]
        self.virtual_dim = np.array([1] + [t.shape[2] for t in self.mps])
        self.center = -1
        self.orthogonality = np.zeros(l)
        self.lm = [np.zeros(0) for _ in range(l - 1)]
        self.ent = np.zeros(l - 1)
        self.decomp_way = "qr"
        self._cache = {}
        self.n_matvec = 0

    # -- gauge --------------------------------------------------------------
    def _changed(self, site):
        """Drop cached operators whose transfer passes through `site` (cf. MPSClass.py:306-325)."""
        self._cache = {k: v for k, v in self._cache.items() if not (v[1] <= site <= v[2])}

    def orthogonalize_mps(self, l0, l1):
        """MPSClass.py:143-167."""
        if l0 < l1:
            for n in range(l0, l1):
                self.mps[n], mat, self.virtual_dim[n + 1], lm = left2right_decompose(self.mps[n], self.decomp_way)
                if lm.size > 0 and self.center > -1:
                    self.lm[n] = lm.copy()
                self.mps[n + 1] = absorb_matrix2tensor(self.mps[n + 1], mat, 0)
                self._changed(n)
                self._changed(n + 1)
            self.orthogonality[l0:l1] = -1
            self.orthogonality[l1] = 0
        elif l0 > l1:
            for n in range(l0, l1, -1):
                self.mps[n], mat, self.virtual_dim[n], lm = right2left_decompose(self.mps[n], self.decomp_way)
                if lm.size > 0 and self.center > -1:
                    self.lm[n - 1] = lm.copy()
                self.mps[n - 1] = absorb_matrix2tensor(self.mps[n - 1], mat, 2)
                self._changed(n)
                self._changed(n - 1)
            self.orthogonality[l1 + 1:l0 + 1] = 1
            self.orthogonality[l1] = 0

    def correct_orthogonal_center(self, p):
        """MPSClass.py:188-198 (explicit p >= 0)."""
        if self.center < 0:
            self.orthogonalize_mps(0, p)
            self.orthogonalize_mps(self.length - 1, p)
        elif self.center != p:
            self.orthogonalize_mps(self.center, p)
        self.center = p

    # -- effective operators -------------------------------------------------
    def _memo(self, key, lo, hi, fn):
        hit = self._cache.get(key)
        if hit is None:
            hit = (fn(), lo, hi)
            self._cache[key] = hit
        return hit[0]

    def left_one(self, sn, q, b):
        """ops[sn] at site q carried to bond b > q through left-canonical tensors q..b-1
        (get_effective_operators_one_body, MPSClass.py:252-279, left-to-right branch)."""
        if b == q + 1:
            return self._memo(("L1", sn, q, b), q, q, lambda: transfer_left(self.mps[q], self.ops[sn]))
        return self._memo(("L1", sn, q, b), q, b - 1,
                          lambda: transfer_left(self.mps[b - 1], None, self.left_one(sn, q, b - 1)))

    def right_one(self, sn, q, b):
        """ops[sn] at site q carried to bond b <= q through right-canonical tensors b..q
        (MPSClass.py:271-279, right-to-left branch; bond b sits left of site b)."""
        if b == q:
            return self._memo(("R1", sn, q, b), q, q, lambda: transfer_right(self.mps[q], self.ops[sn]))
        return self._memo(("R1", sn, q, b), b, q,
                          lambda: transfer_right(self.mps[b], None, self.right_one(sn, q, b + 1)))

    def left_two(self, a, i, bop, j, b):
        """ops[a] at i and ops[bop] at j (i < j < b) carried to bond b
        (update_effect_from_op1_to_op2, MPSClass.py:504-515)."""
        if b == j + 1:
            return self._memo(("L2", a, i, bop, j, b), i, j,
                              lambda: transfer_left(self.mps[j], self.ops[bop], self.left_one(a, i, j)))
        return self._memo(("L2", a, i, bop, j, b), i, b - 1,
                          lambda: transfer_left(self.mps[b - 1], None, self.left_two(a, i, bop, j, b - 1)))

    def right_two(self, a, i, bop, j, b):
        """Right-side mirror (MPSClass.py:516-525): both ops right of the centre, carried to bond b <= i."""
        if b == i:
            return self._memo(("R2", a, i, bop, j, b), i, j,
                              lambda: transfer_right(self.mps[i], self.ops[a], self.right_one(bop, j, i + 1)))
        return self._memo(("R2", a, i, bop, j, b), b, j,
                          lambda: transfer_right(self.mps[b], None, self.right_two(a, i, bop, j, b + 1)))

    def site_buckets(self, p, one, two):
        """Bucket dictionary of classify_and_update_env (MPSClass.py:684-733) at centre p."""
        env = {}

        def add(key, m):
            env[key] = env[key] + m if key in env else m

        for q, sn, c in one:
            if q < p:
                add("1_0_0", c * self.left_one(sn, q, p))
            elif q == p:
                add("0_%d_0" % sn, c * self.ops[sn])
            else:
                add("0_0_1", c * self.right_one(sn, q, p + 1))
        for i, j, a, b, c in two:
            if j < p:
                add("1_0_0", c * self.left_two(a, i, b, j, p))
            elif i > p:
                add("0_0_1", c * self.right_two(a, i, b, j, p + 1))
            elif j == p:
                add("1_%d_0" % b, c * self.left_one(a, i, p))
            elif i == p:
                add("0_%d_1" % a, c * self.right_one(b, j, p + 1))
            else:
                env.setdefault("1_0_1", []).append([c, self.left_one(a, i, p), self.right_one(b, j, p + 1)])
        return env

    def apply_heff(self, env, psi):
        """sum over buckets of (L (x) O (x) R) psi (update_tensor_eigs_f_handle_optimized,
        MPSClass.py:755-776, without the identity/tau shift)."""
        out = np.zeros_like(psi)
        for key, m in env.items():
            x = key.split("_")
            if key == "1_0_1":
                for c, lmat, rmat in m:
                    out += c * np.einsum("xa,asb,yb->xsy", lmat, psi, rmat, optimize=True)
            elif x[0] == "1" and x[1] == "0":
                out += np.tensordot(m, psi, ([1], [0]))
            elif x[2] == "1" and x[1] == "0":
                out += np.tensordot(psi, m, ([2], [1]))
            elif x[0] == "0" and x[2] == "0":
                out += np.einsum("xs,asb->axb", m, psi)
            elif x[0] == "1":
                out += np.einsum("xa,ys,asb->xyb", m, self.ops[int(x[1])], psi, optimize=True)
            else:
                out += np.einsum("yb,xs,asb->axy", m, self.ops[int(x[1])], psi, optimize=True)
        return out

    def dense_heff(self, p, one, two):
        """Dense effective Hamiltonian at p (effective_hamiltonian_dmrg, MPSClass.py:532-580)."""
        env = self.site_buckets(p, one, two)
        s = (self.virtual_dim[p], self.phys_dim, self.virtual_dim[p + 1])
        n = int(np.prod(s))
        h = np.zeros((n, n))
        for k in range(n):
            e = np.zeros(n)
            e[k] = 1.0
            h[:, k] = self.apply_heff(env, e.reshape(s)).reshape(-1)
        return h

    def update_tensor_eigs(self, p, one, two, tau, tol):
        """MPSClass.py:778-809 with eig_way=1: eigsh 'LM' of I - tau*H_eff started from the
        current centre tensor; returns the eigenvalue of H_eff."""
        self.correct_orthogonal_center(p)
        env = self.site_buckets(p, one, two)
        s = self.mps[p].shape
        dim = int(np.prod(s))

        def mv(a):
            self.n_matvec += 1
            a = np.reshape(a, s)
            return (a - tau * self.apply_heff(env, a)).reshape(-1)

        op = LinearOperator((dim, dim), matvec=mv, dtype=float)
        w, v = eigsh(op, k=1, which="LM", v0=self.mps[p].reshape(-1), tol=tol)
        self.mps[p] = np.real(v[:, 0]).reshape(s)
        self._changed(p)
        return float((1.0 - w[0]) / tau)

    # -- observables -----------------------------------------------------------
    def expect(self, sites_ops):
        """<prod_k ops[op_k] at site_k> using the canonical form around the centre
        (observation_s1 / observation_s1_s2, MPSClass.py:857-909)."""
        c = self.center
        pos = dict()
        for q, sn in sites_ops:
            pos[q] = self.ops[sn] if q not in pos else self.ops[sn].dot(pos[q])
        lo = min(min(pos), c)
        hi = max(max(pos), c)
        v = None
        for n in range(lo, hi + 1):
            v = transfer_left(self.mps[n], pos.get(n), v)
        return float(np.trace(v))

    def observe_magnetization(self, sn):
        """MPSClass.py:911-921."""
        return np.array([self.expect([(i, sn)]) for i in range(self.length)])

    def observe_bond_energy(self, index2, coeff2):
        """MPSClass.py:923-934: coeff * <op_i op_j> for every row, unfiltered."""
        index2 = np.asarray(index2).reshape(-1, 4)
        c2 = np.ravel(np.asarray(coeff2, dtype=float))
        return np.array([c2[n] * self.expect([(int(index2[n, 0]), int(index2[n, 2])),
                                              (int(index2[n, 1]), int(index2[n, 3]))])
                         for n in range(index2.shape[0])])

    def observe_correlators_from_middle(self, op1, op2, ob_len=None):
        """MPSClass.py:936-952 (Python's round() for the middle site)."""
        if ob_len is None:
            ob_len = self.length
        corr = []
        pos1 = round(self.length / 2)
        pos2 = pos1 + 1
        n = 0
        while pos1 > -0.1 and pos2 < self.length and ob_len > -0.1:
            corr.append(self.expect([(pos1, op1), (pos2, op2)]))
            if n % 2 == 0:
                pos1 -= 1
            else:
                pos2 += 1
            n += 1
            ob_len -= 1
        return np.array(corr)

    def calculate_entanglement_spectrum(self):
        """MPSClass.py:812-832 (if_fast branch): SVD moves to the ends and back fill lm."""
        way, c0 = self.decomp_way, self.center
        self.decomp_way = "svd"
        p0, p1 = self.length - 1, 0
        for n in range(self.length - 1):
            if self.lm[n].size == 0:
                p0 = min(p0, n)
                p1 = max(p1, n)
        self.correct_orthogonal_center(p0)
        self.correct_orthogonal_center(p1 + 1)
        self.correct_orthogonal_center(c0)
        self.decomp_way = way

    def calculate_entanglement_entropy(self):
        """MPSClass.py:834-839."""
        for i in range(self.length - 1):
            self.ent[i] = -1 if self.lm[i].size == 0 else entanglement_entropy(self.lm[i])


def get_bond_energies(eb_full, positions, index2):
    """DMRG_anyH.py:250-258."""
    positions = np.asarray(positions)
    index2 = np.asarray(index2).reshape(-1, 4)
    eb = np.zeros(positions.shape[0])
    for i in range(index2.shape[0]):
        hit = (index2[i, 0] == positions[:, 0]) & (index2[i, 1] == positions[:, 1])
        eb[np.nonzero(hit)] += eb_full[i]
    return eb


def dmrg_finite_size(l, d, chi, ops, index1, coeff1, index2, coeff2, positions_h2, *, tau, eigs_tol,
                     sweep_time, dt_ob=1, break_tol=-1.0, hx=0.0, hz=0.0, ob_position=0, mps=None,
                     seed=None, final_observables=True):
    """Restates dmrg_finite_size (DMRG_anyH.py:18-101) on plain arrays.

    Returns (ob, A, info): ob keys as in the reference plus 'history' (energy per site after
    every observed sweep) and 'solve_energies' (eigenvalue of H_eff of every local solve).
    """
    if seed is not None:
        np.random.seed(seed)
    A = OracleMPS(l, d, chi, ops, mps=mps)
    one, two = canonical_terms(index1, coeff1, index2, coeff2, A.ops, eigs_tol)
    A.correct_orthogonal_center(ob_position)
    e0 = 0.0
    info = {"convergence": 1.0, "sweeps": 0}
    ob = {"history": [], "solve_energies": []}
    for t in range(sweep_time):
        if_ob = ((t + 1) % dt_ob == 0) or t == sweep_time - 1
        order = list(range(ob_position + 1, l)) + list(range(l - 2, -1, -1)) + list(range(1, ob_position))
        for n in order:
            ob["solve_energies"].append(A.update_tensor_eigs(n, one, two, tau, eigs_tol))
        info["sweeps"] = t + 1
        if if_ob:
            ob["eb_full"] = A.observe_bond_energy(index2, coeff2)
            ob["mx"] = A.observe_magnetization(1)
            ob["mz"] = A.observe_magnetization(3)
            ob["e_per_site"] = (np.sum(ob["eb_full"]) - hx * np.sum(ob["mx"]) - hz * np.sum(ob["mz"])) / l
            ob["history"].append(ob["e_per_site"])
            info["convergence"] = abs(ob["e_per_site"] - e0)
            if info["convergence"] < break_tol:
                break
            e0 = ob["e_per_site"]
    if final_observables:
        ob["eb"] = get_bond_energies(ob["eb_full"], positions_h2, index2)
        A.calculate_entanglement_spectrum()
        A.calculate_entanglement_entropy()
        ob["corr_x"] = A.observe_correlators_from_middle(1, 1)
        ob["corr_z"] = A.observe_correlators_from_middle(3, 3)
    info["n_matvec"] = A.n_matvec
    return ob, A, info
