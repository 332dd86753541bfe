"""Device-resident one-site DMRG engine behind MpsOpenBoundaryClass.

Host-side orchestration only: every contraction, decomposition and eigen-solve
is a call into libtnalg_gb300.so (include/tnalg_gb300.h).

Effective operators (the reference's effect_s / effect_ss caches and
classify_and_update_env buckets, MPSClass.py:202-325,474-530,684-733) are kept
per bond as one stacked device tensor:

    EL[b] : (1 + |open_left(b)|, chi_b, chi_b)   slot 0 = sum of all terms inside sites < b,
            slot 1+k = operator open_left(b)[k] = (site i, op a) of a two-body term i < b <= j
    ER[b] : (1 + |open_right(b)|, chi_b, chi_b)  mirror for sites >= b

and are updated incrementally when the centre moves (one block-operator GEMM
pair per carried operator) instead of being rebuilt from the chain end as the
reference does (MPSClass.py:491-502).

For long-range coupling lists the carried slots are rank-compressed
combinations of the open operators instead (CompressedModel): a fully
connected chain then carries a constant number of slots per bond instead of
O(N).
"""
import os
from collections import OrderedDict

import numpy as np
import torch

from . import _lib as L


# ---------------------------------------------------------------------------
# coupling-list compiler


def canonical_terms(index1, coeff1, index2, coeff2, ops, tol):
    """Filtered, oriented term lists (the filters of MPSClass.py:643-652).

    One-body rows [site, op] with |coeff| > tol and ||op|| > tol; two-body rows
    [i, j, a, b] with |coeff| > tol, oriented so that i < j (environment_s1_s2
    sorts positions, MPSClass.py:345-347; the orientation also fixes the
    operator used for the '1_sn_0' / '0_sn_1' buckets).
    """
    one, two = [], []
    idx1 = np.asarray(index1).reshape(-1, 2) if np.size(index1) else np.zeros((0, 2), int)
    idx2 = np.asarray(index2).reshape(-1, 4) if np.size(index2) else np.zeros((0, 4), int)
    c1 = np.ravel(np.asarray(coeff1, dtype=float)) if np.size(coeff1) else np.zeros(0)
    c2 = np.ravel(np.asarray(coeff2, dtype=float)) if np.size(coeff2) else np.zeros(0)
    for n in range(idx1.shape[0]):
        q, sn = int(idx1[n, 0]), int(idx1[n, 1])
        if abs(c1[n]) > tol and np.linalg.norm(np.reshape(np.asarray(ops[sn]), -1)) > tol:
            one.append((q, sn, float(c1[n])))
    for n in range(idx2.shape[0]):
        i, j, a, b = (int(x) for x in idx2[n])
        if abs(c2[n]) > tol:
            if i == j:
                raise ValueError("two-body term with both operators on site %d" % i)
            if i > j:
                i, j, a, b = j, i, b, a
            two.append((i, j, a, b, float(c2[n])))
    return one, two


class Model:
    """Per-bond / per-site tables derived from the coupling lists (static for a run)."""

    compressed = False

    def __init__(self, length, d, ops, one, two, device):
        self._init_common(length, d, ops, one, two, device)
        Ln = length
        # open operators per bond b (0..L): term (i, j) is open at b iff i < b <= j
        self.open_left = []
        self.open_right = []
        for b in range(Ln + 1):
            lk = OrderedDict()
            rk = OrderedDict()
            for i, j, a, bo, c in two:
                if i < b <= j:
                    lk.setdefault((i, a), None)
                    rk.setdefault((j, bo), None)
            self.open_left.append({k: s + 1 for s, k in enumerate(lk)})
            self.open_right.append({k: s + 1 for s, k in enumerate(rk)})

    def _init_common(self, length, d, ops, one, two, device):
        self.length = length
        self.d = d
        self.device = device
        ops_np = np.stack([np.real(np.asarray(o, dtype=complex)).astype(float) for o in ops])
        if ops_np.shape[1:] != (d, d):
            raise ValueError("operators must be %dx%d" % (d, d))
        self.ops_np = ops_np
        self.ops = torch.tensor(ops_np, dtype=torch.float64, device=device)
        self.one = one
        self.two = two
        Ln = length
        self.one_at = [[] for _ in range(Ln)]
        for q, sn, c in one:
            if not 0 <= q < Ln:
                raise ValueError("one-body term on site %d outside 0..%d" % (q, Ln - 1))
            self.one_at[q].append((sn, c))
        for i, j, a, b, c in two:
            if not (0 <= i < Ln and 0 <= j < Ln):
                raise ValueError("two-body term (%d,%d) outside 0..%d" % (i, j, Ln - 1))
        self._tables = {}
        self._memo = {}

    def n_left(self, b):
        """Carried (non-Hamiltonian) slots of EL[b]."""
        return len(self.open_left[b])

    def n_right(self, b):
        """Carried slots of ER[b]."""
        return len(self.open_right[b])

    # -- block-operator term lists (slot, op, coeff) ----------------------------
    def left_block_terms(self, p):
        """W_L at site p: H_L(p) (x) 1 + 1 (x) O_site(p) + sum_{(i,p)} c C_L(i,a) (x) op_b."""
        t = [(0, -1, 1.0)]
        t += [(-1, sn, c) for sn, c in self.one_at[p]]
        ol = self.open_left[p]
        for i, j, a, b, c in self.two:
            if j == p:
                t.append((ol[(i, a)], b, c))
        return t

    def right_block_terms(self, p, with_site=True):
        """W_R at site p: 1 (x) H_R(p+1) [+ O_site(p) (x) 1] + sum_{(p,j)} c op_a (x) C_R(j,b)."""
        t = [(0, -1, 1.0)]
        if with_site:
            t += [(-1, sn, c) for sn, c in self.one_at[p]]
        orr = self.open_right[p + 1]
        for i, j, a, b, c in self.two:
            if i == p:
                t.append((orr[(j, b)], a, c))
        return t

    def left_carry_plan(self, b):
        """How each slot of EL[b+1] is produced from EL[b] and site b: ('carry', old_slot) or ('fresh', op)."""
        plan = []
        for (i, a), slot in self.open_left[b + 1].items():
            plan.append(("carry", self.open_left[b][(i, a)]) if i < b else ("fresh", a))
        return plan

    def right_carry_plan(self, b):
        """Slots of ER[b] from ER[b+1] and site b."""
        plan = []
        for (j, bo), slot in self.open_right[b].items():
            plan.append(("carry", self.open_right[b + 1][(j, bo)]) if j > b else ("fresh", bo))
        return plan

    def straddle_groups(self, p):
        """Straddling terms i < p < j as sum_g SL_g (x) 1 (x) SR_g, grouped on the smaller side.

        Returns (sl_terms, sr_terms, ngroups) for tn_combine_slots (op field = group id).
        """
        ol, orr = self.open_left[p], self.open_right[p + 1]
        pairs = {}
        for i, j, a, b, c in self.two:
            if i < p < j:
                key = (ol[(i, a)], orr[(j, b)])
                pairs[key] = pairs.get(key, 0.0) + c
        if not pairs:
            return [], [], 0
        us = sorted({u for u, _ in pairs})
        vs = sorted({v for _, v in pairs})
        sl, sr = [], []
        if len(us) <= len(vs):
            for g, u in enumerate(us):
                sl.append((u, g, 1.0))
                for (uu, v), c in pairs.items():
                    if uu == u:
                        sr.append((v, g, c))
            return sl, sr, len(us)
        for g, v in enumerate(vs):
            sr.append((v, g, 1.0))
            for (u, vv), c in pairs.items():
                if vv == v:
                    sl.append((u, g, c))
        return sl, sr, len(vs)

    def table(self, key, terms):
        """Cached device copy of a term list."""
        hit = self._tables.get(key)
        if hit is None:
            hit = L.terms_tensor(terms, self.device)
            self._tables[key] = hit
        return hit

    def table_lazy(self, key, make):
        """table(key, make()) with the term list built only when the key is not cached yet."""
        hit = self._tables.get(key)
        if hit is None:
            hit = L.terms_tensor(make(), self.device)
            self._tables[key] = hit
        return hit

    def memo(self, key, make):
        """A per-model cache of host-side plans (the coupling lists are fixed for a model)."""
        hit = self._memo.get(key)
        if hit is None:
            hit = self._memo[key] = make()
        return hit

    def opidx(self, key, ops):
        hit = self._tables.get(key)
        if hit is None:
            hit = torch.tensor(list(ops) if ops else [0], dtype=torch.int32, device=self.device)
            self._tables[key] = hit
        return hit

    def matrix(self, key, arr):
        """Cached device copy (FP64, contiguous) of a small host coefficient matrix."""
        hit = self._tables.get(key)
        if hit is None:
            hit = torch.tensor(np.ascontiguousarray(arr, dtype=float), dtype=torch.float64, device=self.device)
            self._tables[key] = hit
        return hit


class CompressedModel(Model):
    """Two-body couplings carried as rank-reduced operator combinations (MPO compression).

    The reference carries one effective operator per open (site, op) of every two-body term
    crossing a bond (MPSClass.py:474-530, 684-733), so a fully connected or power-law chain
    ('full' / 'longRange', Parameters.py:244-278) carries O(N) operators per bond and its
    matvec sums O(N) straddling pairs. Here the coupling matrix M[(i,a), (j,b)] (left ports
    i < j) is factorised bond by bond:

      * left basis at bond b: orthonormal columns U_b over the ports (i, a), i < b, spanning
        the columns of M[i < b, j >= b]. Slot 1+k of EL[b] holds sum_(i,a) U_b[(i,a), k] C_L(i, a).
        Moving to bond b+1 the still-needed part lies in span(U_b): its coordinates
        X = U_b^T M[:, j >= b+1] are reduced by an SVD to P (singular values above
        tol * ||M||_2 kept), the carried slots of EL[b+1] are the combinations P^T of the carried
        slots of EL[b] (carry is linear), and the ports of site b enter as fresh slots;
      * right basis V_b mirrors it (rows of M[i < b, j >= b]);
      * W_L at site p takes, per operator b of site p, coefficients U_p^T M[:, (p, b)]; W_R takes
        M[(p, a), :] V_(p+1); the straddling pairs i < p < j become the core
        C = U_p^T M V_(p+1), split by its SVD into rank(C) groups sum_g SL_g (x) 1 (x) SR_g.

    All of this is exact up to the singular values dropped (tol = 1e-14 by default, i.e. the
    couplings to 1e-14 of their spectral norm); a larger tol gives a lossy compression. Uniform
    all-to-all couplings have rank 1 per operator pair, so their environments carry a constant
    number of slots instead of O(N).
    """

    compressed = True

    def __init__(self, length, d, ops, one, two, device, tol=1e-14):
        self._init_common(length, d, ops, one, two, device)
        Ln = length
        lports = sorted({(i, a) for i, j, a, b, c in two})
        rports = sorted({(j, b) for i, j, a, b, c in two})
        self.lports, self.rports = lports, rports
        li = {p: k for k, p in enumerate(lports)}
        ri = {p: k for k, p in enumerate(rports)}
        M = np.zeros((len(lports), len(rports)))
        for i, j, a, b, c in two:
            M[li[(i, a)], ri[(j, b)]] += c
        self.M = M
        lsite = np.array([p[0] for p in lports], dtype=int)
        rsite = np.array([p[0] for p in rports], dtype=int)
        self.lsite, self.rsite = lsite, rsite
        self.cut = float(tol) * (float(np.linalg.norm(M, 2)) if M.size else 0.0)

        # left bases, bond 0 -> L
        self.U = [np.zeros((len(lports), 0))]
        self.lcombine = []   # per site b: (P (r_b x r'), [fresh ops of site b])
        for b in range(Ln):
            U = self.U[b]
            cols = rsite >= b + 1
            P = self._reduce(U.T @ M[:, cols] if (U.shape[1] and cols.any()) else None, U.shape[1], left=True)
            fresh = [k for k in np.nonzero(lsite == b)[0] if np.any(M[k, cols] != 0)]
            Un = np.zeros((len(lports), P.shape[1] + len(fresh)))
            Un[:, :P.shape[1]] = U @ P
            for q, k in enumerate(fresh):
                Un[k, P.shape[1] + q] = 1.0
            self.U.append(Un)
            self.lcombine.append((P, [lports[k][1] for k in fresh]))

        # right bases, bond L -> 0
        self.V = [None] * (Ln + 1)
        self.V[Ln] = np.zeros((len(rports), 0))
        self.rcombine = [None] * Ln
        for b in range(Ln - 1, -1, -1):
            V = self.V[b + 1]
            rows = lsite < b
            P = self._reduce(M[rows, :] @ V if (V.shape[1] and rows.any()) else None, V.shape[1], left=False)
            fresh = [k for k in np.nonzero(rsite == b)[0] if np.any(M[rows, k] != 0)]
            Vn = np.zeros((len(rports), P.shape[1] + len(fresh)))
            Vn[:, :P.shape[1]] = V @ P
            for q, k in enumerate(fresh):
                Vn[k, P.shape[1] + q] = 1.0
            self.V[b] = Vn
            self.rcombine[b] = (P, [rports[k][1] for k in fresh])
        self._straddle = {}

    def _reduce(self, X, r, left):
        """Orthonormal basis (r x r') of the span needed next: left singular vectors of X
        (left side, X = r x cols) or right singular vectors of X (right side, X = rows x r)."""
        if X is None or X.size == 0:
            return np.zeros((r, 0))
        if left:
            P, s, _ = np.linalg.svd(X, full_matrices=False)
            return P[:, s > self.cut]
        _, s, Pt = np.linalg.svd(X, full_matrices=False)
        return Pt[s > self.cut].T

    def n_left(self, b):
        return self.U[b].shape[1]

    def n_right(self, b):
        return self.V[b].shape[1]

    def _keep(self, coef):
        return [(k, float(c)) for k, c in enumerate(coef) if abs(c) > self.cut]

    def left_block_terms(self, p):
        t = [(0, -1, 1.0)]
        t += [(-1, sn, c) for sn, c in self.one_at[p]]
        for k in np.nonzero(self.rsite == p)[0]:
            op = self.rports[k][1]
            t += [(1 + s, op, c) for s, c in self._keep(self.U[p].T @ self.M[:, k])]
        return t

    def right_block_terms(self, p, with_site=True):
        t = [(0, -1, 1.0)]
        if with_site:
            t += [(-1, sn, c) for sn, c in self.one_at[p]]
        for k in np.nonzero(self.lsite == p)[0]:
            op = self.lports[k][1]
            t += [(1 + s, op, c) for s, c in self._keep(self.M[k, :] @ self.V[p + 1])]
        return t

    def left_carry_plan(self, b):
        P, fresh = self.lcombine[b]
        return [("combine", k) for k in range(P.shape[1])] + [("fresh", a) for a in fresh]

    def right_carry_plan(self, b):
        P, fresh = self.rcombine[b]
        return [("combine", k) for k in range(P.shape[1])] + [("fresh", a) for a in fresh]

    def left_combine(self, b):
        """(P^T as a device matrix (r', r_b) or None, fresh ops): slots of EL[b+1] from EL[b]."""
        P, fresh = self.lcombine[b]
        return (self.matrix(("lc", b), P.T) if P.size else None), fresh

    def right_combine(self, b):
        """Slots of ER[b] from ER[b+1]: (P^T (r', r_(b+1)) or None, fresh ops)."""
        P, fresh = self.rcombine[b]
        return (self.matrix(("rc", b), P.T) if P.size else None), fresh

    def straddle_core(self, p):
        """Host (cl (ng x r_L), cr (ng x r_R)) with sum_g cl[g] (x) cr[g] = U_p^T M V_(p+1)."""
        hit = self._straddle.get(p)
        if hit is None:
            U, V = self.U[p], self.V[p + 1]
            if U.shape[1] == 0 or V.shape[1] == 0:
                hit = (np.zeros((0, U.shape[1])), np.zeros((0, V.shape[1])))
            else:
                A, s, Bt = np.linalg.svd(U.T @ self.M @ V, full_matrices=False)
                keep = s > self.cut
                hit = ((A[:, keep] * s[keep]).T, Bt[keep])
            self._straddle[p] = hit
        return hit

    def straddle_mats(self, p):
        """Device (cl, cr, ng) of straddle_core."""
        cl, cr = self.straddle_core(p)
        ng = cl.shape[0]
        if ng == 0:
            return None, None, 0
        return self.matrix(("scl", p), cl), self.matrix(("scr", p), cr), ng

    def straddle_groups(self, p):
        raise NotImplementedError("the compressed model provides straddle_mats")


def carried_cost(two, length):
    """(slots, groups) of the uncompressed model without building it: carried slots summed over
    all bonds and both sides, and straddling groups (min of distinct left/right operators)
    summed over all sites."""
    Ln = length
    jmax, imin = {}, {}
    for i, j, a, b, c in two:
        jmax[(i, a)] = max(jmax.get((i, a), -1), j)
        imin[(j, b)] = min(imin.get((j, b), Ln), i)
    dl = np.zeros(Ln + 2)
    for (i, a), j in jmax.items():          # open on the left at bonds i+1..j
        dl[i + 1] += 1
        dl[j + 1] -= 1
    dr = np.zeros(Ln + 2)
    for (j, b), i in imin.items():          # open on the right at bonds i+1..j
        dr[i + 1] += 1
        dr[j + 1] -= 1
    slots = float(np.sum(np.cumsum(dl)) + np.sum(np.cumsum(dr)))
    groups = 0.0
    for p in range(Ln):
        nu = sum(1 for (i, a), j in jmax.items() if i < p < j)
        nv = sum(1 for (j, b), i in imin.items() if i < p < j)
        groups += min(nu, nv)
    return slots, groups


def make_model(length, d, ops, one, two, device, compress="auto", tol=1e-14):
    """The coupling model for a run: uncompressed (one slot per open (site, op), the reference's
    bookkeeping) or CompressedModel. compress='auto' picks the compressed one when it carries at
    most 3/4 of the slots plus straddling groups."""
    if compress is False or compress is None or compress == "off" or not two:
        return Model(length, d, ops, one, two, device)
    cm = CompressedModel(length, d, ops, one, two, device, tol=tol)
    if compress is True or compress == "on":
        return cm
    if compress != "auto":
        raise ValueError("mpo_compress must be 'auto', True or False")
    slots, groups = carried_cost(two, length)
    c_slots = float(sum(cm.n_left(b) + cm.n_right(b) for b in range(length + 1)))
    c_groups = float(sum(cm.straddle_core(p)[0].shape[0] for p in range(length)))
    if c_slots + c_groups <= 0.75 * (slots + groups):
        return cm
    return Model(length, d, ops, one, two, device)


# ---------------------------------------------------------------------------
# device MPS


class DeviceMPS:
    """Open-boundary MPS on one GPU with incrementally updated environments."""

    def __init__(self, tensors, d, device, precision="fp64"):
        self.device = torch.device(device)
        if self.device.type != "cuda" and not L._host_test:
            raise RuntimeError("tnalg_gb300 runs on CUDA devices only")
        L.load()
        self.length = len(tensors)
        self.d = d
        self.mps = [torch.as_tensor(np.ascontiguousarray(t), dtype=torch.float64).to(self.device) for t in tensors]
        self.virtual_dim = np.array([1] + [int(t.shape[2]) for t in tensors])
        self.center = -1
        self.orthogonality = np.zeros(self.length)
        # True once a local solve has left a unit-norm centre; QR moves keep the norm, bond growth
        # and loaded tensors make it unknown (a random 100-site MPS centred by QR carries ~1e103).
        self.unit_norm = False
        self.precision = L.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self.ws = L.Workspace(self.device)
        self.ws2 = L.Workspace(self.device)
        self.model = None
        self.EL = [None] * (self.length + 1)
        self.ER = [None] * (self.length + 1)
        self.el_upto = -1      # EL[0..el_upto] valid
        self.er_from = self.length + 1   # ER[er_from..L] valid
        self.stats = {"matvecs": 0, "solves": 0, "restarts": 0, "unconverged": 0, "qr_mixed": 0}
        # tn_qr_mixed (FP32 cluster QR + FP64 re-orthogonalisation) for the seeding moves of the
        # tf32x3 path, and for every move while fast_gauge is set (bond growth, entanglement
        # spectrum: the state is then kept to ~1e-7); TNALG_MIXED_QR=0 keeps every move on the
        # FP64 Householder QR
        self.mixed_qr = os.environ.get("TNALG_MIXED_QR", "1") != "0"
        self.fast_gauge = False

    # -- model / environments ----------------------------------------------------
    def set_model(self, model):
        if self.model is not model:
            self.model = model
            self.EL = [None] * (self.length + 1)
            self.ER = [None] * (self.length + 1)
            self.el_upto = -1
            self.er_from = self.length + 1

    def _edge_envs(self):
        m = self.model
        if self.el_upto < 0:
            self.EL[0] = torch.zeros((1 + m.n_left(0), 1, 1), dtype=torch.float64, device=self.device)
            self.el_upto = 0
        if self.er_from > self.length:
            self.ER[self.length] = torch.zeros((1 + m.n_right(self.length), 1, 1), dtype=torch.float64,
                                               device=self.device)
            self.er_from = self.length

    def tensor_changed(self, n):
        """Environments that contracted site n become stale."""
        self.el_upto = min(self.el_upto, n)
        self.er_from = max(self.er_from, n + 1)

    def ensure_envs(self, p):
        self._edge_envs()
        while self.el_upto < p:
            self._left_update(self.el_upto)
        while self.er_from > p + 1:
            self._right_update(self.er_from - 1)

    def _left_update(self, b):
        """EL[b+1] from EL[b] and the left-canonical tensor at site b (transfer_left,
        TensorBasicModule.py:530-573, for every carried operator at once)."""
        m, A = self.model, self.mps[b]
        if m.compressed:
            return self._update_compressed(b, left=True)
        cl, d, cr = A.shape
        env = self.EL[b]
        plan = m.memo(("lcp", b), lambda: m.left_carry_plan(b))
        ns = 1 + len(plan)
        lib, st = L.load(), L.stream_handle()
        T = torch.empty((ns, cl * d * cr), dtype=torch.float64, device=self.device)
        W = torch.empty((cl * d, cl * d), dtype=torch.float64, device=self.device)
        terms, nt = m.table_lazy(("wl", b), lambda: m.left_block_terms(b))
        L.check(lib.tn_assemble_block(0, cl, d, L.ptr(env), L.ptr(m.ops), L.ptr(terms), nt, L.ptr(W), st), "assemble")
        L.gemm(W, A, T[0], cl * d, cr, cl * d, (cl * d, 1), (cr, 1), (cr, 1), precision=self.precision, ws=self.ws)
        carry = [(k, s) for k, (kind, s) in enumerate(plan) if kind == "carry"]
        fresh = [(k, a) for k, (kind, a) in enumerate(plan) if kind == "fresh"]
        if carry:
            # T[1+k] = EL[b][slot] . A(cl, d*cr); slots gathered into a contiguous stack first
            g = torch.empty((len(carry), cl, cl), dtype=torch.float64, device=self.device)
            gt, ng = m.table_lazy(("lg", b), lambda: [(s, q, 1.0) for q, (_, s) in enumerate(carry)])
            L.check(lib.tn_combine_slots(cl, L.ptr(env), L.ptr(gt), ng, len(carry), L.ptr(g), st), "gather")
            ks = [k for k, _ in carry]
            if ks == list(range(ks[0], ks[0] + len(ks))):
                L.gemm(g, A, T[1 + ks[0]], cl, d * cr, cl, (cl, 1), (d * cr, 1), (d * cr, 1), batch=len(carry),
                       bstrides=(cl * cl, 0, cl * d * cr), precision=self.precision, ws=self.ws)
            else:
                for q, (k, _) in enumerate(carry):
                    L.gemm(g[q], A, T[1 + k], cl, d * cr, cl, (cl, 1), (d * cr, 1), (d * cr, 1),
                           precision=self.precision, ws=self.ws)
        for k, a in fresh:
            oi = m.opidx(("op", a), [a])
            L.check(lib.tn_apply_site_ops(cl, d, cr, L.ptr(A), L.ptr(m.ops), L.ptr(oi), 1, L.ptr(T[1 + k]),
                                          cl * d * cr, st), "site op")
        out = torch.empty((ns, cr, cr), dtype=torch.float64, device=self.device)
        L.gemm(A, T, out, cr, cr, cl * d, (1, cr), (cr, 1), (cr, 1), batch=ns, bstrides=(0, cl * d * cr, cr * cr),
               precision=self.precision, ws=self.ws)
        self.EL[b + 1] = out
        self.el_upto = b + 1

    def _right_update(self, b):
        """ER[b] from ER[b+1] and the right-canonical tensor at site b (transfer_right,
        TensorBasicModule.py:576-619)."""
        m, B = self.model, self.mps[b]
        if m.compressed:
            return self._update_compressed(b, left=False)
        cl, d, cr = B.shape
        env = self.ER[b + 1]
        plan = m.memo(("rcp", b), lambda: m.right_carry_plan(b))
        ns = 1 + len(plan)
        lib, st = L.load(), L.stream_handle()
        T = torch.empty((ns, cl * d * cr), dtype=torch.float64, device=self.device)
        W = torch.empty((d * cr, d * cr), dtype=torch.float64, device=self.device)
        terms, nt = m.table_lazy(("wrf", b), lambda: m.right_block_terms(b, with_site=True))
        L.check(lib.tn_assemble_block(1, cr, d, L.ptr(env), L.ptr(m.ops), L.ptr(terms), nt, L.ptr(W), st), "assemble")
        # T0 = B(cl, d*cr) . W^T
        L.gemm(B, W, T[0], cl, d * cr, d * cr, (d * cr, 1), (1, d * cr), (d * cr, 1), precision=self.precision,
               ws=self.ws)
        carry = [(k, s) for k, (kind, s) in enumerate(plan) if kind == "carry"]
        fresh = [(k, a) for k, (kind, a) in enumerate(plan) if kind == "fresh"]
        if carry:
            g = torch.empty((len(carry), cr, cr), dtype=torch.float64, device=self.device)
            gt, ng = m.table_lazy(("rg", b), lambda: [(s, q, 1.0) for q, (_, s) in enumerate(carry)])
            L.check(lib.tn_combine_slots(cr, L.ptr(env), L.ptr(gt), ng, len(carry), L.ptr(g), st), "gather")
            ks = [k for k, _ in carry]
            if ks == list(range(ks[0], ks[0] + len(ks))):
                L.gemm(B, g, T[1 + ks[0]], cl * d, cr, cr, (cr, 1), (1, cr), (cr, 1), batch=len(carry),
                       bstrides=(0, cr * cr, cl * d * cr), precision=self.precision, ws=self.ws)
            else:
                for q, (k, _) in enumerate(carry):
                    L.gemm(B, g[q], T[1 + k], cl * d, cr, cr, (cr, 1), (1, cr), (cr, 1), precision=self.precision,
                           ws=self.ws)
        for k, a in fresh:
            oi = m.opidx(("op", a), [a])
            L.check(lib.tn_apply_site_ops(cl, d, cr, L.ptr(B), L.ptr(m.ops), L.ptr(oi), 1, L.ptr(T[1 + k]),
                                          cl * d * cr, st), "site op")
        out = torch.empty((ns, cl, cl), dtype=torch.float64, device=self.device)
        L.gemm(B, T, out, cl, cl, d * cr, (d * cr, 1), (1, d * cr), (cl, 1), batch=ns,
               bstrides=(0, cl * d * cr, cl * cl), precision=self.precision, ws=self.ws)
        self.ER[b] = out
        self.er_from = b

    def _update_compressed(self, b, left):
        """EL[b+1] (left) or ER[b] (right) under a CompressedModel. Slot 0 as in the plain
        update; the carried slots are first combined (P^T times the stacked carried slots of the
        previous bond, one FP64 GEMM), then carried through site b like plain slots; the ports
        of site b enter as site operators."""
        m, A = self.model, self.mps[b]
        cl, d, cr = A.shape
        lib, st = L.load(), L.stream_handle()
        if left:
            env = self.EL[b]
            Pt, fresh = m.left_combine(b)
            rb, chi = m.n_left(b), cl
        else:
            env = self.ER[b + 1]
            Pt, fresh = m.right_combine(b)
            rb, chi = m.n_right(b + 1), cr
        rp = int(Pt.shape[0]) if Pt is not None else 0
        ns = 1 + rp + len(fresh)
        T = torch.empty((ns, cl * d * cr), dtype=torch.float64, device=self.device)
        if left:
            W = torch.empty((cl * d, cl * d), dtype=torch.float64, device=self.device)
            terms, nt = m.table_lazy(("wl", b), lambda: m.left_block_terms(b))
            L.check(lib.tn_assemble_block(0, cl, d, L.ptr(env), L.ptr(m.ops), L.ptr(terms), nt, L.ptr(W), st),
                    "assemble")
            L.gemm(W, A, T[0], cl * d, cr, cl * d, (cl * d, 1), (cr, 1), (cr, 1), precision=self.precision,
                   ws=self.ws)
        else:
            W = torch.empty((d * cr, d * cr), dtype=torch.float64, device=self.device)
            terms, nt = m.table_lazy(("wrf", b), lambda: m.right_block_terms(b, with_site=True))
            L.check(lib.tn_assemble_block(1, cr, d, L.ptr(env), L.ptr(m.ops), L.ptr(terms), nt, L.ptr(W), st),
                    "assemble")
            L.gemm(A, W, T[0], cl, d * cr, d * cr, (d * cr, 1), (1, d * cr), (d * cr, 1), precision=self.precision,
                   ws=self.ws)
        if rp:
            if int(env.shape[0]) != 1 + rb:
                raise RuntimeError("environment at bond %d has %d slots, the model %d" % (b, env.shape[0], 1 + rb))
            g = torch.empty((rp, chi, chi), dtype=torch.float64, device=self.device)
            L.gemm(Pt, env[1:], g, rp, chi * chi, rb, (rb, 1), (chi * chi, 1), (chi * chi, 1), ws=self.ws)
            if left:   # T[1+k] = g[k] . A(cl, d*cr)
                L.gemm(g, A, T[1], cl, d * cr, cl, (cl, 1), (d * cr, 1), (d * cr, 1), batch=rp,
                       bstrides=(cl * cl, 0, cl * d * cr), precision=self.precision, ws=self.ws)
            else:      # T[1+k] = A(cl*d, cr) . g[k]^T
                L.gemm(A, g, T[1], cl * d, cr, cr, (cr, 1), (1, cr), (cr, 1), batch=rp,
                       bstrides=(0, cr * cr, cl * d * cr), precision=self.precision, ws=self.ws)
        for q, a in enumerate(fresh):
            oi = m.opidx(("op", a), [a])
            L.check(lib.tn_apply_site_ops(cl, d, cr, L.ptr(A), L.ptr(m.ops), L.ptr(oi), 1, L.ptr(T[1 + rp + q]),
                                          cl * d * cr, st), "site op")
        if left:
            out = torch.empty((ns, cr, cr), dtype=torch.float64, device=self.device)
            L.gemm(A, T, out, cr, cr, cl * d, (1, cr), (cr, 1), (cr, 1), batch=ns,
                   bstrides=(0, cl * d * cr, cr * cr), precision=self.precision, ws=self.ws)
            self.EL[b + 1] = out
            self.el_upto = b + 1
        else:
            out = torch.empty((ns, cl, cl), dtype=torch.float64, device=self.device)
            L.gemm(A, T, out, cl, cl, d * cr, (d * cr, 1), (1, d * cr), (cl, 1), batch=ns,
                   bstrides=(0, cl * d * cr, cl * cl), precision=self.precision, ws=self.ws)
            self.ER[b] = out
            self.er_from = b

    # -- gauge -------------------------------------------------------------------
    def _qr(self, mm, nn, A, sA, Q, sQ, R, seed_only, exact=False):
        """tn_qr, or tn_qr_mixed on the mixed-precision path for a seeding move (R only seeds the
        next local solve) or while fast_gauge is set; Q stays orthonormal to ~1e-12 either way.
        exact: always tn_qr (a Q whose span must equal col(A) to FP64 accuracy)."""
        lib, st = L.load(), L.stream_handle()
        if (not exact and self.mixed_qr and (seed_only or self.fast_gauge) and self.precision == L.PREC_TF32X3
                and min(mm, nn) >= 64):
            self.stats["qr_mixed"] += 1
            wp, wb = self.ws2.args(lib.tn_qr_mixed_workspace_bytes(mm, nn))
            L.check(lib.tn_qr_mixed(mm, nn, L.ptr(A), sA[0], sA[1], L.ptr(Q), sQ[0], sQ[1], L.ptr(R), nn, 1, wp, wb,
                                    st), "qr_mixed")
        else:
            wp, wb = self.ws2.args(lib.tn_qr_workspace_bytes(mm, nn))
            L.check(lib.tn_qr(mm, nn, L.ptr(A), sA[0], sA[1], L.ptr(Q), sQ[0], sQ[1], L.ptr(R), nn, 1, wp, wb, st),
                    "qr")

    def _seed_precision(self, seed_only):
        """Precision of the R-absorb of a gauge move. seed_only: the receiving site is re-solved
        next, so its tensor is only the Lanczos start vector and may use the working precision,
        provided the state has unit norm (split TF32 keeps FP32's exponent range, |x| < 3.4e38).
        Otherwise the absorbed tensor carries the state and stays FP64."""
        if seed_only and self.unit_norm:
            return self.precision
        return L.PREC_FP64

    def qr_left(self, n, seed_only=False):
        """left2right_decompose_tensor + absorb_matrix2tensor(mps[n+1], R^T, 0)
        (TensorBasicModule.py:314-348, 387-424; MPSClass.py:150-158)."""
        A = self.mps[n]
        cl, d, cr = A.shape
        mm, nn = cl * d, cr
        k = min(mm, nn)
        lib, st = L.load(), L.stream_handle()
        Q = torch.empty((cl, d, k), dtype=torch.float64, device=self.device)
        R = torch.empty((k, nn), dtype=torch.float64, device=self.device)
        self._qr(mm, nn, A, (nn, 1), Q, (k, 1), R, seed_only)
        nxt = self.mps[n + 1]
        c2, d2, r2 = nxt.shape
        new = torch.empty((k, d2, r2), dtype=torch.float64, device=self.device)
        L.gemm(R, nxt, new, k, d2 * r2, nn, (nn, 1), (d2 * r2, 1), (d2 * r2, 1), ws=self.ws,
               precision=self._seed_precision(seed_only))
        self.mps[n] = Q
        self.mps[n + 1] = new
        self._last_r = R
        self.virtual_dim[n + 1] = k
        self.tensor_changed(n)
        self.tensor_changed(n + 1)

    def qr_right(self, n, seed_only=False):
        """right2left_decompose_tensor + absorb_matrix2tensor(mps[n-1], R^T, 2)
        (TensorBasicModule.py:351-384; MPSClass.py:159-167)."""
        A = self.mps[n]
        cl, d, cr = A.shape
        mm, nn = d * cr, cl  # QR of A(cl, d*cr)^T
        k = min(mm, nn)
        lib, st = L.load(), L.stream_handle()
        Bt = torch.empty((k, d, cr), dtype=torch.float64, device=self.device)
        R = torch.empty((k, nn), dtype=torch.float64, device=self.device)
        # a(i, j) = A[j, i]: sAm = 1, sAn = d*cr ; Q(i, j) -> Bt[j, i]: sQm = 1, sQn = d*cr
        self._qr(mm, nn, A, (1, d * cr), Bt, (1, d * cr), R, seed_only)
        prv = self.mps[n - 1]
        c0, d0, r0 = prv.shape
        new = torch.empty((c0, d0, k), dtype=torch.float64, device=self.device)
        # prv(c0*d0, cl) . R^T(cl, k)
        L.gemm(prv, R, new, c0 * d0, k, nn, (nn, 1), (1, nn), (k, 1), ws=self.ws,
               precision=self._seed_precision(seed_only))
        self.mps[n] = Bt
        self.mps[n - 1] = new
        self._last_r = R
        self.virtual_dim[n] = k
        self.tensor_changed(n)
        self.tensor_changed(n - 1)

    def orthogonalize_mps(self, l0, l1):
        """MPSClass.py:143-167 with QR."""
        if l0 < l1:
            for n in range(l0, l1):
                self.qr_left(n)
            self.orthogonality[l0:l1] = -1
            self.orthogonality[l1] = 0
        elif l0 > l1:
            for n in range(l0, l1, -1):
                self.qr_right(n)
            self.orthogonality[l1 + 1:l0 + 1] = 1
            self.orthogonality[l1] = 0

    def grow_bonds(self, chi_new, noise=1e-3, seed=0):
        """Enlarge every bond to min(chi_new, d^b, d^(L-b)); the new entries are seeded
        Gaussian noise of scale `noise`, the old tensor is kept in the leading block.
        The MPS loses its canonical form (centre -1); the caller re-centres it. The reference
        keeps chi fixed (TensorBasicModule.py:314-384); this is the bond ramp of a chi schedule."""
        Ln, d = self.length, self.d
        cap = [1] + [min(chi_new, d ** min(b, 60), d ** min(Ln - b, 60)) for b in range(1, Ln)] + [1]
        dims = [max(int(c), int(v)) for c, v in zip(cap, self.virtual_dim)]
        if dims == [int(v) for v in self.virtual_dim]:
            return False
        g = torch.Generator(device=self.device)
        g.manual_seed(int(seed))
        for n in range(Ln):
            t = self.mps[n]
            cl, dd, cr = t.shape
            ncl, ncr = dims[n], dims[n + 1]
            if (ncl, ncr) != (cl, cr):
                new = noise * torch.randn((ncl, dd, ncr), generator=g, dtype=torch.float64, device=self.device)
                new[:cl, :, :cr] = t
                self.mps[n] = new
        self.virtual_dim = np.array(dims)
        self.center = -1
        self.unit_norm = False
        self.orthogonality[:] = 0
        self.el_upto = min(self.el_upto, 0)
        self.er_from = max(self.er_from, self.length)
        return True

    def expand_bonds(self, chi_new, seed=0, oversample=8):
        """Grow every bond to min(chi_new, d^b, d^(L-b)) by subspace expansion and truncated SVD, in
        one left-to-right pass of gauge moves: at bond (b, b+1), with the centre at b, the new bond
        directions are the dominant left singular vectors of P_perp = (1 - Q Q^T) P, where Q spans
        the centre tensor psi (its QR gauge move) and P = [T_0 | T_1 | ...] are the channels of the
        Hamiltonian left of the bond applied to psi (T_0 = W_L psi with the block operator of site
        b, T_k = the k-th operator left open at bond b+1 times psi: the products of an environment
        update). P_perp is sketched by a seeded Gaussian matrix (chi_new - chi_b + oversample
        columns, a randomised range finder), and its sketch is truncated by tn_svd_jacobi. The
        site right of the bond receives zero rows for the new directions, so the state is
        unchanged; the local solves of the next sweep then use the enlarged bond spaces. The
        reference keeps chi fixed (TensorBasicModule.py:314-384); this is the bond ramp of a chi
        schedule, and replaces growth by random noise. Returns True if a bond grew."""
        Ln, d = self.length, self.d
        cap = [1] + [min(chi_new, d ** min(b, 60), d ** min(Ln - b, 60)) for b in range(1, Ln)] + [1]
        if all(int(c) <= int(v) for c, v in zip(cap, self.virtual_dim)):
            return False
        m = self.model
        if m is None or m.compressed:
            raise RuntimeError("expand_bonds needs the uncompressed coupling model of the run")
        lib = L.load()
        rng = np.random.default_rng(int(seed))
        self.correct_orthogonal_center(0)
        grew = False
        for b in range(Ln - 1):
            target = int(cap[b + 1])
            A = self.mps[b]
            cl, dd, cr = (int(x) for x in A.shape)
            if target <= cr:
                self.qr_left(b)
                self.orthogonality[b] = -1
                self.center = b + 1
                continue
            grew = True
            self.ensure_envs(b)
            mm = cl * dd
            extra = min(target, mm) - min(mm, cr)
            # the open channels at bond b+1 applied to psi: T[j] (mm x cr)
            plan = m.memo(("lcp", b), lambda: m.left_carry_plan(b))
            ns = 1 + len(plan)
            T = torch.empty((ns, mm * cr), dtype=torch.float64, device=self.device)
            W = torch.empty((mm, mm), dtype=torch.float64, device=self.device)
            terms, nt = m.table_lazy(("wl", b), lambda: m.left_block_terms(b))
            st = L.stream_handle()
            L.check(lib.tn_assemble_block(0, cl, dd, L.ptr(self.EL[b]), L.ptr(m.ops), L.ptr(terms), nt, L.ptr(W), st),
                    "assemble")
            # the channels only choose directions: the working precision is enough
            prec = self.precision if self.unit_norm else L.PREC_FP64
            L.gemm(W, A, T[0], mm, cr, mm, (mm, 1), (cr, 1), (cr, 1), ws=self.ws, precision=prec)
            for j, (kind, x) in enumerate(plan):
                if kind == "carry":
                    L.gemm(self.EL[b][x], A, T[1 + j], cl, dd * cr, cl, (cl, 1), (dd * cr, 1), (dd * cr, 1), ws=self.ws,
                           precision=prec)
                else:
                    oi = m.opidx(("op", x), [x])
                    L.check(lib.tn_apply_site_ops(cl, dd, cr, L.ptr(A), L.ptr(m.ops), L.ptr(oi), 1, L.ptr(T[1 + j]),
                                                  mm * cr, st), "site op")
            # Q R = psi (the plain gauge move), then the sketch Y = sum_j T_j G_j projected off range(Q)
            k = min(mm, cr)
            Q = torch.empty((mm, k), dtype=torch.float64, device=self.device)
            R = torch.empty((k, cr), dtype=torch.float64, device=self.device)
            self._qr(mm, cr, A, (cr, 1), Q, (k, 1), R, False)
            s = min(extra + oversample, mm - k)
            G = torch.tensor(rng.standard_normal((ns * cr, s)), dtype=torch.float64, device=self.device)
            Y = torch.empty((mm, s), dtype=torch.float64, device=self.device)
            L.gemm(T, G, Y, mm, s, cr, (cr, 1), (s, 1), (s, 1), nred=ns, rstrides=(mm * cr, cr * s), ws=self.ws,
                   precision=prec)
            QtY = torch.empty((k, s), dtype=torch.float64, device=self.device)
            L.gemm(Q, Y, QtY, k, s, mm, (1, k), (s, 1), (s, 1), ws=self.ws)
            L.gemm(Q, QtY, Y, mm, s, k, (k, 1), (s, 1), (s, 1), Cin=Y, alpha=-1.0, beta=1.0, ws=self.ws)
            # truncated SVD of the sketch: its dominant left singular vectors (rows of Vt of Y^T). The
            # directions only need ranking, and they are projected and re-orthonormalised in FP64
            # below, so the Jacobi stops once the rows are orthogonal to 1e-7 (the singular values
            # are then accurate to ~1e-14 relative) or after 6 sweeps (a sketch with more columns
            # than independent channels keeps a few noise rows rotating; the oversampled sketch only
            # drops its 8 weakest directions, and their ranking is settled long before)
            Ut, sv, Vt = L.svd_truncated(Y.t(), extra, ws=self.ws2, tol=1e-7, max_sweeps=6)
            r = int(Vt.shape[0])
            Vn = torch.empty((mm, r), dtype=torch.float64, device=self.device)
            Vn.copy_(Vt.t())
            # one more projection off range(Q) and an orthonormal basis of what is left
            QtV = torch.empty((k, r), dtype=torch.float64, device=self.device)
            L.gemm(Q, Vn, QtV, k, r, mm, (1, k), (r, 1), (r, 1), ws=self.ws)
            L.gemm(Q, QtV, Vn, mm, r, k, (k, 1), (r, 1), (r, 1), Cin=Vn, alpha=-1.0, beta=1.0, ws=self.ws)
            Vq = torch.empty((mm, r), dtype=torch.float64, device=self.device)
            Rv = torch.empty((r, r), dtype=torch.float64, device=self.device)
            # FP64: the new directions must stay orthogonal to range(Q) to FP64 accuracy
            self._qr(mm, r, Vn, (r, 1), Vq, (r, 1), Rv, False, exact=True)
            newk = k + r
            Anew = torch.empty((cl, dd, newk), dtype=torch.float64, device=self.device)
            Anew.view(mm, newk)[:, :k].copy_(Q)
            Anew.view(mm, newk)[:, k:].copy_(Vq)
            nxt = self.mps[b + 1]
            c2, d2, r2 = (int(x) for x in nxt.shape)
            new_next = torch.zeros((newk, d2, r2), dtype=torch.float64, device=self.device)
            L.gemm(R, nxt, new_next, k, d2 * r2, cr, (cr, 1), (d2 * r2, 1), (d2 * r2, 1), ws=self.ws)
            self.mps[b] = Anew
            self.mps[b + 1] = new_next
            self.virtual_dim[b + 1] = newk
            self.orthogonality[b] = -1
            self.center = b + 1
            self.tensor_changed(b)
            self.tensor_changed(b + 1)
        self.orthogonality[Ln - 1] = 0
        self.center = Ln - 1
        return grew

    def move_center_for_solve(self, p):
        """Centre to p ahead of a local solve at p: a one-site move seeds site p in the working
        precision (the solve replaces it); longer moves go through correct_orthogonal_center."""
        if self.center == p - 1 and p >= 1:
            self.qr_left(p - 1, seed_only=True)
            self.orthogonality[p - 1] = -1
            self.orthogonality[p] = 0
            self.center = p
        elif self.center == p + 1:
            self.qr_right(p + 1, seed_only=True)
            self.orthogonality[p + 1] = 1
            self.orthogonality[p] = 0
            self.center = p
        else:
            self.correct_orthogonal_center(p)

    def correct_orthogonal_center(self, p):
        """MPSClass.py:188-198 for an explicit p."""
        if self.center < 0:
            self.orthogonalize_mps(0, p)
            self.orthogonalize_mps(self.length - 1, p)
        elif self.center != p:
            self.orthogonalize_mps(self.center, p)
        self.center = p

    # -- local solve ---------------------------------------------------------------
    def site_operator(self, p):
        """Assemble the effective Hamiltonian of site p; returns (desc, keep-alive tensors)."""
        m = self.model
        self.ensure_envs(p)
        cl, d, cr = self.mps[p].shape
        lib, st = L.load(), L.stream_handle()
        el, er = self.EL[p], self.ER[p + 1]
        wl = torch.empty((cl * d, cl * d), dtype=torch.float64, device=self.device)
        wr = torch.empty((d * cr, d * cr), dtype=torch.float64, device=self.device)
        t, nt = m.table_lazy(("wl", p), lambda: m.left_block_terms(p))
        L.check(lib.tn_assemble_block(0, cl, d, L.ptr(el), L.ptr(m.ops), L.ptr(t), nt, L.ptr(wl), st), "assemble")
        t, nt = m.table_lazy(("wr", p), lambda: m.right_block_terms(p, with_site=False))
        L.check(lib.tn_assemble_block(1, cr, d, L.ptr(er), L.ptr(m.ops), L.ptr(t), nt, L.ptr(wr), st), "assemble")
        keep = [wl, wr]
        sl = sr = None
        if m.compressed:
            # SL = cL . (stacked carried slots of EL[p]), SR = cR . (those of ER[p+1]): one GEMM each
            cL, cR, ng = m.straddle_mats(p)
            if ng:
                rl, rr = m.n_left(p), m.n_right(p + 1)
                sl = torch.empty((ng, cl, cl), dtype=torch.float64, device=self.device)
                sr = torch.empty((ng, cr, cr), dtype=torch.float64, device=self.device)
                L.gemm(cL, el[1:], sl, ng, cl * cl, rl, (rl, 1), (cl * cl, 1), (cl * cl, 1), ws=self.ws)
                L.gemm(cR, er[1:], sr, ng, cr * cr, rr, (rr, 1), (cr * cr, 1), (cr * cr, 1), ws=self.ws)
                keep += [sl, sr]
        else:
            slt, srt, ng = m.memo(("sg", p), lambda: m.straddle_groups(p))
        if ng and not m.compressed:
            sl = torch.empty((ng, cl, cl), dtype=torch.float64, device=self.device)
            sr = torch.empty((ng, cr, cr), dtype=torch.float64, device=self.device)
            a, na = m.table(("sl", p), slt)
            b, nb = m.table(("sr", p), srt)
            L.check(lib.tn_combine_slots(cl, L.ptr(el), L.ptr(a), na, ng, L.ptr(sl), st), "straddle")
            L.check(lib.tn_combine_slots(cr, L.ptr(er), L.ptr(b), nb, ng, L.ptr(sr), st), "straddle")
            keep += [sl, sr]
        desc = L.SiteDesc(cl, d, cr, wl.data_ptr(), wr.data_ptr(), ng, sl.data_ptr() if ng else None,
                          sr.data_ptr() if ng else None)
        return desc, keep

    def solve(self, p, eigs_tol, tau, *, tol_cap=0.0, max_krylov=40, max_restarts=50, check_every=3,
              refine=None, mixed_floor=2e-6, refine_cycles=4):
        """Lowest eigenvector of H_eff at the centre p (MPSClass.py:778-809). refine: 0 none,
        1 FP64 Rayleigh quotient of the final vector, 2 the vector refined to the FP64 tolerance
        (split-TF32 path); None = 1 on the split-TF32 path, 0 on FP64."""
        desc, keep = self.site_operator(p)
        psi = self.mps[p].contiguous()
        opts = L.LanczosOpts(float(eigs_tol), float(tau), float(tol_cap), float(mixed_floor), int(max_krylov),
                             int(max_restarts), int(check_every), int(self.precision),
                             int(self.precision != L.PREC_FP64 if refine is None else refine), int(refine_cycles))
        lib = L.load()
        need = lib.tn_lanczos_workspace_bytes(ctypes_ref(desc), ctypes_ref(opts))
        wp, wb = self.ws.args(need)
        res = L.LanczosResult()
        status = lib.tn_lanczos(ctypes_ref(desc), L.ptr(psi), ctypes_ref(opts), wp, wb, ctypes_ref(res),
                                L.stream_handle())
        if status not in (L.TN_OK, L.TN_ERR_NOCONV):
            L.check(status, "lanczos")
        self.stats["solves"] += 1
        self.stats["matvecs"] += res.matvecs
        self.stats["restarts"] += res.restarts
        if status == L.TN_ERR_NOCONV:
            self.stats["unconverged"] += 1
        self.mps[p] = psi
        self.unit_norm = True  # the solver returns a unit vector
        self.tensor_changed(p)
        del keep
        return res

    def apply_heff(self, p, psi, alpha=1.0, beta=0.0, precision=None):
        """y = beta*psi + alpha*H_eff psi at site p (tn_matvec)."""
        desc, keep = self.site_operator(p)
        y = torch.empty_like(psi)
        prec = self.precision if precision is None else precision
        lib = L.load()
        wp, wb = self.ws.args(lib.tn_matvec_workspace_bytes(ctypes_ref(desc), prec))
        L.check(lib.tn_matvec(ctypes_ref(desc), L.ptr(psi), L.ptr(y), float(alpha), float(beta), prec, wp, wb,
                              L.stream_handle()), "matvec")
        del keep
        return y

    def numpy_tensors(self):
        return [t.detach().cpu().numpy() for t in self.mps]


def ctypes_ref(obj):
    import ctypes
    return ctypes.byref(obj)


# ---------------------------------------------------------------------------
# observables (observation_s1 / observation_s1_s2, MPSClass.py:857-909)


class _Observer:
    """Expectation values of products of one-site operators on a canonical MPS.

    For a centre c, sites < c are left-canonical and sites > c right-canonical, so a
    product of operators on sites i <= j is contracted only over [min(i, c), max(j, c)]
    with identity boundaries. Terms with j >= c are contracted left-to-right from an
    identity (or the shared chain E_q for q > c); terms with j < c right-to-left.
    Operator chains that share their first site and operator are contracted once.
    """

    def __init__(self, mps, precision=L.PREC_FP64):
        self.s = mps
        self.dev = mps.device
        self.c = mps.center
        self.E = {}
        self.F = {}
        self.lib = L.load()
        self.st = L.stream_handle()
        # transfer products in FP64, or split TF32 for long operator strings of the mixed path
        self.prec = int(precision)
        self.ws = mps.ws if self.prec != L.PREC_FP64 else None

    # transfer helpers -------------------------------------------------------------
    def _op_apply(self, X, shape, op):
        cl, d, cr = shape
        out = torch.empty_like(X)
        oi = self.s.model.opidx(("op", op), [op])
        L.check(self.lib.tn_apply_site_ops(cl, d, cr, L.ptr(X), L.ptr(self.s.model.ops), L.ptr(oi), 1, L.ptr(out),
                                           cl * d * cr, self.st), "site op")
        return out

    def left_x(self, M, V):
        """X = V . M(cl, d*cr) (V None = identity)."""
        if V is None:
            return M
        cl, d, cr = M.shape
        X = torch.empty_like(M)
        L.gemm(V, M, X, cl, d * cr, cl, (cl, 1), (d * cr, 1), (d * cr, 1), precision=self.prec, ws=self.ws)
        return X

    def left_close(self, M, X):
        """V' = M(cl*d, cr)^T . X(cl*d, cr)."""
        cl, d, cr = M.shape
        out = torch.empty((cr, cr), dtype=torch.float64, device=self.dev)
        L.gemm(M, X, out, cr, cr, cl * d, (1, cr), (cr, 1), (cr, 1), precision=self.prec, ws=self.ws)
        return out

    def tl(self, M, V, op=None):
        X = self.left_x(M, V)
        if op is not None:
            X = self._op_apply(X, M.shape, op)
        return self.left_close(M, X)

    def right_x(self, M, V):
        """X = M(cl*d, cr) . V^T (V None = identity)."""
        if V is None:
            return M
        cl, d, cr = M.shape
        X = torch.empty_like(M)
        L.gemm(M, V, X, cl * d, cr, cr, (cr, 1), (1, cr), (cr, 1), precision=self.prec, ws=self.ws)
        return X

    def right_close(self, M, X):
        """V'[a', a] = sum M[a', (s b)] X[a, (s b)]."""
        cl, d, cr = M.shape
        out = torch.empty((cl, cl), dtype=torch.float64, device=self.dev)
        L.gemm(M, X, out, cl, cl, d * cr, (d * cr, 1), (1, d * cr), (cl, 1), precision=self.prec, ws=self.ws)
        return out

    def tr(self, M, V, op=None):
        X = self.right_x(M, V)
        if op is not None:
            X = self._op_apply(X, M.shape, op)
        return self.right_close(M, X)

    def E_at(self, q):
        """Left environment (identity operators) at bond q; None means identity (q <= c)."""
        if q <= self.c:
            return None
        if q not in self.E:
            self.E[q] = self.tl(self.s.mps[q - 1], self.E_at(q - 1))
        return self.E[q]

    def F_at(self, q):
        """Right environment at bond q; None means identity (q > c)."""
        if q > self.c:
            return None
        if q not in self.F:
            self.F[q] = self.tr(self.s.mps[q], self.F_at(q + 1))
        return self.F[q]

    def density(self, M, X, out):
        cl, d, cr = M.shape
        L.check(self.lib.tn_pair_contract(cl, d, cr, L.ptr(M), L.ptr(X), 1.0, L.ptr(out), self.st), "pair")

    def site_densities(self, sites):
        """g[k][x, y] = <E_xy(sites[k])>, E_xy = |x><y| (unnormalised one-site densities), as numpy."""
        s, d = self.s, self.s.d
        G = torch.zeros((max(len(sites), 1), d, d), dtype=torch.float64, device=self.dev)
        for k, q in enumerate(sites):
            M = s.mps[q]
            X = self.left_x(M, self.E_at(q)) if q >= self.c else self.right_x(M, self.F_at(q + 1))
            self.density(M, X, G[k])
        return G.cpu().numpy()[: len(sites)]

    def two_site_density(self, p1, p2):
        """rho[(x1 x2), (y1 y2)] = <E_x1y1(p1) E_x2y2(p2)> for p1 < p2, E_xy = |x><y| (unnormalised):
        the d^2 elementary operators are applied at one end in one tn_apply_site_ops call, each is
        carried to the other end and closed with the local density there. Toward the centre side
        that is not canonical, as the one- and two-body queries do."""
        s, d = self.s, self.s.d
        nk = d * d
        elem = np.zeros((nk, d, d))
        for x in range(d):
            for y in range(d):
                elem[x * d + y, x, y] = 1.0
        elem = torch.tensor(elem, dtype=torch.float64, device=self.dev)
        oi = torch.arange(nk, dtype=torch.int32, device=self.dev)
        G = torch.zeros((nk, d, d), dtype=torch.float64, device=self.dev)
        fwd = p2 >= self.c
        q = p1 if fwd else p2
        M = s.mps[q]
        cl, _, cr = M.shape
        X = self.left_x(M, self.E_at(q)) if fwd else self.right_x(M, self.F_at(q + 1))
        Xk = torch.empty((nk, cl, d, cr), dtype=torch.float64, device=self.dev)
        L.check(self.lib.tn_apply_site_ops(cl, d, cr, L.ptr(X), L.ptr(elem), L.ptr(oi), nk, L.ptr(Xk), cl * d * cr,
                                           self.st), "site op")
        for k in range(nk):
            if fwd:
                V = self.left_close(M, Xk[k])
                for r in range(p1 + 1, p2):
                    V = self.tl(s.mps[r], V)
                M2 = s.mps[p2]
                self.density(M2, self.left_x(M2, V), G[k])
            else:
                V = self.right_close(M, Xk[k])
                for r in range(p2 - 1, p1, -1):
                    V = self.tr(s.mps[r], V)
                M1 = s.mps[p1]
                self.density(M1, self.right_x(M1, V), G[k])
        g = G.cpu().numpy().reshape(d, d, d, d)   # [k = (x, y) at the start site][x', y' at the end site]
        rho = g.transpose(0, 2, 1, 3) if fwd else g.transpose(2, 0, 3, 1)
        return rho.reshape(nk, nk)

    # queries ------------------------------------------------------------------------
    def run(self, one, two):
        """one: [(q, op)], two: [(i, j, a, b)] with i != j. Returns (vals_one, vals_two)."""
        s = self.s
        d = s.d
        G1 = torch.zeros((max(len(one), 1), d, d), dtype=torch.float64, device=self.dev)
        G2 = torch.zeros((max(len(two), 1), d, d), dtype=torch.float64, device=self.dev)
        # one-body: local density at q
        dens = {}
        for k, (q, op) in enumerate(one):
            if q not in dens:
                M = s.mps[q]
                X = self.left_x(M, self.E_at(q)) if q >= self.c else self.right_x(M, self.F_at(q + 1))
                dens[q] = (M, X)
            M, X = dens[q]
            self.density(M, X, G1[k])
        # two-body, grouped by the first operator of the contraction direction
        fwd, bwd = {}, {}
        closing = []
        for k, (i, j, a, b) in enumerate(two):
            if i > j:
                i, j, a, b = j, i, b, a
            if j >= self.c:
                fwd.setdefault((i, a), []).append((j, b, k))
                closing.append(b)
            else:
                bwd.setdefault((j, b), []).append((i, a, k))
                closing.append(a)
        for (i, a), lst in fwd.items():
            lst.sort()
            V = self.tl(s.mps[i], self.E_at(i), a)
            pos = i + 1
            for j, b, k in lst:
                while pos < j:
                    V = self.tl(s.mps[pos], V)
                    pos += 1
                M = s.mps[j]
                self.density(M, self.left_x(M, V), G2[k])
        for (j, b), lst in bwd.items():
            lst.sort(reverse=True)
            V = self.tr(s.mps[j], self.F_at(j + 1), b)
            pos = j - 1
            for i, a, k in lst:
                while pos > i:
                    V = self.tr(s.mps[pos], V)
                    pos -= 1
                M = s.mps[i]
                self.density(M, self.right_x(M, V), G2[k])
        g1 = G1.cpu().numpy()
        g2 = G2.cpu().numpy()
        ops = s.model.ops_np
        v1 = np.array([np.sum(ops[op] * g1[k]) for k, (q, op) in enumerate(one)])
        v2 = np.array([np.sum(ops[closing[k]] * g2[k]) for k in range(len(two))])
        return v1, v2


def observe(mps, one, two, precision=L.PREC_FP64):
    """Device expectation values; see _Observer. precision applies to the transfer products."""
    if mps.center < 0:
        raise RuntimeError("observables need a central-orthogonal MPS (call correct_orthogonal_center first)")
    return _Observer(mps, precision).run(one, two)
