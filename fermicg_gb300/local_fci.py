"""Local (per-cluster) determinant space, FCI bases and transition densities.

This is the host-side restatement of what FermiCG delegates to
ActiveSpaceSolvers (not vendored with the reference; pinned in its
Manifest.toml as ActiveSpaceSolvers 0.1.0, git-tree 5bcc3a9d):
  * FCIAnsatz / build_H_matrix / eigen per Fock sector
      (build_local_quantities.jl:1090-1180, compute_cluster_eigenbasis)
  * compute_operator_{c_a,c_b,cc_aa,cc_bb,ca_aa,ca_bb,ca_ab,cc_ab,cca_aaa,
    cca_bbb,cca_aba,cca_abb} (build_local_quantities.jl:203-607)
  * the op-string table, adjoints and (orbital-multi-index, I, J) reshape of
    compute_cluster_ops (build_local_quantities.jl:40-191).

Conventions (own, self-consistent; verified by full-space TPS = FCI):
  * a local determinant is  prod_{p in alpha, increasing} a+_{p,a}
    prod_{q in beta, increasing} a+_{q,b} |0>;  spin-orbital order is all
    alpha orbitals, then all beta orbitals.
  * determinant index = ia * n_beta_strings + ib, strings in lexical order.
  * an op string such as "ABa" means p+_alpha q+_beta r_alpha with orbital
    indices (p, q, r) in that order; its TDM  G[(p,q,r), I, J] = <I|op|J>
    flattens (p,q,r) with p fastest (Julia column-major), exactly as the
    reference reshapes at build_local_quantities.jl:176-188.
Storage of a TDM block here: numpy array of shape (M_ket, M_bra, n_orbidx),
i.e. the bytes of the reference's column-major (n_orbidx, M_bra, M_ket).
"""
from __future__ import annotations

from itertools import combinations

import numpy as np

from .integrals import InCoreInts, subset

# letter -> (is_creation, spin)  spin 0 = alpha, 1 = beta
_LETTER = {"A": (True, 0), "a": (False, 0), "B": (True, 1), "b": (False, 1)}

# every op string that appears in a ClusteredTerm after the renames of
# type_ClusteredOperator.jl:275-315,446-472 (see terms.py)
OP_STRINGS = [
    "A", "a", "B", "b",
    "AA", "aa", "BB", "bb", "Aa", "Bb", "Ab", "Ba", "AB", "ab",
    "AAa", "Aaa", "BBb", "Bbb", "ABa", "Aba", "ABb", "Bba",
]
OP_ID = {s: i for i, s in enumerate(OP_STRINGS)}
OP_H = len(OP_STRINGS)        # local Hamiltonian "H"
OP_HCMF = len(OP_STRINGS) + 1  # embedded local Hamiltonian "Hcmf"
N_OPS = len(OP_STRINGS) + 2


def op_delta(op: str):
    """Change of (n_alpha, n_beta) an op string makes on its cluster."""
    da = db = 0
    for ch in op:
        cre, spin = _LETTER[ch]
        d = 1 if cre else -1
        if spin == 0:
            da += d
        else:
            db += d
    return da, db


def _popcount_table(nbits):
    t = np.zeros(1 << nbits, dtype=np.int64)
    for i in range(1, 1 << nbits):
        t[i] = t[i >> 1] + (i & 1)
    return t


class LocalSpace:
    """Determinant strings of one cluster of `n` orbitals, all sectors."""

    def __init__(self, n: int):
        self.n = n
        self.pop = _popcount_table(2 * n)
        self.strings = [[sum(1 << p for p in c) for c in combinations(range(n), k)] for k in range(n + 1)]
        self.str_index = [dict((s, i) for i, s in enumerate(sl)) for sl in self.strings]
        self._ladder = {}

    def dim(self, na, nb):
        if na < 0 or nb < 0 or na > self.n or nb > self.n:
            return 0
        return len(self.strings[na]) * len(self.strings[nb])

    def dets(self, na, nb):
        """occupation words (alpha bits low, beta bits high) of sector dets"""
        a = np.array(self.strings[na], dtype=np.int64)
        b = np.array(self.strings[nb], dtype=np.int64)
        return (a[:, None] | (b[None, :] << self.n)).reshape(-1)

    def ladder(self, cre: bool, spin: int, na: int, nb: int):
        """Matrices (n, dim_target, dim_source) of a+_p / a_p (spin) on sector (na, nb)."""
        key = (cre, spin, na, nb)
        if key in self._ladder:
            return self._ladder[key]
        n = self.n
        d = 1 if cre else -1
        ta, tb = (na + d, nb) if spin == 0 else (na, nb + d)
        dim_t = self.dim(ta, tb)
        occ = self.dets(na, nb)
        out = np.zeros((n, dim_t, occ.size))
        if dim_t > 0:
            nbs_t = len(self.strings[tb])
            for p in range(n):
                so = p + spin * n
                bit = (occ >> so) & 1
                ok = bit == 0 if cre else bit == 1
                sign = 1.0 - 2.0 * (self.pop[occ & ((1 << so) - 1)] & 1)
                new = occ ^ (1 << so)
                cols = np.nonzero(ok)[0]
                for j in cols:
                    w = int(new[j])
                    ia = self.str_index[ta][w & ((1 << n) - 1)]
                    ib = self.str_index[tb][w >> n]
                    out[p, ia * nbs_t + ib, j] = sign[j]
        self._ladder[key] = out
        return out

    def op_matrices(self, op: str, na: int, nb: int):
        """Dense matrices of op string `op` acting on sector (na, nb).

        Returns (target_sector, array of shape (n,)*k + (dim_t, dim_s)) or None.
        Operators act right to left: the last letter is applied first.
        """
        cur = (na, nb)
        mats = []
        for ch in reversed(op):
            cre, spin = _LETTER[ch]
            if self.dim(*cur) == 0:
                return None
            m = self.ladder(cre, spin, *cur)
            d = 1 if cre else -1
            cur = (cur[0] + d, cur[1]) if spin == 0 else (cur[0], cur[1] + d)
            if self.dim(*cur) == 0:
                return None
            mats.append(m)
        # mats[0] is the rightmost operator; build prod = M_first_letter ... M_last_letter
        k = len(mats)
        res = mats[0]  # (n, t1, s)  index of last letter
        for i in range(1, k):
            # new operator to the left: (n, t2, t1) @ (..., t1, s)
            res = np.einsum("aij,...jk->a...ik", mats[i], res, optimize=True)
        # res axes: (letter_1, letter_2, ..., letter_k, dim_t, dim_s) because each new
        # (more-left) letter was prepended
        return cur, res

    def one_body_E(self, na, nb):
        """Spin-summed E_pq = sum_s p+_s q_s on sector (na, nb): (n, n, dim, dim)."""
        n = self.n
        dim = self.dim(na, nb)
        E = np.zeros((n, n, dim, dim))
        for spin in (0, 1):
            r = self.op_matrices("Aa" if spin == 0 else "Bb", na, nb)
            if r is not None:
                E += r[1]
        return E

    def hamiltonian(self, ints: InCoreInts, na, nb):
        """Local FCI Hamiltonian sum h_pq E_pq + 1/2 sum (pr|qs)(E_pr E_qs - d_qr E_ps) (+h0)."""
        dim = self.dim(na, nb)
        if dim == 0:
            return np.zeros((0, 0))
        E = self.one_body_E(na, nb)
        n = E.shape[0]
        H = np.einsum("pq,pqij->ij", ints.h1, E)
        # 1/2 sum_pr E_pr W_pr with W_pr = sum_qs (pr|qs) E_qs: n^2 products of dim x dim
        # matrices instead of the n^4 of E_pr E_qs
        W = (ints.h2.reshape(n * n, n * n) @ E.reshape(n * n, dim * dim)).reshape(n * n, dim, dim)
        H += 0.5 * np.matmul(E.reshape(n * n, dim, dim), W).sum(axis=0)
        H -= 0.5 * np.einsum("prrs,psik->ik", ints.h2, E, optimize=True)
        H += ints.h0 * np.eye(dim)
        return 0.5 * (H + H.T)


class ClusterBasis:
    """Local eigenbasis of one cluster: sector (na, nb) -> (energies, vectors (dim, M))."""

    def __init__(self, idx: int, orbs, space: LocalSpace):
        self.idx = idx
        self.orbs = list(orbs)
        self.space = space
        self.basis = {}
        self.energies = {}

    def __len__(self):
        return len(self.orbs)


def possible_focksectors(n, delta_elec=None):
    """Sectors (na, nb) of an n-orbital cluster, optionally within
    |na - na0| + |nb - nb0| <= delta of a reference (QCBase.possible_focksectors,
    called at build_local_quantities.jl:1136)."""
    out = []
    for na in range(n + 1):
        for nb in range(n + 1):
            if delta_elec is not None:
                na0, nb0, dl = delta_elec
                if abs(na - na0) + abs(nb - nb0) > dl:
                    continue
            out.append((na, nb))
    return out


def compute_cluster_eigenbasis(ints: InCoreInts, clusters, init_fspace=None, delta_elec=None,
                               max_roots=10, rdm1a=None, rdm1b=None):
    """Per cluster and Fock sector, the lowest `max_roots` eigenvectors of the
    local (optionally embedded) FCI Hamiltonian
    (build_local_quantities.jl:1090-1170; dense eigen path)."""
    bases = []
    spaces = {}
    for ci, orbs in enumerate(clusters):
        n = len(orbs)
        if n not in spaces:
            spaces[n] = LocalSpace(n)
        sp = spaces[n]
        if rdm1a is None and rdm1b is None:
            ints_i = subset(ints, orbs)
        else:
            ints_i = subset(ints, orbs, rdm1a, rdm1b)
        de = None
        if delta_elec is not None and init_fspace is not None:
            de = (init_fspace[ci][0], init_fspace[ci][1], delta_elec)
        cb = ClusterBasis(ci, orbs, sp)
        for sec in possible_focksectors(n, de):
            H = sp.hamiltonian(ints_i, *sec)
            w, v = np.linalg.eigh(H)
            nr = min(max_roots, H.shape[0])
            cb.basis[sec] = np.ascontiguousarray(v[:, :nr])
            cb.energies[sec] = w[:nr].copy()
        bases.append(cb)
    return bases


class ClusterOps:
    """op string -> {(fock_bra, fock_ket): TDM block} for one cluster.

    Blocks of 1..3-letter ops have shape (M_ket, M_bra, n^k) (see module doc);
    "H" and "Hcmf" blocks have shape (M_ket, M_bra) (2-D in the reference too).
    """

    def __init__(self, idx):
        self.idx = idx
        self.data = {}

    def __getitem__(self, op):
        return self.data[op]


def _project(U_bra, mats, U_ket):
    # mats: (n,)*k + (dim_t, dim_s) ; returns (M_ket, M_bra, n^k) with first orbital index fastest
    k = mats.ndim - 2
    n = mats.shape[0] if k > 0 else 1
    g = np.einsum("iI,...ij,jJ->...IJ", U_bra, mats, U_ket, optimize=True)  # (p,q,r,I,J)
    # column-major flatten of (p,q,r) -> p fastest ; then store as (J, I, pidx)
    g = g.reshape((n ** k,) + g.shape[k:], order="F") if k > 0 else g[None]
    return np.ascontiguousarray(np.transpose(g, (2, 1, 0)))


def compute_cluster_ops(bases, ints: InCoreInts):
    """TDMs of every op string between every pair of sectors present in the
    basis, plus the local Hamiltonian "H" (build_local_quantities.jl:40-191).

    Adjoint blocks ("a" from "A", "Aaa" from "AAa", ...) are formed directly
    from their own operator strings, which equals the reference's adjoint
    permutations (:303, :356, :440, :482-486, :539, :588-601) by construction.
    """
    ops = []
    for cb in bases:
        co = ClusterOps(cb.idx)
        sp = cb.space
        ints_i = subset(ints, cb.orbs)
        hd = {}
        for sec, U in cb.basis.items():
            H = sp.hamiltonian(ints_i, *sec)
            hd[(sec, sec)] = np.ascontiguousarray((U.T @ H @ U).T)  # (M_ket, M_bra)
        co.data["H"] = hd
        for op in OP_STRINGS:
            d = {}
            for sec_k, U_k in cb.basis.items():
                r = sp.op_matrices(op, *sec_k)
                if r is None:
                    continue
                sec_b, mats = r
                if sec_b not in cb.basis:
                    continue
                d[(sec_b, sec_k)] = _project(cb.basis[sec_b], mats, U_k)
            co.data[op] = d
        ops.append(co)
    return ops


def add_cmf_operators(ops, bases, ints: InCoreInts, rdm1a, rdm1b):
    """Embedded local Hamiltonian blocks "Hcmf" (build_local_quantities.jl:616-652)."""
    for cb, co in zip(bases, ops):
        sp = cb.space
        ints_i = subset(ints, cb.orbs, rdm1a, rdm1b)
        d = {}
        for sec, U in cb.basis.items():
            H = sp.hamiltonian(ints_i, *sec)
            d[(sec, sec)] = np.ascontiguousarray((U.T @ H @ U).T)
        co.data["Hcmf"] = d
