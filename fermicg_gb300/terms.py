"""ClusteredTerm / ClusteredOperator: the clustered Hamiltonian.

Host-side restatement of extract_ClusteredTerms (type_ClusteredOperator.jl:53-636)
and unique! (type_ClusteredOperator.jl:724-806), plus the term helpers
check_term (type_ClusteredTerm.jl:92-176) and compute_terms_state_sign
(type_ClusteredTerm.jl:181-196).

Term integrals are kept with the reference's axis meaning (a numpy array whose
axis i is Julia dimension i+1) and flattened column-major for the device, so
that `ints[(p..), (q..), ...]` lines up with the TDM multi-indices.
Cluster indices are 0-based.
"""
from __future__ import annotations

from itertools import permutations

import numpy as np

from .integrals import InCoreInts


class ClusteredTerm:
    __slots__ = ("ops", "delta", "parity", "clusters", "ints")

    def __init__(self, ops, delta, parity, clusters, ints):
        self.ops = tuple(ops)
        self.delta = tuple(tuple(int(x) for x in d) for d in delta)
        self.parity = tuple(int(p) for p in parity)
        self.clusters = tuple(int(c) for c in clusters)
        self.ints = np.asarray(ints, dtype=np.float64)

    @property
    def nbody(self):
        return len(self.clusters)

    def key(self):
        return "".join(f"{o}({c + 1})" for o, c in zip(self.ops, self.clusters))

    def __repr__(self):
        return f"{self.nbody}B{self.clusters}{self.ops}"


class ClusteredOperator:
    """TransferConfig (tuple of (da, db) per cluster) -> list of ClusteredTerm."""

    def __init__(self, n_clusters):
        self.n_clusters = n_clusters
        self.trans = {}

    def __iter__(self):
        return iter(self.trans.items())

    def __len__(self):
        return len(self.trans)

    def n_terms(self):
        return sum(len(v) for v in self.trans.values())


def bubble_sort(inp):
    """Stable sort returning (permutation, swap count) (Utils.jl:47-64); 0-based perm."""
    blist = list(inp)
    bperm = list(range(len(inp)))
    swaps = 0
    for j in range(1, len(blist) + 1):
        for i in range(0, len(blist) - j):
            if blist[i] > blist[i + 1]:
                swaps += 1
                blist[i], blist[i + 1] = blist[i + 1], blist[i]
                bperm[i], bperm[i + 1] = bperm[i + 1], bperm[i]
    return bperm, swaps


def _unique_perms(seq):
    seen = []
    for p in permutations(seq):
        if p not in seen:
            seen.append(p)
    return seen


def _replace(zero, idxs, focks):
    t = list(zero)
    for i, f in zip(idxs, focks):
        t[i] = (int(f[0]), int(f[1]))
    return tuple(t)


def _add(terms, key, term):
    terms.trans.setdefault(key, []).append(term)


_SPIN2 = [["A", "A", "a", "a"], ["B", "B", "b", "b"], ["A", "B", "b", "a"], ["B", "A", "a", "b"]]
_FOCK2 = [[(1, 0), (1, 0), (-1, 0), (-1, 0)], [(0, 1), (0, 1), (0, -1), (0, -1)],
          [(1, 0), (0, 1), (0, -1), (-1, 0)], [(0, 1), (1, 0), (-1, 0), (0, -1)]]
_SPIN1 = [["A", "a"], ["B", "b"]]
_FOCK1 = [[(1, 0), (-1, 0)], [(0, 1), (0, -1)]]

# renames of type_ClusteredOperator.jl:275-315 (2B), :446-472 (3B):
# (operator position in term, old string) -> (new string, axis swap applied with a minus sign)


def _split_ops(term_sorted, active, oper, fock):
    """Concatenate the sorted operator letters per active cluster."""
    opers = ["" for _ in active]
    focks = [[0, 0] for _ in active]
    for cidx, c in enumerate(term_sorted):
        a = active.index(c)
        opers[a] += oper[cidx]
        focks[a][0] += fock[cidx][0]
        focks[a][1] += fock[cidx][1]
    return opers, focks


def _sorted_2e_ints(ints, term, orbs):
    """0.5 * permsign * (pr|qs) aligned with the sorted operator string p'q's r
    (type_ClusteredOperator.jl:218-239)."""
    perm, swaps = bubble_sort(term)
    permsign = -1.0 if swaps % 2 else 1.0
    o = [orbs[c] for c in term]
    vprqs = ints.h2[np.ix_(o[0], o[3], o[1], o[2])]
    vpqsr = np.transpose(vprqs, (0, 2, 3, 1))
    v = (0.5 * permsign) * np.transpose(vpqsr, perm)
    return perm, v


def extract_ClusteredTerms(ints: InCoreInts, clusters):
    """Split H into 1-4 body ClusteredTerms grouped by TransferConfig.

    `clusters` is a list of 0-based orbital lists (consecutive clusters)."""
    nc = len(clusters)
    orbs = [list(c) for c in clusters]
    terms = ClusteredOperator(nc)
    zero = tuple((0, 0) for _ in range(nc))
    terms.trans[zero] = []

    # 1-body: precontracted local Hamiltonians
    for ci in range(nc):
        _add(terms, zero, ClusteredTerm(("H",), ((0, 0),), (0,), (ci,), np.zeros(1)))

    # 2-body 1-electron terms  h_pq p'q
    for ci in range(nc):
        for cj in range(ci + 1, nc):
            for term in _unique_perms([ci, cj]):
                perm, swaps = bubble_sort(term)
                permsign = -1.0 if swaps % 2 else 1.0
                hpq = ints.h1[np.ix_(orbs[term[0]], orbs[term[1]])]
                h = permsign * np.transpose(hpq, perm)
                ts = [term[p] for p in perm]
                for sidx in range(2):
                    oper = [_SPIN1[sidx][p] for p in perm]
                    fock = [_FOCK1[sidx][p] for p in perm]
                    (o1, o2), (f1, f2) = _split_ops(ts, [ci, cj], oper, fock)
                    par = (len(o1) % 2, len(o2) % 2)
                    t = ClusteredTerm((o1, o2), (f1, f2), par, (ci, cj), h.copy())
                    _add(terms, _replace(zero, (ci, cj), (f1, f2)), t)

    # 2-body 2-electron terms
    for ci in range(nc):
        for cj in range(ci + 1, nc):
            termstr = (_unique_perms([ci, ci, cj, cj]) + _unique_perms([ci, cj, cj, cj])
                       + _unique_perms([ci, ci, ci, cj]))
            for term in termstr:
                perm, v = _sorted_2e_ints(ints, term, orbs)
                ts = [term[p] for p in perm]
                shape = [1, 1]
                for cidx, c in enumerate(ts):
                    shape[0 if c == ci else 1] *= v.shape[cidx]
                for sidx in range(4):
                    oper = [_SPIN2[sidx][p] for p in perm]
                    fock = [_FOCK2[sidx][p] for p in perm]
                    (o1, o2), (f1, f2) = _split_ops(ts, [ci, cj], oper, fock)
                    vc = v.copy()
                    if o1 == "BA":
                        o1, vc = "AB", -np.transpose(vc, (1, 0, 2, 3))
                    elif o1 == "ba":
                        o1, vc = "ab", -np.transpose(vc, (1, 0, 2, 3))
                    elif o1 == "BAa":
                        o1, vc = "ABa", -np.transpose(vc, (1, 0, 2, 3))
                    elif o1 == "BAb":
                        o1, vc = "ABb", -np.transpose(vc, (1, 0, 2, 3))
                    elif o1 == "Bab":
                        o1, vc = "Bba", -np.transpose(vc, (0, 2, 1, 3))
                    elif o1 == "Aab":
                        o1, vc = "Aba", -np.transpose(vc, (0, 2, 1, 3))
                    if o2 == "BA":
                        o2, vc = "AB", -np.transpose(vc, (0, 1, 3, 2))
                    elif o2 == "ba":
                        o2, vc = "ab", -np.transpose(vc, (0, 1, 3, 2))
                    elif o2 == "BAa":
                        o2, vc = "ABa", -np.transpose(vc, (0, 2, 1, 3))
                    elif o2 == "BAb":
                        o2, vc = "ABb", -np.transpose(vc, (0, 2, 1, 3))
                    elif o2 == "Bab":
                        o2, vc = "Bba", -np.transpose(vc, (0, 1, 3, 2))
                    elif o2 == "Aab":
                        o2, vc = "Aba", -np.transpose(vc, (0, 1, 3, 2))
                    vc = vc.reshape(shape, order="F").copy(order="F")
                    par = (len(o1) % 2, len(o2) % 2)
                    t = ClusteredTerm((o1, o2), (f1, f2), par, (ci, cj), vc)
                    _add(terms, _replace(zero, (ci, cj), (f1, f2)), t)

    # 3-body 2-electron terms
    for ci in range(nc):
        for cj in range(ci + 1, nc):
            for ck in range(cj + 1, nc):
                termstr = (_unique_perms([ci, ci, cj, ck]) + _unique_perms([ci, cj, cj, ck])
                           + _unique_perms([ci, cj, ck, ck]))
                act = [ci, cj, ck]
                for term in termstr:
                    perm, v = _sorted_2e_ints(ints, term, orbs)
                    ts = [term[p] for p in perm]
                    shape = [1, 1, 1]
                    for cidx, c in enumerate(ts):
                        shape[act.index(c)] *= v.shape[cidx]
                    for sidx in range(4):
                        oper = [_SPIN2[sidx][p] for p in perm]
                        fock = [_FOCK2[sidx][p] for p in perm]
                        (o1, o2, o3), (f1, f2, f3) = _split_ops(ts, act, oper, fock)
                        vc = v.copy()
                        if o1 == "BA":
                            o1, vc = "AB", -np.transpose(vc, (1, 0, 2, 3))
                        elif o1 == "ba":
                            o1, vc = "ab", -np.transpose(vc, (1, 0, 2, 3))
                        if o2 == "BA":
                            o2, vc = "AB", -np.transpose(vc, (0, 2, 1, 3))
                        elif o2 == "ba":
                            o2, vc = "ab", -np.transpose(vc, (0, 2, 1, 3))
                        if o3 == "BA":
                            o3, vc = "AB", -np.transpose(vc, (0, 1, 3, 2))
                        elif o3 == "ba":
                            o3, vc = "ab", -np.transpose(vc, (0, 1, 3, 2))
                        vc = vc.reshape(shape, order="F").copy(order="F")
                        par = (len(o1) % 2, len(o2) % 2, len(o3) % 2)
                        t = ClusteredTerm((o1, o2, o3), (f1, f2, f3), par, (ci, cj, ck), vc)
                        _add(terms, _replace(zero, act, (f1, f2, f3)), t)

    # 4-body 2-electron terms
    for ci in range(nc):
        for cj in range(ci + 1, nc):
            for ck in range(cj + 1, nc):
                for cl in range(ck + 1, nc):
                    act = [ci, cj, ck, cl]
                    for term in _unique_perms(act):
                        perm, v = _sorted_2e_ints(ints, term, orbs)
                        ts = [term[p] for p in perm]
                        for sidx in range(4):
                            oper = [_SPIN2[sidx][p] for p in perm]
                            fock = [_FOCK2[sidx][p] for p in perm]
                            opers, focks = _split_ops(ts, act, oper, fock)
                            par = tuple(len(o) % 2 for o in opers)
                            t = ClusteredTerm(opers, focks, par, act, v.copy(order="F"))
                            _add(terms, _replace(zero, act, focks), t)

    unique(terms)
    return terms


def unique(terms: ClusteredOperator):
    """Sum the integrals of terms with equal (ops, clusters) within a transfer
    (type_ClusteredOperator.jl:783-802)."""
    for ftrans, tl in list(terms.trans.items()):
        u = {}
        for t in tl:
            k = t.key()
            if k in u:
                u[k].ints = u[k].ints + t.ints
            else:
                u[k] = ClusteredTerm(t.ops, t.delta, t.parity, t.clusters, t.ints.copy(order="F"))
        terms.trans[ftrans] = list(u.values())


def extract_1body_operator(terms: ClusteredOperator, op_string="H"):
    """The 1-body part of H with its op renamed (type_ClusteredOperator.jl:819-835)."""
    out = ClusteredOperator(terms.n_clusters)
    for ftrans, tl in terms:
        for t in tl:
            if t.nbody == 1:
                out.trans.setdefault(ftrans, []).append(
                    ClusteredTerm((op_string,), t.delta, t.parity, t.clusters, t.ints))
    return out


def check_term(term: ClusteredTerm, fock_bra, bra, fock_ket, ket):
    """type_ClusteredTerm.jl:92-176"""
    n = len(bra)
    for ci in range(n):
        if ci in term.clusters:
            continue
        if fock_bra[ci] != fock_ket[ci] or bra[ci] != ket[ci]:
            return False
    for c, d in zip(term.clusters, term.delta):
        if fock_bra[c] != (fock_ket[c][0] + d[0], fock_ket[c][1] + d[1]):
            return False
    return True


def compute_terms_state_sign(term: ClusteredTerm, fock_ket):
    """(-1)^(electrons in ket clusters before c) for every odd op (type_ClusteredTerm.jl:181-196)."""
    s = 1
    for o, p, c in zip(term.ops, term.parity, term.clusters):
        if p == 1:
            ne = sum(fock_ket[ci][0] + fock_ket[ci][1] for ci in range(c))
            if ne % 2:
                s = -s
    return s
