"""CPU restatement of the BST (block-sparse Tucker) sigma build -- TEST INFRASTRUCTURE ONLY.

build_sigma! (src/tucker_inner.jl:165-245) -> form_sigma_block! (:253-304) ->
build_dense_H_term (src/tucker_build_dense_H_term.jl:5-175) and
contract_dense_H_with_state (src/tucker_contract_dense_H_with_state.jl:4-330), with
transform_basis (src/hosvd.jl:634-670) for the spectator overlaps.  numpy, float64.

A BST vector here is a dict
    (fock tuple, tconfig tuple of (start, stop) per cluster) -> {"core": [R arrays], "factors": [N matrices]}
with 0-based, half-open local-state ranges (the reference's 1-based UnitRanges), factors
of shape (stop - start, rank) and cores of shape (rank_1, ..., rank_N).
Block-pair/term enumeration and check_term follow the reference; the tensor algebra is
written with einsum over named indices (same sums, same index meaning).
"""
from __future__ import annotations

import numpy as np

from fermicg_gb300.terms import compute_terms_state_sign


def check_term_tucker(term, fb, tb, fk, tk):
    """check_term on TuckerConfigs (type_ClusteredTerm.jl:92-176): spectator clusters need
    equal Fock sectors and equal ranges; active clusters need fb = fk + delta."""
    n = len(tb)
    for ci in range(n):
        if ci in term.clusters:
            continue
        if fb[ci] != fk[ci] or tb[ci] != tk[ci]:
            return False
    for c, d in zip(term.clusters, term.delta):
        if fb[c] != (fk[c][0] + d[0], fk[c][1] + d[1]):
            return False
    return True


def _gamma(ops, c, op, fb, fk, rb, rk):
    """TDM slice G[p, I, J] over the bra / ket local-state ranges (p fastest in the blob)."""
    blk = ops[c].data[op].get((fb[c], fk[c]))
    if blk is None:
        return None
    g = np.transpose(blk, (2, 1, 0))  # (p, I, J)
    return g[:, rb[0]:rb[1], rk[0]:rk[1]]


def build_dense_H_term(term, ops, fb, tb, bra, fk, tk, ket):
    """Dense operator of `term` in the Tucker bases of the active clusters.

    Returns op with axes (ket ranks of the active clusters..., bra ranks...), i.e. the
    reference's op[J, L, ..., I, K, ...] (tucker_build_dense_H_term.jl:19-175)."""
    if term.nbody == 1:
        c = term.clusters[0]
        H = ops[c].data[term.ops[0]][(fb[c], fk[c])].T  # (I, J)
        Hs = H[tb[c][0]:tb[c][1], tk[c][0]:tk[c][1]]
        return (bra["factors"][c].T @ Hs @ ket["factors"][c]).T  # (kk, kb) -> ket index first
    gs = []
    for c, op in zip(term.clusters, term.ops):
        g = _gamma(ops, c, op, fb, fk, tb[c], tk[c])
        if g is None:
            return None
        Ul, Ur = bra["factors"][c], ket["factors"][c]
        gs.append(np.einsum("Ik,pIJ,Jl->pkl", Ul, g, Ur, optimize=True))  # g[p, kb, kk]
    v = term.ints
    if term.nbody == 2:
        return np.einsum("pq,pIJ,qKL->JLIK", v, gs[0], gs[1], optimize=True)
    if term.nbody == 3:
        return np.einsum("pqr,pIJ,qKL,rMN->JLNIKM", v, gs[0], gs[1], gs[2], optimize=True)
    return np.einsum("pqrs,pIJ,qKL,rMN,sOP->JLNPIKMO", v, gs[0], gs[1], gs[2], gs[3], optimize=True)


def contract_dense_H_with_state(term, op, state_sign, bra, ket, N, R):
    """bra core += s * op^T * (ket core with spectator overlaps applied)
    (tucker_contract_dense_H_with_state.jl:4-330); returns the R added tensors."""
    act = list(term.clusters)
    s = 1.0 if term.nbody == 1 else float(state_sign)
    overlaps = {}
    for ci in range(N):
        if ci in act:
            continue
        S = bra["factors"][ci].T @ ket["factors"][ci]
        if S.size == 1:
            s *= float(S.reshape(-1)[0])
        else:
            overlaps[ci] = S
    na = len(act)
    out = []
    for r in range(R):
        k2 = ket["core"][r]
        for ci, S in overlaps.items():  # transform_basis(..., trans=true): new[.., kb, ..] = S[kb, kk] old[.., kk, ..]
            k2 = np.moveaxis(np.tensordot(S, k2, axes=([1], [ci])), 0, ci)
        # op axes: (kk_active..., kb_active...)
        letters = "abcdefghijklmnopqrstuvwxyz"
        kk = [letters[i] for i in range(na)]
        kb = [letters[na + i] for i in range(na)]
        rest = [letters[2 * na + ci] for ci in range(N)]
        ket_idx = list(rest)
        bra_idx = list(rest)
        for q, c in enumerate(act):
            ket_idx[c] = kk[q]
            bra_idx[c] = kb[q]
        spec = "".join(kk + kb) + "," + "".join(ket_idx) + "->" + "".join(bra_idx)
        out.append(s * np.einsum(spec, op, k2, optimize=True))
    return out


def build_sigma(sigma, vec, ops, ham, N, R, nbody=4):
    """build_sigma! (tucker_inner.jl:165-245): sigma blocks += H vec, block by block."""
    for (fb, tb), bra in sigma.items():
        for (fk, tk), ket in vec.items():
            tr = tuple((fb[c][0] - fk[c][0], fb[c][1] - fk[c][1]) for c in range(N))
            if tr not in ham.trans:
                continue
            for term in ham.trans[tr]:
                if term.nbody > nbody or not check_term_tucker(term, fb, tb, fk, tk):
                    continue
                sgn = compute_terms_state_sign(term, fk)
                op = build_dense_H_term(term, ops, fb, tb, bra, fk, tk, ket)
                if op is None:
                    continue
                add = contract_dense_H_with_state(term, op, sgn, bra, ket, N, R)
                for r in range(R):
                    bra["core"][r] = bra["core"][r] + add[r]
    return sigma


def zero_like(vec, R):
    return {k: {"core": [np.zeros_like(b["core"][0]) for _ in range(R)], "factors": b["factors"]}
            for k, b in vec.items()}
