"""CPU restatement of the BST compressed first-order interacting space -- TEST INFRASTRUCTURE ONLY.

Follows, step for step:
  * build_compressed_1st_order_state + its per-FockConfig job (src/tucker_outer.jl:717-910)
  * form_sigma_block_expand 1B-4B (src/tucker_form_sigma_block_expand.jl:7-722), including
    the SVD pre-contraction of the 3B / 4B local operators (precontract = true, prescreen =
    thresh; 1B / 2B keep identity bra factors)
  * Tucker compress / tucker_decompose / nonorth_add / nonorth_dot (src/hosvd.jl:83-545, 949)
  * BSTstate compress / compress_iteratively (src/type_BSTstate.jl:260-296), project_out!
    (src/tucker_outer.jl:1511-1538), orth_dot, compute_expectation_value (src/bst.jl:651-656)
  * the CMF BSTstate and its P / Q spaces (src/type_BSTstate.jl:82-124,
    get_ortho_compliment src/build_local_quantities.jl:12-33)
  * hylleraas_compressed_mp2 (src/tucker_pt.jl:358-532) and do_fois_pt2 (:551-605)
  * cg! of IterativeSolvers.jl (an un-vendored dependency of the reference; restated from its
    published algorithm: plain conjugate gradients from x0 = 0, stopping when the residual
    norm is <= max(sqrt(eps) * |b|, abstol))
numpy, float64.  BST vectors are the dicts of oracle/bst.py:
    (fock tuple, tconfig tuple of (start, stop)) -> {"core": [R arrays], "factors": [N matrices]}
P / Q spaces: one dict per cluster, local Fock sector -> (start, stop).
"""
from __future__ import annotations

import itertools

import numpy as np

from fermicg_gb300.terms import compute_terms_state_sign, extract_1body_operator

from .bst import _gamma, build_dense_H_term, build_sigma, check_term_tucker, contract_dense_H_with_state


# ---- Tucker helpers (src/hosvd.jl) ----------------------------------------------------------
def tucker_len(t):
    return int(np.prod([f.shape[1] for f in t["factors"]]))


def tucker_norm(t):
    """norm(A::Tucker) = norm(A.core): the 2-norm over all roots' cores (hosvd.jl:949)."""
    return float(np.sqrt(sum(float(np.sum(c * c)) for c in t["core"])))


def transform_modes(core, mats, trans=False):
    """new[.., j, ..] = sum_i core[.., i, ..] M[i, j] on every mode with a matrix
    (M^T when trans): transform_basis (hosvd.jl:634-670)."""
    out = core
    for i, M in enumerate(mats):
        if M is None:
            continue
        A = M.T if trans else M
        out = np.moveaxis(np.tensordot(out, A, axes=([i], [0])), -1, i)
    return out


def tucker_decompose(cores, thresh):
    """HOSVD of R tensors of equal shape (hosvd.jl:450-545): for every mode, the eigenvectors
    of sum_r A_r(i) A_r(i)^T with sqrt|eigenvalue| > thresh, largest first.  Returns the
    projected cores and the factors (a mode with none kept gets a (dim, 0) factor)."""
    dims = cores[0].shape
    N = len(dims)
    factors = []
    for i in range(N):
        G = np.zeros((dims[i], dims[i]))
        for A in cores:
            M = np.moveaxis(A, i, 0).reshape(dims[i], -1)
            G += M @ M.T
        w, U = np.linalg.eigh(G)
        w = np.abs(w)
        perm = np.argsort(-w, kind="stable")
        S = np.sqrt(w[perm])
        U = U[:, perm]
        nkeep = int(np.sum(np.abs(S) > thresh))
        factors.append(U[:, :nkeep] if nkeep > 0 else np.zeros((dims[i], 0)))
    new = [transform_modes(A, factors) for A in cores]
    return new, factors


def compress_tucker(t, thresh):
    """compress(t::Tucker; thresh) (hosvd.jl:337-349)."""
    if tucker_len(t) == 0:
        return t
    cores, facs = tucker_decompose(t["core"], thresh)
    return {"core": cores, "factors": [t["factors"][i] @ facs[i] for i in range(len(facs))]}


def nonorth_add_tuckers(tucks, thresh=1e-10):
    """nonorth_add (hosvd.jl:83-156): sort by norm (largest first), per mode the left
    singular vectors of the stacked factors with singular value > thresh, then the sum of
    the cores transformed into those bases."""
    if len(tucks) == 0:
        raise ValueError("not enough Tuckers to add")
    norms = [tucker_norm(t) for t in tucks]
    order = sorted(range(len(tucks)), key=lambda k: -norms[k])
    tucks = [tucks[k] for k in order]
    if len(tucks) == 1:
        return tucks[0]
    N = len(tucks[0]["factors"])
    R = len(tucks[0]["core"])
    new_f = []
    for i in range(N):
        Ui = np.hstack([t["factors"][i] for t in tucks])
        U, S, _ = np.linalg.svd(Ui, full_matrices=False)
        nkeep = int(np.sum(S > thresh))
        new_f.append(U[:, :nkeep])
    shape = tuple(f.shape[1] for f in new_f)
    new_core = [np.zeros(shape) for _ in range(R)]
    for t in tucks:
        tr = [new_f[i].T @ t["factors"][i] for i in range(N)]
        for r in range(R):
            new_core[r] = new_core[r] + transform_modes(t["core"][r], tr, trans=True)
    return {"core": new_core, "factors": new_f}


def nonorth_dot_tucker(t1, t2, r1, r2):
    """nonorth_dot(t1, t2, r1, r2) (hosvd.jl:469-480)."""
    ov = [t1["factors"][f].T @ t2["factors"][f] for f in range(len(t1["factors"]))]
    return float(np.sum(transform_modes(t1["core"][r1], ov) * t2["core"][r2]))


# ---- BSTstate helpers (src/type_BSTstate.jl, src/tucker_outer.jl) ---------------------------
def cmf_bst(bases, init_fspace, R=1):
    """BSTstate(clusters, FockConfig(init_fspace), cluster_bases): P space = the lowest local
    state of each cluster in the reference sector; Q space = its orthogonal complement
    (the rest of that sector, and every other sector whole).  One 1 x ... x 1 block."""
    N = len(bases)
    ref = tuple(tuple(int(x) for x in f) for f in init_fspace)
    p_spaces, q_spaces = [], []
    for c in range(N):
        p = {ref[c]: (0, 1)}
        q = {}
        for fock, B in bases[c].basis.items():
            M = B.shape[1]
            rng = (1, M) if fock == ref[c] else (0, M)
            if rng[1] - rng[0] > 0:
                q[fock] = rng
        p_spaces.append(p)
        q_spaces.append(q)
    tcfg = tuple(p_spaces[c][ref[c]] for c in range(N))
    core = [np.ones((1,) * N) for _ in range(R)]
    vec = {(ref, tcfg): {"core": core, "factors": [np.eye(1) for _ in range(N)]}}
    return vec, p_spaces, q_spaces


def bst_len(vec):
    return sum(tucker_len(t) for t in vec.values())


def compress_bst(vec, thresh):
    """compress(ts::BSTstate; thresh): every block compressed, empty blocks dropped."""
    out = {}
    for k, t in vec.items():
        tt = compress_tucker(t, thresh)
        if tucker_len(tt) > 0:
            out[k] = tt
    return out


def compress_iteratively(vec, thresh, maxiter=20):
    for _ in range(maxiter):
        d1 = bst_len(vec)
        vec = compress_bst(vec, thresh)
        if not bst_len(vec) < d1:
            break
    return vec


def project_out(v, w):
    """project_out!(v, w): |v> -= |w><w|v> block by block, as the reference does it."""
    Rw = len(next(iter(w.values()))["core"]) if w else 0
    for rw in range(Rw):
        for key in list(v.keys()):
            if key not in w:
                continue
            wt = w[key]
            ww = float(np.sum(wt["core"][rw] * wt["core"][rw]))
            Rv = len(v[key]["core"])
            for rv in range(Rv):
                t = v[key]
                ovlp = nonorth_dot_tucker(t, wt, rv, rw) / ww
                tmp = {"core": [c * (-ovlp) for c in wt["core"]], "factors": wt["factors"]}
                v[key] = nonorth_add_tuckers([t, tmp], thresh=1e-16)
    return v


def zero_copy(vec, R=None):
    return {k: {"core": [np.zeros_like(t["core"][0]) for _ in range(R or len(t["core"]))],
                "factors": t["factors"]} for k, t in vec.items()}


def get_vector(vec, R):
    return np.column_stack([np.concatenate([t["core"][r].reshape(-1, order="F") for t in vec.values()])
                            for r in range(R)]) if vec else np.zeros((0, R))


def set_vector(vec, x, r):
    o = 0
    for t in vec.values():
        n = t["core"][r].size
        t["core"][r] = x[o:o + n].reshape(t["core"][r].shape, order="F").copy()
        o += n


def orth_dot(a, b, R):
    return np.array([sum(float(np.sum(a[k]["core"][r] * b[k]["core"][r])) for k in a if k in b) for r in range(R)])


def expectation(vec, ops, ham, N, R):
    tmp = zero_copy(vec, R)
    build_sigma(tmp, vec, ops, ham, N, R)
    return orth_dot(tmp, vec, R)


# ---- the expansion (src/tucker_form_sigma_block_expand.jl) ----------------------------------
def _precontract(g, scale1, prescreen):
    """SVD of the local operator g[p, I, l] over its bra index I: keep s * scale1 > prescreen;
    returns (new bra factor U (I x k), g'[p, k, l] = (S Vt) reshaped)."""
    P, I, L = g.shape
    D = np.transpose(g, (1, 0, 2)).reshape(I, P * L)
    U, S, Vt = np.linalg.svd(D, full_matrices=False)
    nkeep = int(np.sum(S * scale1 > prescreen))
    gp = (S[:nkeep, None] * Vt[:nkeep]).reshape(nkeep, P, L)
    return U[:, :nkeep], np.transpose(gp, (1, 0, 2))


def form_sigma_block_expand(term, ops, fb, tb, fk, tk, ket, N, R, prescreen):
    """H term applied to one ket Tucker block, into the bra TuckerConfig's full local ranges on
    the active clusters (1B / 2B: identity bra factors) or into SVD-truncated bra factors
    (3B / 4B); spectator factors are the ket's.  Returns a Tucker or None."""
    sgn = compute_terms_state_sign(term, fk)
    act = list(term.clusters)
    factors = list(ket["factors"])
    if term.nbody <= 2:
        for c in act:
            factors[c] = np.eye(tb[c][1] - tb[c][0])
        bra = {"factors": factors}
        op = build_dense_H_term(term, ops, fb, tb, bra, fk, tk, ket)
        if op is None:
            return None
    else:
        scale0 = max(1.0, max(float(np.linalg.norm(ket["core"][r])) for r in range(R)))
        scale1 = scale0 * float(np.linalg.norm(term.ints))
        gs = []
        for c, o in zip(term.clusters, term.ops):
            g = _gamma(ops, c, o, fb, fk, tb[c], tk[c])
            if g is None:
                return None
            g = np.einsum("pIJ,Jl->pIl", g, ket["factors"][c])
            U, gp = _precontract(g, scale1, prescreen)
            factors[c] = U
            gs.append(gp)
        v = term.ints
        if term.nbody == 3:
            op = np.einsum("pqr,pIJ,qKL,rMN->JLNIKM", v, gs[0], gs[1], gs[2], optimize=True)
        else:
            op = np.einsum("pqrs,pIJ,qKL,rMN,sOP->JLNPIKMO", v, gs[0], gs[1], gs[2], gs[3], optimize=True)
        bra = {"factors": factors}
    cores = contract_dense_H_with_state(term, op, sgn, bra, ket, N, R)
    return {"core": cores, "factors": factors}


def build_compressed_1st_order_state(psi, p_spaces, q_spaces, ops, ham, N, R, thresh=1e-7, nbody=4,
                                     compress_twice=True, norb=None):
    """build_compressed_1st_order_state (tucker_outer.jl:717-910)."""
    jobs = {}
    by_fock = {}
    for (fk, tk), tuck in psi.items():
        by_fock.setdefault(fk, {})[tk] = tuck
    for fk, configs in by_fock.items():
        for tr, terms in ham:
            fs = tuple((fk[c][0] + tr[c][0], fk[c][1] + tr[c][1]) for c in range(N))
            if any(f[0] < 0 or f[1] < 0 for f in fs):
                continue
            if norb is not None and any(fs[c][0] > norb[c] or fs[c][1] > norb[c] for c in range(N)):
                continue
            if any((fs[c], fs[c]) not in ops[c].data["H"] for c in range(N)):
                continue
            jobs.setdefault(fs, []).append((terms, fk, configs))
    sigma = {}
    for fs, job in jobs.items():
        data = {}
        for terms, fk, configs in job:
            for term in terms:
                if term.nbody > nbody:
                    continue
                for tk, tuck in configs.items():
                    avail = []
                    for c in term.clusters:
                        lst = []
                        if fs[c] in p_spaces[c]:
                            lst.append(p_spaces[c][fs[c]])
                        if fs[c] in q_spaces[c]:
                            lst.append(q_spaces[c][fs[c]])
                        avail.append(lst)
                    for prod in itertools.product(*avail):
                        tb = list(tk)
                        for q, c in enumerate(term.clusters):
                            tb[c] = prod[q]
                        tb = tuple(tb)
                        if not check_term_tucker(term, fs, tb, fk, tk):
                            continue
                        t = form_sigma_block_expand(term, ops, fs, tb, fk, tk, tuck, N, R, thresh)
                        if t is None or tucker_len(t) == 0:
                            continue
                        t = compress_tucker(t, thresh)
                        if tucker_len(t) == 0:
                            continue
                        data.setdefault(tb, []).append(t)
        for tb, tucks in data.items():
            s = nonorth_add_tuckers(tucks)
            sigma[(fs, tb)] = compress_tucker(s, thresh) if compress_twice else s
    return compress_iteratively(sigma, thresh)


# ---- PT2 in the compressed FOIS (src/tucker_pt.jl) ------------------------------------------
def cg(matvec, b, abstol=1e-6, maxiter=100):
    """Conjugate gradients from x = 0 as IterativeSolvers.cg! runs them: stop when the
    residual norm is <= max(sqrt(eps) |b|, abstol) or after maxiter products."""
    x = np.zeros_like(b)
    r = b.copy()
    u = np.zeros_like(b)
    res = float(np.linalg.norm(r))
    tol = max(np.sqrt(np.finfo(float).eps) * res, abstol)
    prev = 1.0
    it = 0
    while it < maxiter and not res <= tol:
        beta = res * res / (prev * prev)
        u = r + beta * u
        c = matvec(u)
        alpha = res * res / float(np.dot(u, c))
        x = x + alpha * u
        r = r - alpha * c
        prev = res
        res = float(np.linalg.norm(r))
        it += 1
    return x, it


def hylleraas_compressed_mp2(sig_in, ref, ops, ham, N, R, tol=1e-6, max_iter=100):
    """hylleraas_compressed_mp2 (tucker_pt.jl:358-532) with H0 = Hcmf: returns (psi1, e_pt2)."""
    ham0 = extract_1body_operator(ham, "Hcmf")
    sig = zero_copy(sig_in, R)
    build_sigma(sig, ref, ops, ham, N, R)
    e_ref = expectation(ref, ops, ham, N, R)
    e0 = expectation(ref, ops, ham0, N, R)
    Sx = zero_copy(sig, R)
    for key, t in Sx.items():
        if key in ref:
            rt = ref[key]
            ov = [rt["factors"][i].T @ t["factors"][i] for i in range(N)]
            for r in range(R):
                t["core"][r] = transform_modes(rt["core"][r], ov)
    b = -get_vector(sig, R)
    tmp = zero_copy(sig, R)
    build_sigma(tmp, ref, ops, ham0, N, R)
    b = b + get_vector(tmp, R)
    psi1 = zero_copy(sig, R)
    sxv = get_vector(Sx, R)

    def matvec(x):
        xr = zero_copy(sig, 1)
        set_vector(xr, x, 0)
        xl = zero_copy(sig, 1)
        build_sigma(xl, xr, ops, ham0, N, 1)
        return get_vector(xl, 1)[:, 0] - e0[0] * x

    for r in range(R):
        br = b[:, r] + sxv[:, r] * (e_ref[r] - e0[r])
        x, _ = cg(matvec, br, abstol=tol, maxiter=max_iter)
        set_vector(psi1, x, r)
    SxC = orth_dot(Sx, psi1, R)
    tmp = zero_copy(ref, R)
    build_sigma(tmp, psi1, ops, ham, N, R)
    ecorr = orth_dot(tmp, ref, R)
    return psi1, (e_ref + ecorr) / (1.0 + SxC)


def ci_solve_dense(vec, ops, ham, N, R):
    """ci_solve on a small BST space (tucker_outer.jl:68-190), dense: the lowest R eigenpairs of
    H over the cores (each block's factors orthonormal, blocks disjoint)."""
    n = bst_len(vec)
    H = np.zeros((n, n))
    for j in range(n):
        e = np.zeros(n)
        e[j] = 1.0
        x = zero_copy(vec, 1)
        set_vector(x, e, 0)
        y = zero_copy(vec, 1)
        build_sigma(y, x, ops, ham, N, 1)
        H[:, j] = get_vector(y, 1)[:, 0]
    w, V = np.linalg.eigh(0.5 * (H + H.T))
    out = zero_copy(vec, R)
    for r in range(R):
        set_vector(out, V[:, r], r)
    return w[:R], out


def do_fois_pt2(ref, p_spaces, q_spaces, ops, ham, N, R, thresh_foi=1e-6, norb=None):
    """do_fois_pt2 (tucker_pt.jl:551-605): zeroth-order solve, compressed FOIS, project out
    the reference, compress, Hylleraas functional.  Returns (e_pt2, psi1, fois length)."""
    _, ref_vec = ci_solve_dense(ref, ops, ham, N, R)
    pt1 = build_compressed_1st_order_state(ref_vec, p_spaces, q_spaces, ops, ham, N, R, thresh=thresh_foi,
                                           norb=norb)
    project_out(pt1, ref)
    pt1 = compress_bst(pt1, thresh_foi)
    psi1, e_pt2 = hylleraas_compressed_mp2(pt1, ref_vec, ops, ham, N, R)
    return e_pt2, psi1, bst_len(pt1)
