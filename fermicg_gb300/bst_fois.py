"""Block-sparse Tucker first-order interacting space (FOIS) and FOIS-PT2 on the GPU.

build_compressed_1st_order_state (src/tucker_outer.jl:717-910) runs in the library
(fcg_bst_fois: the expansion through the device BST sigma, the HOSVD compressions and
nonorth_add in device kernels).  do_fois_pt2 (src/tucker_pt.jl:551-605) and
hylleraas_compressed_mp2 (src/tucker_pt.jl:358-532) run here on top of it: every sigma build
(<X|H|0>, <X|F|0>, F|x> inside the conjugate gradient, <0|H|1>) is one device BST sigma over
the reference and FOIS blocks together; the conjugate gradient (IterativeSolvers.cg!, from
x = 0 with its stopping rule), the projection of the reference out of the FOIS and the few
block compressions around it are host work on vectors of the FOIS length.

BST vectors are dicts (fock tuple, tconfig tuple of (start, stop)) ->
{"core": [R arrays], "factors": [N matrices]}, as in fermicg_gb300.bst; P / Q spaces are one
dict per cluster, local Fock sector -> (start, stop).
"""
from __future__ import annotations

import numpy as np

from . import pack
from .gpu import GpuSigma
from .terms import extract_1body_operator


# ---- layouts ------------------------------------------------------------------------------------
def cmf_state(bases, init_fspace, R=1):
    """BSTstate(clusters, FockConfig(init_fspace), cluster_bases) (src/type_BSTstate.jl:82-124):
    the P space is each cluster's lowest local state in the reference sector, the Q space its
    complement in the cluster basis (get_ortho_compliment, src/build_local_quantities.jl:12-33),
    and the state one 1 x ... x 1 block."""
    N = len(bases)
    ref = tuple(tuple(int(x) for x in f) for f in init_fspace)
    P, Q = [], []
    for c in range(N):
        P.append({ref[c]: (0, 1)})
        q = {}
        for fock, B in bases[c].basis.items():
            rng = (1, B.shape[1]) if fock == ref[c] else (0, B.shape[1])
            if rng[1] > rng[0]:
                q[fock] = rng
        Q.append(q)
    tcfg = tuple(P[c][ref[c]] for c in range(N))
    vec = {(ref, tcfg): {"core": [np.ones((1,) * N) for _ in range(R)], "factors": [np.eye(1) for _ in range(N)]}}
    return vec, P, Q


def spaces_array(P, Q, N, nmax):
    """int32 [N][nmax+1][nmax+1][4] = {p_start, p_len, q_start, q_len} (the fcg_bst_fois layout)."""
    out = np.zeros((N, nmax + 1, nmax + 1, 4), dtype=np.int32)
    for c in range(N):
        for (na, nb), (a, b) in P[c].items():
            out[c, na, nb, 0:2] = (a, b - a)
        for (na, nb), (a, b) in Q[c].items():
            out[c, na, nb, 2:4] = (a, b - a)
    return out


def pack_blocks(entries, N, R):
    """entries: list of ((fock, tconfig), tucker) -> fock, blocks {rank, start, len}, factor_off,
    factors, cores (R, core_total), core offsets.  Keys may repeat (the blocks are separate)."""
    fock = np.zeros((len(entries), N, 2), dtype=np.int16)
    blocks = np.zeros((len(entries), 3 * N), dtype=np.int64)
    foff = np.zeros((len(entries), N), dtype=np.int64)
    fac, offs, cores = [], [], [[] for _ in range(R)]
    fo = co = 0
    for i, ((fk, tc), t) in enumerate(entries):
        fock[i] = fk
        for c in range(N):
            f = np.asarray(t["factors"][c], dtype=np.float64)
            blocks[i, c] = f.shape[1]
            blocks[i, N + c] = tc[c][0]
            blocks[i, 2 * N + c] = tc[c][1] - tc[c][0]
            foff[i, c] = fo
            fac.append(f.reshape(-1, order="F"))
            fo += f.size
        offs.append(co)
        for r in range(R):
            cores[r].append(np.asarray(t["core"][r], dtype=np.float64).reshape(-1, order="F"))
        co += int(np.prod(blocks[i, :N]))
    core_arr = np.stack([np.concatenate(cr) if cr else np.zeros(0) for cr in cores])
    return fock, blocks, foff, np.concatenate(fac), core_arr, offs


def unpack_blocks(fock, blocks, foff, factors, cores, N, R):
    vec = {}
    co = 0
    for i in range(blocks.shape[0]):
        rk = [int(x) for x in blocks[i, :N]]
        st = [int(x) for x in blocks[i, N:2 * N]]
        ln = [int(x) for x in blocks[i, 2 * N:]]
        fk = tuple((int(fock[i, c, 0]), int(fock[i, c, 1])) for c in range(N))
        tc = tuple((st[c], st[c] + ln[c]) for c in range(N))
        facs = [factors[foff[i, c]:foff[i, c] + ln[c] * rk[c]].reshape((ln[c], rk[c]), order="F") for c in range(N)]
        n = int(np.prod(rk))
        vec[(fk, tc)] = {"core": [cores[r, co:co + n].reshape(rk, order="F") for r in range(R)], "factors": facs}
        co += n
    return vec


# ---- small host Tucker algebra (project_out! and the compressions around it) --------------------
def _transform(core, mats, trans=False):
    out = core
    for i, M in enumerate(mats):
        A = M.T if trans else M
        out = np.moveaxis(np.tensordot(out, A, axes=([i], [0])), -1, i)
    return out


def _len(t):
    return int(np.prod([f.shape[1] for f in t["factors"]]))


def compress_block(t, thresh):
    """compress (src/hosvd.jl:337-349) of one block on the host: HOSVD of its cores."""
    if _len(t) == 0:
        return t
    cores = t["core"]
    N = cores[0].ndim
    facs = []
    for i in range(N):
        d = cores[0].shape[i]
        G = np.zeros((d, d))
        for A in cores:
            M = np.moveaxis(A, i, 0).reshape(d, -1)
            G += M @ M.T
        w, U = np.linalg.eigh(G)
        w = np.abs(w)
        order = np.argsort(-w, kind="stable")
        S = np.sqrt(w[order])
        k = int(np.sum(S > thresh))
        facs.append(U[:, order][:, :k])
    return {"core": [_transform(A, facs) for A in cores], "factors": [t["factors"][i] @ facs[i] for i in range(N)]}


def _add_two(t1, t2, thresh):
    """nonorth_add(t1, t2) (src/hosvd.jl:83-156, 297)."""
    ts = sorted([t1, t2], key=lambda t: -np.sqrt(sum(float(np.sum(c * c)) for c in t["core"])))
    N = len(ts[0]["factors"])
    R = len(ts[0]["core"])
    nf = []
    for i in range(N):
        U, S, _ = np.linalg.svd(np.hstack([t["factors"][i] for t in ts]), full_matrices=False)
        nf.append(U[:, :int(np.sum(S > thresh))])
    core = [np.zeros(tuple(f.shape[1] for f in nf)) for _ in range(R)]
    for t in ts:
        tr = [nf[i].T @ t["factors"][i] for i in range(N)]
        for r in range(R):
            core[r] = core[r] + _transform(t["core"][r], tr, trans=True)
    return {"core": core, "factors": nf}


def project_out(v, w):
    """project_out!(v, w) (src/tucker_outer.jl:1511-1538), block by block."""
    if not w:
        return v
    Rw = len(next(iter(w.values()))["core"])
    for rw in range(Rw):
        for key in list(v.keys()):
            if key not in w:
                continue
            wt = w[key]
            ww = float(np.sum(wt["core"][rw] * wt["core"][rw]))
            for rv in range(len(v[key]["core"])):
                t = v[key]
                ov = [t["factors"][f].T @ wt["factors"][f] for f in range(len(t["factors"]))]
                ovlp = float(np.sum(_transform(t["core"][rv], ov) * wt["core"][rw])) / ww
                v[key] = _add_two(t, {"core": [c * (-ovlp) for c in wt["core"]], "factors": wt["factors"]}, 1e-16)
    return v


def compress_state(vec, thresh, only=None):
    """compress(ts::BSTstate) (src/type_BSTstate.jl:260-281): empty blocks dropped.  With `only`,
    the other blocks are kept as they are: for a state that is already a fixed point of compress
    (the output of compress_iteratively) compressing them again changes nothing but a rotation
    of their factors."""
    out = {}
    for k, t in vec.items():
        tt = compress_block(t, thresh) if only is None or k in only else t
        if _len(tt) > 0:
            out[k] = tt
    return out


def _vector(vec, R):
    return np.column_stack([np.concatenate([t["core"][r].reshape(-1, order="F") for t in vec.values()])
                            for r in range(R)]) if vec else np.zeros((0, R))


def _set_vector(vec, x, r):
    o = 0
    for t in vec.values():
        n = t["core"][r].size
        t["core"][r] = x[o:o + n].reshape(t["core"][r].shape, order="F").copy()
        o += n


def _zero(vec, R):
    return {k: {"core": [np.zeros(tuple(f.shape[1] for f in t["factors"])) for _ in range(R)], "factors": t["factors"]}
            for k, t in vec.items()}


# ---- device driver ------------------------------------------------------------------------------
class JointSigma:
    """H applied on the device to vectors over [reference blocks; FOIS blocks]: one
    fcg_bst_set of the joined structure, then fcg_bst_sigma per product."""

    def __init__(self, g: GpuSigma, ref, fois, R, nbody=4, between=False):
        self.g = g
        self.N = g.N
        self.R = R
        self.ref_keys = list(ref.keys())
        self.fois_keys = list(fois.keys())
        entries = [(k, ref[k]) for k in self.ref_keys] + [(k, fois[k]) for k in self.fois_keys]
        self.fock, self.blocks, self.foff, self.fac, _, offs = pack_blocks(entries, self.N, 1)
        self.n_ref = len(self.ref_keys)
        if between and fois:  # only <FOIS|H|ref> and <ref|H|FOIS>
            g.bst_set_between_raw(self.n_ref, self.fock, self.blocks, self.foff, self.fac, nbody)
        else:
            g.bst_set_raw(self.fock, self.blocks, self.foff, self.fac, nbody)
        self.offs = offs
        self.lens = [int(np.prod(self.blocks[i, :self.N])) for i in range(len(entries))]
        self.total = sum(self.lens)
        self.ref_len = sum(self.lens[:self.n_ref])

    def apply(self, x_ref, x_fois):
        """x_ref (ref_len, R), x_fois (fois_len, R) -> (H x)_ref, (H x)_fois."""
        R = x_ref.shape[1] if x_ref is not None else x_fois.shape[1]
        cin = np.zeros((R, self.total))
        if x_ref is not None:
            cin[:, :self.ref_len] = x_ref.T
        if x_fois is not None:
            cin[:, self.ref_len:] = x_fois.T
        out = self.g.bst_sigma(cin, "fp64")
        return out[:, :self.ref_len].T.copy(), out[:, self.ref_len:].T.copy()


class GpuBSTFois:
    """The FOIS builder and FOIS-PT2 on one GPU: H and H0 = Hcmf contexts over the same ops."""

    def __init__(self, ops, bases, ham, device: int = 0):
        self.N = ham.n_clusters
        po = pack.pack_ops(ops, bases)
        self.nmax = int(np.max(po.cluster_norb))
        self.H = GpuSigma(device)
        self.H.set_ops(po)
        self.H.set_terms(pack.pack_terms(ham))
        self.H0 = GpuSigma(device)
        self.H0.set_ops(po)
        self.H0.set_terms(pack.pack_terms(extract_1body_operator(ham, "Hcmf")))

    def close(self):
        self.H.close()
        self.H0.close()

    def fois(self, vec, P, Q, thresh=1e-7, nbody=4, compress_twice=True):
        """build_compressed_1st_order_state(vec; thresh, nbody, compress_twice) on the device."""
        R = len(next(iter(vec.values()))["core"])
        entries = list(vec.items())
        fock, blocks, foff, fac, cores, _ = pack_blocks(entries, self.N, R)
        sp = spaces_array(P, Q, self.N, self.nmax)
        of, ob, oo, ofa, oc = self.H.bst_fois(fock, blocks, foff, fac, cores, sp, thresh, nbody, compress_twice)
        return unpack_blocks(of, ob, oo, ofa, oc, self.N, R)

    def ci_solve(self, vec, R):
        """The lowest R eigenpairs of H over a small BST space (ci_solve, src/tucker_outer.jl:68-190),
        from its dense matrix built with device sigma builds of unit vectors."""
        J = JointSigma(self.H, vec, {}, 1)
        n = J.ref_len
        H = np.zeros((n, n))
        for j0 in range(0, n, 64):
            E = np.zeros((n, min(64, n - j0)))
            for q in range(E.shape[1]):
                E[j0 + q, q] = 1.0
            H[:, j0:j0 + E.shape[1]] = J.apply(E, None)[0]
        w, V = np.linalg.eigh(0.5 * (H + H.T))
        out = _zero(vec, R)
        for r in range(R):
            _set_vector(out, V[:, r], r)
        return w[:R], out

    def hylleraas(self, fois, ref, R, tol=1e-6, max_iter=100):
        """hylleraas_compressed_mp2 (src/tucker_pt.jl:358-532) with H0 = Hcmf: (psi1, e_pt2)."""
        c0 = _vector(ref, R)
        href = JointSigma(self.H, ref, {}, R).apply(c0, None)[0]
        JH = JointSigma(self.H, ref, fois, R, between=True)
        JF = JointSigma(self.H0, ref, fois, R)
        _, hx0 = JH.apply(c0, None)
        fref, fx0 = JF.apply(c0, None)
        e_ref = np.einsum("ir,ir->r", href, c0)
        e0 = np.einsum("ir,ir->r", fref, c0)
        Sx = _zero(fois, R)
        for key, t in Sx.items():
            if key in ref:
                rt = ref[key]
                ov = [rt["factors"][i].T @ t["factors"][i] for i in range(self.N)]
                for r in range(R):
                    t["core"][r] = _transform(rt["core"][r], ov)
        sxv = _vector(Sx, R)
        b = -hx0 + fx0

        def matvec(x):
            return JF.apply(None, x[:, None])[1][:, 0] - e0[0] * x

        X = np.zeros_like(b)
        self.cg_info = []  # per root: (products, converged, final residual norm)
        for r in range(R):
            X[:, r], info = _cg(matvec, b[:, r] + sxv[:, r] * (e_ref[r] - e0[r]), abstol=tol, maxiter=max_iter)
            self.cg_info.append(info)
        psi1 = _zero(fois, R)
        for r in range(R):
            _set_vector(psi1, X[:, r], r)
        SxC = np.einsum("ir,ir->r", sxv, X)
        ecorr = np.einsum("ir,ir->r", JH.apply(None, X)[0], c0)
        return psi1, (e_ref + ecorr) / (1.0 + SxC)

    def do_fois_pt2(self, ref, P, Q, thresh_foi=1e-6, nbody=4, tol=1e-6, max_iter=100):
        """do_fois_pt2 (src/tucker_pt.jl:551-605): zeroth-order solve in the reference space, the
        compressed FOIS, the reference projected out, compression, the Hylleraas functional.
        Returns (e_pt2, psi1)."""
        R = len(next(iter(ref.values()))["core"])
        _, ref_vec = self.ci_solve(ref, R)
        pt1 = self.fois(ref_vec, P, Q, thresh=thresh_foi, nbody=nbody)
        project_out(pt1, ref)
        pt1 = compress_state(pt1, thresh_foi, only=set(ref))
        psi1, e = self.hylleraas(pt1, ref_vec, R, tol=tol, max_iter=max_iter)
        return e, psi1


def _cg(matvec, b, abstol=1e-6, maxiter=100):
    """IterativeSolvers.cg! from x = 0: stop when |r| <= max(sqrt(eps) |b|, abstol) or after
    maxiter products.  Returns (x, (products, converged, residual norm)); like the reference it
    returns the last iterate when maxiter is reached (H0 - E0 need not be positive definite)."""
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
    return x, (it, bool(res <= tol), res)
