"""Block-sparse Tucker (BST) vectors and their sigma build on the GPU.

A BST vector (type_BSTstate.jl:13-18) is a map
    (fock tuple, tconfig) -> {"core": [R arrays (r_1..r_N)], "factors": [N matrices (len_c, r_c)]}
where tconfig holds one half-open range of local states per cluster (0-based; the
reference's TuckerConfig UnitRanges) and the factors are that block's Tucker bases.

build_sigma! (tucker_inner.jl:165-245) couples every bra block with every ket block
through every term that passes check_term on TuckerConfigs (spectators: equal Fock
sector and equal range; actives: fock_bra = fock_ket + delta).  The host plans that
triple list once per BST structure (`plan_triples`); the device builds the dense term
operators in the Tucker bases once (cache_hamiltonian, tucker_inner.jl:90-159) and then
applies them in every sigma build (form_sigma_block! + contract_dense_H_with_state).
"""
from __future__ import annotations

import itertools

import numpy as np

from . import pack
from .terms import compute_terms_state_sign


def synthetic_bst(prob, sectors, max_q=2, rank_range=(2, 6), R=1, seed=0):
    """A seeded BST vector: for each given global Fock sector, every TuckerConfig with at
    most `max_q` clusters in their excited range (local states 1..M-1; the others hold the
    lowest state, range 0..1), random orthonormal factors of rank in `rank_range`
    (capped by the range length) and N(0,1) cores."""
    rng = np.random.default_rng(seed)
    N = len(prob.clusters)
    vec = {}
    for fs in sectors:
        Ms = [prob.bases[c].basis[fs[c]].shape[1] for c in range(N)]
        qable = [c for c in range(N) if Ms[c] > 1]
        for nq in range(0, max_q + 1):
            for qset in itertools.combinations(qable, nq):
                tcfg, factors, shape = [], [], []
                for c in range(N):
                    rng_c = (1, Ms[c]) if c in qset else (0, 1)
                    L = rng_c[1] - rng_c[0]
                    rk = 1 if L == 1 else int(min(L, rng.integers(rank_range[0], rank_range[1] + 1)))
                    Q, _ = np.linalg.qr(rng.standard_normal((L, L)))
                    tcfg.append(rng_c)
                    factors.append(np.ascontiguousarray(Q[:, :rk]))
                    shape.append(rk)
                cores = [rng.standard_normal(shape) for _ in range(R)]
                vec[(tuple(fs), tuple(tcfg))] = {"core": cores, "factors": factors}
    return vec


class PackedBST:
    """Flat form of a BST vector.

    blocks: int64 [n_blocks][5 + 3N] = {core_off, core_len, fock_sector_id, pad, pad,
            ranks[N], range_start[N], range_len[N]}
    factor_off: int64 [n_blocks][N] offsets of each (range_len x rank) factor, column-major
    cores: float64 [R][core_total] with each block's core column-major (cluster 0 fastest)
    """

    def __init__(self, vec, N, R):
        self.keys = list(vec.keys())
        self.N, self.R = N, R
        rows, foffs, fchunks, coffs = [], [], [], []
        core_off = 0
        f_off = 0
        for key in self.keys:
            blk = vec[key]
            fs, tcfg = key
            ranks = [f.shape[1] for f in blk["factors"]]
            clen = int(np.prod(ranks))
            rows.append([core_off, clen, 0, 0, 0] + ranks + [t[0] for t in tcfg] + [t[1] - t[0] for t in tcfg])
            offs = []
            for f in blk["factors"]:
                offs.append(f_off)
                fchunks.append(np.asarray(f, dtype=np.float64).reshape(-1, order="F"))
                f_off += f.size
            foffs.append(offs)
            coffs.append(core_off)
            core_off += clen
        self.blocks = np.array(rows, dtype=np.int64).reshape(-1, 5 + 3 * N)
        self.factor_off = np.array(foffs, dtype=np.int64).reshape(-1, N)
        self.factors = np.concatenate(fchunks) if fchunks else np.zeros(0)
        self.core_total = core_off
        self.index = {k: i for i, k in enumerate(self.keys)}

    def cores_of(self, vec):
        """(R, core_total) float64 with each block's cores column-major."""
        out = np.zeros((self.R, self.core_total))
        for i, key in enumerate(self.keys):
            o, n = self.blocks[i, 0], self.blocks[i, 1]
            for r in range(self.R):
                out[r, o:o + n] = np.asarray(vec[key]["core"][r]).reshape(-1, order="F")
        return out

    def to_vec(self, vec, cores):
        """Cores (R, core_total) back into a BST dict with vec's factors."""
        out = {}
        for i, key in enumerate(self.keys):
            o, n = self.blocks[i, 0], self.blocks[i, 1]
            shape = tuple(int(x) for x in self.blocks[i, 5:5 + self.N])
            out[key] = {"core": [cores[r, o:o + n].reshape(shape, order="F") for r in range(self.R)],
                        "factors": vec[key]["factors"]}
        return out


def plan_triples(pb: PackedBST, ham, ops=None, nbody=4):
    """(bra block, ket block, term) triples of build_sigma! that pass check_term on
    TuckerConfigs, with the state sign of each (compute_terms_state_sign on the ket
    sector).  With `ops` (ClusterOps list), terms whose TDM block of an active cluster is
    absent for the sector pair are left out (build_dense_H_term has nothing to contract).
    Returns int32 [n][4] = {bra, ket, term index in pack_terms order, sign}."""
    N = pb.N
    term_index = {}
    ti = 0
    for tid, (tr, terms) in enumerate(ham):
        for t in terms:
            term_index[id(t)] = ti
            ti += 1
    by_fock = {}
    for i, (fs, tcfg) in enumerate(pb.keys):
        by_fock.setdefault(fs, []).append(i)
    # per (fock, active set): ket blocks grouped by their ranges on the spectator clusters
    groups = {}

    def group(fk, act):
        key = (fk, act)
        if key not in groups:
            d = {}
            for i in by_fock.get(fk, []):
                tcfg = pb.keys[i][1]
                d.setdefault(tuple(tcfg[c] if c not in act else None for c in range(N)), []).append(i)
            groups[key] = d
        return groups[key]

    out = []
    for fb, bras in by_fock.items():
        for tr, terms in ham:
            fk = tuple((fb[c][0] - tr[c][0], fb[c][1] - tr[c][1]) for c in range(N))
            if fk not in by_fock:
                continue
            for t in terms:
                if t.nbody > nbody:
                    continue
                if ops is not None and any((fb[c], fk[c]) not in ops[c].data.get(op, {})
                                           for c, op in zip(t.clusters, t.ops)):
                    continue
                act = frozenset(t.clusters)
                g = group(fk, act)
                sgn = compute_terms_state_sign(t, fk)
                for b in bras:
                    tb = pb.keys[b][1]
                    for k in g.get(tuple(tb[c] if c not in act else None for c in range(N)), []):
                        out.append((b, k, term_index[id(t)], 1 if t.nbody == 1 else sgn))
    return np.array(out, dtype=np.int32).reshape(-1, 4)


def hcmf_diagonal(pb: PackedBST, vec, ops, op="Hcmf"):
    """Preconditioner diagonal of a BST solve (one value per core element, the layout of one
    root of PackedBST.cores_of): sum over clusters of the diagonal of U_c^T Hcmf_c U_c for the
    block's factor U_c of the cluster's range.  The reference's ci_solve (precond=true,
    src/tucker_outer.jl:90-95) first rotates every block's factors so that the local Hcmf is
    diagonal and sums its eigenvalues; without the rotation this is the diagonal of the same
    operator in the unrotated Tucker basis."""
    N = pb.N
    out = np.zeros(pb.core_total)
    for i, key in enumerate(pb.keys):
        fs, tcfg = key
        o, n = int(pb.blocks[i, 0]), int(pb.blocks[i, 1])
        facs = vec[key]["factors"]
        d = np.zeros(n)
        shape = [f.shape[1] for f in facs]
        stride = 1
        for c in range(N):
            blocks = ops[c].data.get(op) or ops[c].data["H"]
            Hc = np.asarray(blocks[(fs[c], fs[c])])
            a, b = tcfg[c]
            U = facs[c]
            dc = np.einsum("ik,ij,jk->k", U, Hc[a:b, a:b], U)
            idx = (np.arange(n) // stride) % shape[c]
            d += dc[idx]
            stride *= shape[c]
        out[o:o + n] = d
    return out
