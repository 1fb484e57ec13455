"""BST oracle (build_sigma!) against the pinned TPS sigma: a block-sparse Tucker vector is
a compressed TPS vector, so H applied to it must equal the TPS H applied to the expanded
vector, projected back onto the bra Tucker bases."""
import itertools

import numpy as np

import oracle
from oracle import bst
from fermicg_gb300 import pack, workloads
from fermicg_gb300.state import TPSCIstate
from helpers import packed


def _problem():
    return workloads.build_problem(6, [2, 2, 2], [(1, 1), (1, 1), (1, 0)], 6, 5, max_roots=1000, cmf=False)


def _expand(prob, vec, N, R):
    """BST vector -> TPS coefficients over the full product space of every block."""
    st = TPSCIstate(N, R)
    for (fock, tcfg), blk in vec.items():
        dims = [tcfg[c][1] - tcfg[c][0] for c in range(N)]
        for r in range(R):
            full = blk["core"][r]
            for c in range(N):  # mode product with the factor: ranks -> local states in range
                full = np.moveaxis(np.tensordot(blk["factors"][c], full, axes=([1], [c])), 0, c)
            for idx in itertools.product(*[range(d) for d in dims]):
                cfg = tuple(tcfg[c][0] + idx[c] for c in range(N))
                key = (fock, cfg)
                if fock not in st.data or cfg not in st.data[fock]:
                    st[key] = np.zeros(R)
                st.data[fock][cfg][r] += full[idx]
    return st




def _random_vec(prob, N, R, rank_cut, seed, split):
    rng = np.random.default_rng(seed)
    na = sum(f[0] for f in prob.init_fspace)
    nb = sum(f[1] for f in prob.init_fspace)
    secs = [sorted(b.basis) for b in prob.bases]
    vec = {}
    for fs in itertools.product(*secs):
        if sum(f[0] for f in fs) != na or sum(f[1] for f in fs) != nb:
            continue
        Ms = [prob.bases[c].basis[fs[c]].shape[1] for c in range(N)]
        ranges_per_c = []
        for M in Ms:
            rs = [(0, M)] if (not split or M < 2) else [(0, 1), (1, M)]
            ranges_per_c.append(rs)
        for tcfg in itertools.product(*ranges_per_c):
            factors, shape = [], []
            for c in range(N):
                L = tcfg[c][1] - tcfg[c][0]
                rk = max(1, min(L, L - rank_cut)) if L > 1 else 1
                Q, _ = np.linalg.qr(rng.standard_normal((L, L)))
                factors.append(Q[:, :rk].copy())
                shape.append(rk)
            core = [rng.standard_normal(shape) for _ in range(R)]
            vec[(fs, tcfg)] = {"core": core, "factors": factors}
    return vec


def _check(prob, vec, N, R):
    po, pt = packed(prob)
    O = oracle.Oracle(po, pt)
    tps = _expand(prob, vec, N, R)
    f, c, v, _ = pack.pack_state(tps)
    hv = O.sigma_closed(f, c, v)
    rows = {(tuple(map(tuple, f[i])), tuple(c[i])): hv[i] for i in range(len(f))}
    sig = bst.build_sigma(bst.zero_like(vec, R), vec, prob.ops, prob.ham, N, R)
    err, scale = 0.0, 0.0
    for (fock, tcfg), blk in sig.items():
        dims = [tcfg[cc][1] - tcfg[cc][0] for cc in range(N)]
        for r in range(R):
            full = np.zeros(dims)
            for idx in itertools.product(*[range(d) for d in dims]):
                cfg = tuple(tcfg[cc][0] + idx[cc] for cc in range(N))
                full[idx] = rows[(fock, cfg)][r]
            proj = full
            for cc in range(N):  # bra-basis projection: U^T along every mode
                proj = np.moveaxis(np.tensordot(blk["factors"][cc].T, proj, axes=([1], [cc])), 0, cc)
            err = max(err, float(np.abs(proj - blk["core"][r]).max()))
            scale = max(scale, float(np.abs(proj).max()))
    return err, scale


def test_bst_sigma_full_rank_equals_tps_sigma():
    prob = _problem()
    vec = _random_vec(prob, 3, 2, rank_cut=0, seed=1, split=False)
    err, scale = _check(prob, vec, 3, 2)
    assert err < 1e-11 * scale


def test_bst_sigma_split_truncated_blocks_equals_projected_tps_sigma():
    """P/Q-split TuckerConfigs with truncated ranks: build_sigma! must equal the projection
    of H on the expanded vector when the block spaces do not overlap (they don't: ranges
    partition each sector)."""
    prob = _problem()
    vec = _random_vec(prob, 3, 2, rank_cut=1, seed=2, split=True)
    err, scale = _check(prob, vec, 3, 2)
    assert err < 1e-11 * scale


def test_bst_sigma_four_clusters_with_4body_terms():
    prob = workloads.build_problem(6, [2, 1, 2, 1], [(1, 1), (1, 0), (1, 1), (0, 1)], 6, 7, max_roots=1000,
                                   cmf=False)
    assert any(t.nbody == 4 for tr, ts in prob.ham for t in ts)
    vec = _random_vec(prob, 4, 1, rank_cut=1, seed=3, split=True)
    err, scale = _check(prob, vec, 4, 1)
    assert err < 1e-11 * scale
