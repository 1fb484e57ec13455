"""BST oracle (build_sigma!) against the pinned TPS sigma: a block-sparse Tucker vector is
a compressed TPS vector, so H applied to it must equal the TPS H applied to the expanded
vector, projected back onto the bra Tucker bases."""
import itertools

import numpy as np

import oracle
from oracle import bst
from fermicg_gb300 import pack, workloads
from fermicg_gb300.state import TPSCIstate
from helpers import packed, random_bst


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
    vec = random_bst(prob, 3, 2, rank_cut=0, seed=1, split=False)
    err, scale = _check(prob, vec, 3, 2)
    assert err < 1e-11 * scale


def test_bst_sigma_split_truncated_blocks_equals_projected_tps_sigma():
    """P/Q-split TuckerConfigs with truncated ranks: build_sigma! must equal the projection
    of H on the expanded vector when the block spaces do not overlap (they don't: ranges
    partition each sector)."""
    prob = _problem()
    vec = random_bst(prob, 3, 2, rank_cut=1, seed=2, split=True)
    err, scale = _check(prob, vec, 3, 2)
    assert err < 1e-11 * scale


def test_bst_sigma_four_clusters_with_4body_terms():
    prob = workloads.build_problem(6, [2, 1, 2, 1], [(1, 1), (1, 0), (1, 1), (0, 1)], 6, 7, max_roots=1000,
                                   cmf=False)
    assert any(t.nbody == 4 for tr, ts in prob.ham for t in ts)
    vec = random_bst(prob, 4, 1, rank_cut=1, seed=3, split=True)
    err, scale = _check(prob, vec, 4, 1)
    assert err < 1e-11 * scale


def test_bst_planner_matches_check_term_enumeration():
    """plan_triples enumerates exactly the (bra, ket, term) triples that build_sigma!'s loops
    accept through check_term on TuckerConfigs and then contract (TDM blocks present)."""
    from fermicg_gb300.bst import PackedBST, plan_triples
    from fermicg_gb300.terms import compute_terms_state_sign
    prob = workloads.build_problem(6, [2, 1, 2, 1], [(1, 1), (1, 0), (1, 1), (0, 1)], 6, 7, max_roots=1000,
                                   cmf=False)
    N = 4
    vec = random_bst(prob, N, 1, rank_cut=1, seed=3, split=True)
    pb = PackedBST(vec, N, 1)
    got = {tuple(int(x) for x in r) for r in plan_triples(pb, prob.ham, ops=prob.ops)}
    tindex = {}
    for tr, terms in prob.ham:
        for t in terms:
            tindex[id(t)] = len(tindex)
    want = set()
    for b, (fb, tb) in enumerate(pb.keys):
        for k, (fk, tk) in enumerate(pb.keys):
            tr = tuple((fb[c][0] - fk[c][0], fb[c][1] - fk[c][1]) for c in range(N))
            for t in prob.ham.trans.get(tr, []):
                if not bst.check_term_tucker(t, fb, tb, fk, tk):
                    continue
                # the oracle's build_dense_H_term skips a term whose TDM block is absent
                if any((fb[c], fk[c]) not in prob.ops[c].data.get(op, {}) for c, op in zip(t.clusters, t.ops)):
                    continue
                sgn = 1 if t.nbody == 1 else compute_terms_state_sign(t, fk)
                want.add((b, k, tindex[id(t)], sgn))
    assert len(want) > 1000
    assert got == want
