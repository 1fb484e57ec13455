"""Shared problem builders for the tests (small, seeded)."""
import functools
import itertools

import numpy as np

from fermicg_gb300 import pack, workloads


@functools.lru_cache(maxsize=None)
def small_full(norb=8, sizes=(2, 2, 2, 2), fspace=((1, 1),) * 4, seed=3):
    """Full TPS space of a small system (equals determinant FCI)."""
    prob = workloads.build_problem(norb, list(sizes), list(fspace), 8, seed, max_roots=1000, cmf=True)
    st = workloads.full_space(prob, R=1)
    return prob, st


@functools.lru_cache(maxsize=None)
def config1_subspace(n_cfg=3000, R=4, seed=0):
    """Energy-ordered subspace of the 24-orbital / 6-cluster problem."""
    prob = workloads.config1_problem(seed)
    st = workloads.energy_ordered_space(prob, n_cfg, R=R, seed=seed)
    return prob, st


def packed(prob):
    return pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham)


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def random_bst(prob, N, R, rank_cut, seed, split):
    """Every Fock sector with the right electron count; one full-range TuckerConfig per
    sector, or (split) ranges {0} and {1..M-1} per cluster; random orthonormal factors of
    rank (range length - rank_cut), N(0,1) cores."""
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
