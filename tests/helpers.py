"""Shared problem builders for the tests (small, seeded)."""
import functools

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
