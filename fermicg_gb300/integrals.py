"""In-core integrals and the seeded synthetic Hamiltonian generator.

`InCoreInts` mirrors the container FermiCG receives from InCoreIntegrals
(`h0`, `h1[p,q]`, `h2[p,q,r,s] = (pq|rs)` in chemist order; used as such in
type_ClusteredOperator.jl:231 and build_local_quantities.jl:60).

Indices here are 0-based; the reference's orbital lists are 1-based.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class InCoreInts:
    h0: float
    h1: np.ndarray  # (n, n)
    h2: np.ndarray  # (n, n, n, n), (pq|rs)

    @property
    def n_orb(self) -> int:
        return self.h1.shape[0]


def synthetic_integrals(norb: int, n_chol: int, seed: int) -> InCoreInts:
    """Seeded synthetic Hamiltonian with a banded, PSD two-electron part.

    h_pq = -2 delta_pq + 0.3 exp(-|p-q|) N(0,1), symmetrised.
    L^K_pq = N(0,1) 0.4 exp(-0.5|p-q|), symmetrised; (pq|rs) = sum_K L^K_pq L^K_rs.
    The random stream is numpy's default_rng(seed): h first, then all L^K.
    """
    rng = np.random.default_rng(seed)
    idx = np.arange(norb)
    dist = np.abs(idx[:, None] - idx[None, :]).astype(np.float64)
    h = -2.0 * np.eye(norb) + 0.3 * np.exp(-dist) * rng.standard_normal((norb, norb))
    h = 0.5 * (h + h.T)
    L = rng.standard_normal((n_chol, norb, norb)) * (0.4 * np.exp(-0.5 * dist))[None]
    L = 0.5 * (L + L.transpose(0, 2, 1))
    h2 = np.einsum("kpq,krs->pqrs", L, L, optimize=True)
    return InCoreInts(0.0, np.ascontiguousarray(h), np.ascontiguousarray(h2))


def subset(ints: InCoreInts, orbs, rdm1a=None, rdm1b=None) -> InCoreInts:
    """Integrals restricted to the orbitals `orbs` (a cluster).

    Without densities this is the bare block (InCoreIntegrals.subset, called at
    build_local_quantities.jl:1110 and :60).  With densities the environment
    (all orbitals outside `orbs`) is folded in as a mean field, the embedding
    used for the CMF local Hamiltonian (build_local_quantities.jl:626, 1112):
        h_eff[p,q] = h[p,q] + sum_rs (pq|rs) D[r,s] - 1/2 sum_rs (ps|rq) D[r,s]
    with D = Da + Db restricted to the environment, and h0 the environment
    energy.  For Da == Db this is the exact closed-shell mean field.
    """
    orbs = np.asarray(orbs, dtype=np.int64)
    h1 = ints.h1[np.ix_(orbs, orbs)].copy()
    h2 = ints.h2[np.ix_(orbs, orbs, orbs, orbs)].copy()
    if rdm1a is None and rdm1b is None:
        return InCoreInts(0.0, h1, h2)
    da = np.array(rdm1a, dtype=np.float64, copy=True)
    db = np.array(rdm1b, dtype=np.float64, copy=True)
    for d in (da, db):
        d[orbs, :] = 0.0
        d[:, orbs] = 0.0
    dt = da + db
    j = np.einsum("pqrs,rs->pq", ints.h2[np.ix_(orbs, orbs)], dt)
    k = np.einsum("psrq,rs->pq", ints.h2[np.ix_(orbs, np.arange(ints.n_orb), np.arange(ints.n_orb), orbs)], dt)
    h1 = h1 + j - 0.5 * k
    # environment energy: sum h D + 1/2 sum (pq|rs) [D_pq D_rs - Da_ps Da_rq - Db_ps Db_rq]
    e_env = float(np.einsum("pq,pq", ints.h1, dt))
    e_env += 0.5 * float(np.einsum("pqrs,pq,rs", ints.h2, dt, dt))
    e_env -= 0.5 * float(np.einsum("pqrs,ps,rq", ints.h2, da, da))
    e_env -= 0.5 * float(np.einsum("pqrs,ps,rq", ints.h2, db, db))
    return InCoreInts(e_env, h1, h2)
