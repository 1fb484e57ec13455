"""Seeded synthetic problems shaped like the benchmark configurations.

A problem is: integrals -> consecutive clusters -> local eigenbases (M lowest
per Fock sector) -> cluster operators (TDMs) -> clustered Hamiltonian ->
a variational TPS space.

The variational space stands in for a converged TPSCI selection: it is the
set of the `n_cfg` lowest configurations by the sum of local energies
(sum_c e_c(sector_c, state_c)) over all global Fock sectors with the right
electron count (a deterministic, energy-ordered product space).  Sectors
are inserted in order of their lowest configuration, configurations within a
sector in increasing energy.
"""
from __future__ import annotations

import heapq
import itertools
from dataclasses import dataclass, field

import numpy as np

from .integrals import InCoreInts, synthetic_integrals
from .local_fci import compute_cluster_eigenbasis, compute_cluster_ops, add_cmf_operators
from .state import TPSCIstate
from .terms import extract_ClusteredTerms


@dataclass
class Problem:
    ints: InCoreInts
    clusters: list
    init_fspace: list
    bases: list
    ops: list
    ham: object
    meta: dict = field(default_factory=dict)


def consecutive_clusters(norb, sizes):
    out, p = [], 0
    for s in sizes:
        out.append(list(range(p, p + s)))
        p += s
    assert p == norb
    return out


def build_problem(norb, cluster_sizes, init_fspace, n_chol, seed, max_roots, delta_elec=None,
                  cmf=True):
    """Integrals, bases, TDMs and clustered H for one synthetic system."""
    ints = synthetic_integrals(norb, n_chol, seed)
    clusters = consecutive_clusters(norb, cluster_sizes)
    bases = compute_cluster_eigenbasis(ints, clusters, init_fspace=init_fspace,
                                       delta_elec=delta_elec, max_roots=max_roots)
    ops = compute_cluster_ops(bases, ints)
    if cmf:
        da, db = reference_density(bases, clusters, init_fspace, norb)
        add_cmf_operators(ops, bases, ints, da, db)
    ham = extract_ClusteredTerms(ints, clusters)
    return Problem(ints, clusters, list(init_fspace), bases, ops, ham,
                   dict(norb=norb, cluster_sizes=list(cluster_sizes), n_chol=n_chol, seed=seed,
                        max_roots=max_roots, delta_elec=delta_elec))


def reference_density(bases, clusters, init_fspace, norb):
    """Block-diagonal alpha/beta 1-RDMs of the product of local ground states
    in the reference sectors (the mean field a CMF embedding uses)."""
    da = np.zeros((norb, norb))
    db = np.zeros((norb, norb))
    for cb, orbs, f in zip(bases, clusters, init_fspace):
        sp = cb.space
        v = cb.basis[tuple(f)][:, 0]
        for spin, d in ((0, da), (1, db)):
            r = sp.op_matrices("Aa" if spin == 0 else "Bb", *f)
            if r is None:
                continue
            g = np.einsum("i,pqij,j->pq", v, r[1], v)
            d[np.ix_(orbs, orbs)] = g
    return da, db


def _local_energy_tables(bases):
    return [{sec: np.asarray(e) for sec, e in cb.energies.items()} for cb in bases]


def energy_ordered_space(prob: Problem, n_cfg: int, R: int = 1, seed: int = 0):
    """The n_cfg lowest configurations by summed local energy (see module doc).

    Coefficients are seeded N(0,1), rows normalised per root."""
    N = len(prob.clusters)
    na_tot = sum(f[0] for f in prob.init_fspace)
    nb_tot = sum(f[1] for f in prob.init_fspace)
    et = _local_energy_tables(prob.bases)
    # global sectors with the right electron count, enumerated by branch and bound on their
    # lowest configuration energy: only sectors below a cutoff are visited, and the cutoff
    # grows until n_cfg configurations lie below it (then no excluded sector can hold one
    # of the n_cfg lowest configurations)
    secs = [sorted(b.basis.keys()) for b in prob.bases]
    lo_a = [0] * (N + 1)
    hi_a = [0] * (N + 1)
    lo_b = [0] * (N + 1)
    hi_b = [0] * (N + 1)
    emin = [0.0] * (N + 1)
    for c in range(N - 1, -1, -1):
        lo_a[c] = lo_a[c + 1] + min(s[0] for s in secs[c])
        hi_a[c] = hi_a[c + 1] + max(s[0] for s in secs[c])
        lo_b[c] = lo_b[c + 1] + min(s[1] for s in secs[c])
        hi_b[c] = hi_b[c + 1] + max(s[1] for s in secs[c])
        emin[c] = emin[c + 1] + min(float(et[c][s][0]) for s in secs[c])

    def sectors_below(ecut):
        out = []

        def rec(c, cur, na, nb, e):
            if e + emin[c] > ecut:
                return
            if c == N:
                if na == na_tot and nb == nb_tot:
                    out.append(tuple(cur))
                return
            if not (lo_a[c] <= na_tot - na <= hi_a[c] and lo_b[c] <= nb_tot - nb <= hi_b[c]):
                return
            for s in secs[c]:
                cur.append(s)
                rec(c + 1, cur, na + s[0], nb + s[1], e + float(et[c][s][0]))
                cur.pop()

        rec(0, [], 0, 0, 0.0)
        return out

    def k_best(gsecs, ecut):
        heap = []
        gens = []
        for gi, fs in enumerate(gsecs):
            es = [et[c][fs[c]] for c in range(N)]
            gens.append((fs, es))
            heap.append((sum(float(e[0]) for e in es), gi, (0,) * N))
        heapq.heapify(heap)
        seen = set((gi, (0,) * N) for gi in range(len(gsecs)))
        chosen = []
        while heap and len(chosen) < n_cfg:
            e, gi, st = heapq.heappop(heap)
            if e > ecut:
                break
            chosen.append((e, gi, st))
            fs, es = gens[gi]
            for c in range(N):
                if st[c] + 1 < len(es[c]):
                    nst = st[:c] + (st[c] + 1,) + st[c + 1:]
                    if (gi, nst) in seen:
                        continue
                    seen.add((gi, nst))
                    ne = e - float(es[c][st[c]]) + float(es[c][st[c] + 1])
                    heapq.heappush(heap, (ne, gi, nst))
        return chosen

    e_floor = emin[0]
    width = 1.0
    while True:
        ecut = e_floor + width
        gsecs = sectors_below(ecut)
        chosen = k_best(gsecs, ecut)
        if len(chosen) >= n_cfg or width > 1e6:
            break
        width *= 2.0
    # group by sector; sector order = order of first appearance
    order = []
    by = {}
    for e, gi, st in chosen:
        if gi not in by:
            by[gi] = []
            order.append(gi)
        by[gi].append(st)
    rng = np.random.default_rng(seed)
    state = TPSCIstate(N, R)
    coeffs = rng.standard_normal((len(chosen), R))
    coeffs /= np.linalg.norm(coeffs, axis=0, keepdims=True)
    i = 0
    for gi in order:
        fs = gsecs[gi]
        state.add_fockconfig(fs)
        for st in by[gi]:
            state.data[fs][st] = coeffs[i].copy()
            i += 1
    return state


def full_space(prob: Problem, R: int = 1, seed: int = 0):
    """Every configuration of the right electron count (full TPS space)."""
    N = len(prob.clusters)
    na_tot = sum(f[0] for f in prob.init_fspace)
    nb_tot = sum(f[1] for f in prob.init_fspace)
    secs = [sorted(b.basis.keys()) for b in prob.bases]
    state = TPSCIstate(N, R)
    for fs in itertools.product(*secs):
        if sum(f[0] for f in fs) != na_tot or sum(f[1] for f in fs) != nb_tot:
            continue
        dims = [prob.bases[c].basis[fs[c]].shape[1] for c in range(N)]
        state.add_fockconfig(fs)
        for st in itertools.product(*[range(d) for d in dims]):
            state.data[fs][st] = np.zeros(R)
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((len(state), R))
    v /= np.linalg.norm(v, axis=0, keepdims=True)
    state.set_vector(v)
    return state


# ---- named workloads -------------------------------------------------------------

def config0_problem(seed=0):
    """12 orbitals, 6a/6b, 4 clusters x 3, K=36, full local FCI per sector."""
    return build_problem(12, [3, 3, 3, 3], [(2, 1), (1, 2), (2, 1), (1, 2)], 36, seed,
                         max_roots=1000)


def config1_problem(seed=0):
    """24 orbitals, 12a/12b, 6 clusters x 4, K=72, M=16 per sector within 2 electrons
    of (2,2)."""
    return build_problem(24, [4] * 6, [(2, 2)] * 6, 72, seed, max_roots=16, delta_elec=2)


def config2_problem(seed=0):
    """32 orbitals, 16a/16b, 8 clusters x 4, K=96, M=16 per sector within 1 electron of
    (2,2) (the BST / Tucker configuration)."""
    return build_problem(32, [4] * 8, [(2, 2)] * 8, 96, seed, max_roots=16, delta_elec=1)


def single_transfer_sectors(prob):
    """The reference Fock sector and every sector reached from it by moving one alpha or
    one beta electron between two clusters (the charge-transfer blocks of a BST vector)."""
    ref = tuple(tuple(f) for f in prob.init_fspace)
    N = len(ref)
    out = [ref]
    for i in range(N):
        for j in range(N):
            if i == j:
                continue
            for s in (0, 1):
                fs = [list(f) for f in ref]
                fs[i][s] -= 1
                fs[j][s] += 1
                if fs[i][s] < 0 or fs[j][s] > len(prob.clusters[j]):
                    continue
                key = tuple(tuple(f) for f in fs)
                if all(key[c] in prob.bases[c].basis for c in range(N)):
                    out.append(key)
    return out


def config3_instance(i, base_seed=3000, max_cluster=5, n_cfg_range=(1000, 4000)):
    """Instance i of the batched-uneven workload: seed base_seed + i; orbitals drawn from
    {8, 12, 16, 20}, 2-5 clusters of 2..max_cluster consecutive orbitals, half filling
    spread over the clusters, M = 8-16 local states per sector (sectors within one electron
    of the reference), 1-3 roots, an energy-ordered space of n_cfg_range configurations.
    Returns (problem, state)."""
    rng = np.random.default_rng(base_seed + i)
    while True:
        norb = int(rng.choice([8, 12, 16, 20]))
        nc = int(rng.integers(2, 6))
        sizes = [int(x) for x in rng.integers(2, max_cluster + 1, size=nc)]
        if sum(sizes) == norb:
            break
    na = norb // 2
    alpha = [s // 2 for s in sizes]
    c = 0
    while sum(alpha) < na:
        if alpha[c % nc] < sizes[c % nc]:
            alpha[c % nc] += 1
        c += 1
    fspace = [(a, a) for a in alpha]
    M = int(rng.integers(8, 17))
    R = int(rng.integers(1, 4))
    prob = build_problem(norb, sizes, fspace, 2 * norb, base_seed + i, max_roots=M, delta_elec=1)
    n_cfg = int(rng.integers(n_cfg_range[0], n_cfg_range[1] + 1))
    st = energy_ordered_space(prob, n_cfg, R=R, seed=base_seed + i)
    return prob, st


def config3_packed(i, base_seed=3000, max_cluster=5, n_cfg_range=(1000, 4000)):
    """config3_instance i in the form the C ABI takes: (PackedOps, PackedTerms, fock, cfg,
    coefficients).  Small enough to return from a worker process."""
    from . import pack
    prob, st = config3_instance(i, base_seed, max_cluster, n_cfg_range)
    f, c, v, _ = pack.pack_state(st)
    return pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham), f, c, v


def config3_batch(n_inst, max_cluster=5, workers=None):
    """The first n_inst config-3 instances (config3_packed), built in parallel in worker
    processes started with spawn (safe after CUDA is initialised in the caller)."""
    import multiprocessing as mp
    import os
    from concurrent.futures import ProcessPoolExecutor
    workers = workers or min(16, os.cpu_count() or 1)
    if workers <= 1 or n_inst < 8:
        return [config3_packed(i, max_cluster=max_cluster) for i in range(n_inst)]
    # one BLAS thread per worker (the workers start with this environment)
    keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ[k] = "1"
    try:
        with ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
            return list(ex.map(config3_packed, range(n_inst), [3000] * n_inst, [max_cluster] * n_inst, chunksize=2))
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def davidson_guess(n, R, seed=0, lowest=None, spread=0.05):
    """Starting block for R roots of an n-configuration problem: unit vectors on the
    configurations `lowest` (default the first R, the lowest in an energy-ordered space; pass
    the indices of the R smallest diagonal elements of H otherwise), plus a seeded dense part
    of norm about `spread` per column.  The dense part gives the block a component in every
    symmetry sector of H: unit vectors alone leave Davidson in the sectors they start in, and
    floating-point rounding then decides whether the lowest root of another sector is found."""
    rng = np.random.default_rng(seed)
    g = (spread / np.sqrt(n)) * rng.standard_normal((n, R))
    idx = range(R) if lowest is None else lowest
    for r, k in enumerate(idx):
        g[int(k), r] += 1.0
    return g
