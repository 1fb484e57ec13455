"""Independent determinant-FCI check -- TEST INFRASTRUCTURE ONLY.

Full-space determinant Hamiltonian of n orbitals / (na, nb) electrons built
from sparse spin-summed excitation operators E_pq = sum_s p+_s q_s:
    H = sum_pq h_pq E_pq + 1/2 sum_pqrs (pr|qs) (E_pr E_qs - delta_qr E_ps)
This is the quantity the reference checks TPS spaces against (full-space TPS
eigenvalues equal FCI eigenvalues; test/test_schmidt.jl, test/test_FCI.jl).
It shares no code with the package's local-cluster FCI.
"""
from __future__ import annotations

from itertools import combinations

import numpy as np
import scipy.sparse as sps
import scipy.sparse.linalg as spla


def _strings(n, k):
    return [sum(1 << p for p in c) for c in combinations(range(n), k)]


def excitation_ops(n, na, nb):
    sa, sb = _strings(n, na), _strings(n, nb)
    ia = {s: i for i, s in enumerate(sa)}
    ib = {s: i for i, s in enumerate(sb)}
    nsb = len(sb)
    dim = len(sa) * nsb
    E = {}
    for p in range(n):
        for q in range(n):
            rows, cols, vals = [], [], []
            for spin in (0, 1):
                strs, idx = (sa, ia) if spin == 0 else (sb, ib)
                for si, s in enumerate(strs):
                    if not (s >> q) & 1:
                        continue
                    t = s ^ (1 << q)
                    sg = (-1) ** bin(t & ((1 << q) - 1)).count("1")
                    if (t >> p) & 1:
                        continue
                    sg *= (-1) ** bin(t & ((1 << p) - 1)).count("1")
                    t2 = t | (1 << p)
                    ti = idx[t2]
                    # the other spin's string is a spectator; alpha ops commute past
                    # nothing, beta ops pass all alpha electrons twice (even) -> no sign
                    if spin == 0:
                        for j in range(nsb):
                            rows.append(ti * nsb + j)
                            cols.append(si * nsb + j)
                            vals.append(sg)
                    else:
                        for j in range(len(sa)):
                            rows.append(j * nsb + ti)
                            cols.append(j * nsb + si)
                            vals.append(sg)
            E[(p, q)] = sps.csr_matrix((vals, (rows, cols)), shape=(dim, dim))
    return E, dim


def fci_hamiltonian(h1, h2, na, nb):
    n = h1.shape[0]
    E, dim = excitation_ops(n, na, nb)
    H = sps.csr_matrix((dim, dim))
    for p in range(n):
        for q in range(n):
            if h1[p, q] != 0.0:
                H = H + h1[p, q] * E[(p, q)]
    k = np.einsum("pqqs->ps", h2)
    for p in range(n):
        for s in range(n):
            H = H - 0.5 * k[p, s] * E[(p, s)]
    for p in range(n):
        for r in range(n):
            W = sps.csr_matrix((dim, dim))
            for q in range(n):
                for s in range(n):
                    if h2[p, r, q, s] != 0.0:
                        W = W + h2[p, r, q, s] * E[(q, s)]
            H = H + 0.5 * (E[(p, r)] @ W)
    return H


def fci_energies(h1, h2, na, nb, k=6):
    H = fci_hamiltonian(h1, h2, na, nb)
    if H.shape[0] <= 2000:
        return np.linalg.eigvalsh(H.toarray())[:k]
    w = spla.eigsh(H, k=k, which="SA", tol=1e-12)[0]
    return np.sort(w)
