"""Clustered Hamiltonian structure vs the reference's term table."""
import pytest

from fermicg_gb300 import workloads
from fermicg_gb300.integrals import synthetic_integrals
from fermicg_gb300.terms import extract_ClusteredTerms


@pytest.mark.parametrize("nc,total,n1,n2,n3,n4,ntr", [
    (4, 472, 4, 192, 240, 36, 253),
    (6, 2226, 6, 480, 1200, 540, 1441),
])
def test_term_counts(nc, total, n1, n2, n3, n4, ntr):
    ints = synthetic_integrals(2 * nc, 4, 0)
    H = extract_ClusteredTerms(ints, workloads.consecutive_clusters(2 * nc, [2] * nc))
    counts = {1: 0, 2: 0, 3: 0, 4: 0}
    for tr, terms in H:
        for t in terms:
            counts[t.nbody] += 1
    assert H.n_terms() == total
    assert (counts[1], counts[2], counts[3], counts[4]) == (n1, n2, n3, n4)
    assert len(H) == ntr


def test_term_parity_and_transfer_consistency():
    ints = synthetic_integrals(8, 4, 1)
    H = extract_ClusteredTerms(ints, workloads.consecutive_clusters(8, [2] * 4))
    for tr, terms in H:
        for t in terms:
            for o, d, p, c in zip(t.ops, t.delta, t.parity, t.clusters):
                if o != "H":
                    assert p == len(o) % 2
                assert tr[c] == d
