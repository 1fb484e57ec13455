"""CPU oracle: pinned against determinant FCI and internal identities (no GPU)."""
import numpy as np

import oracle
from oracle.fci import fci_energies
from fermicg_gb300 import pack, workloads
from helpers import small_full, packed


def _dense_H(O, st):
    f, c, _, _ = pack.pack_state(st)
    n = len(st)
    return O.sigma_closed(f, c, np.eye(n)), f, c


def test_full_space_tps_equals_fci_4_clusters():
    prob, st = small_full()
    O = oracle.Oracle(*packed(prob))
    H, f, c = _dense_H(O, st)
    assert np.abs(H - H.T).max() < 1e-12
    e = np.linalg.eigvalsh(H)[:6]
    ef = fci_energies(prob.ints.h1, prob.ints.h2, 4, 4, k=6)
    assert np.abs(e - ef).max() < 1e-10


def test_full_space_tps_equals_fci_uneven_clusters():
    prob = workloads.build_problem(7, [3, 2, 2], [(2, 1), (1, 1), (1, 1)], 6, 11, max_roots=1000, cmf=False)
    st = workloads.full_space(prob)
    O = oracle.Oracle(*packed(prob))
    H, f, c = _dense_H(O, st)
    e = np.linalg.eigvalsh(H)[:5]
    ef = fci_energies(prob.ints.h1, prob.ints.h2, 4, 3, k=5)
    assert np.abs(e - ef).max() < 1e-10


def test_diagonal_and_open_sigma_identities():
    prob, st = small_full()
    O = oracle.Oracle(*packed(prob))
    H, f, c = _dense_H(O, st)
    assert np.abs(O.diagonal_H(f, c) - np.diag(H)).max() < 1e-13
    x = np.random.default_rng(5).standard_normal((len(st), 2))
    of, oc, ov = O.sigma_open(f, c, x, 0.0)
    d = {(of[i].tobytes(), oc[i].tobytes()): ov[i] for i in range(len(of))}
    ref = H @ x
    for i in range(len(st)):
        np.testing.assert_allclose(d[(f[i].tobytes(), c[i].tobytes())], ref[i], atol=1e-12)
