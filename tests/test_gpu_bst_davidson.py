"""The BST ci_solve Davidson on the device (fcg_bst_davidson): lowest eigenvalues of H over the
Tucker cores equal those of the dense projected H (assembled column by column from the device
BST sigma, itself checked against the oracle's build_sigma!), in FP64 and mixed precision,
with and without the Hcmf preconditioner; and BST requests in a serving stream end as they do
alone."""
import numpy as np
import pytest

from fermicg_gb300 import pack, workloads
from fermicg_gb300.bst import PackedBST, hcmf_diagonal, synthetic_bst
from fermicg_gb300.serving import NativeSolveServer, Request, SolveServer
from helpers import packed, random_bst

pytestmark = pytest.mark.gpu


def _problem():
    return workloads.build_problem(8, [2, 3, 3], [(1, 1), (1, 1), (2, 1)], 9, 11, max_roots=1000, cmf=True)


def _dense_h(g, n):
    H = np.zeros((n, n))
    for j0 in range(0, n, 64):
        cols = np.eye(n)[:, j0:j0 + 64].T.copy()  # (m, core_total): unit cores
        H[:, j0:j0 + 64] = g.bst_sigma(cols, "fp64").T
    return 0.5 * (H + H.T)


def _setup():
    prob = _problem()
    vec = random_bst(prob, 3, 1, rank_cut=1, seed=5, split=False)
    pb = PackedBST(vec, 3, 1)
    from fermicg_gb300.gpu import GpuSigma
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    g.bst_set(pb)
    return prob, vec, pb, g


def test_bst_davidson_equals_dense_eigenvalues():
    prob, vec, pb, g = _setup()
    n = pb.core_total
    assert 200 < n < 5000
    w = np.linalg.eigvalsh(_dense_h(g, n))
    R = 3
    rng = np.random.default_rng(0)
    hd = hcmf_diagonal(pb, vec, prob.ops)
    guess = 0.05 * rng.standard_normal((n, R)) / np.sqrt(n)
    for r, k in enumerate(np.argsort(hd)[:R]):
        guess[k, r] += 1.0
    for diag in (hd, None):
        e, X, res, it = g.bst_davidson(guess, diag, tol=1e-7, max_iter=300, precision="fp64")
        assert np.abs(e - w[:R]).max() < 1e-8, (diag is None, e, w[:R])
        assert res.max() < 1e-7 and it > 0
        # eigenvectors: H x = e x through the device sigma
        hx = g.bst_sigma(X.T.copy(), "fp64").T
        assert np.abs(hx - X * e).max() < 1e-6
    e32, _, res32, _ = g.bst_davidson(guess, hd, tol=1e-7, max_iter=300, precision="fp32")
    assert np.abs(e32 - w[:R]).max() < 1e-6  # 1 microhartree
    g.close()


@pytest.mark.parametrize("native", [False, True])
def test_bst_requests_in_a_stream_equal_their_solves_alone(native):
    p0 = workloads.build_problem(12, [3, 3, 3, 3], [(2, 1), (1, 2), (2, 1), (1, 2)], 36, 3, max_roots=1000)
    prob = _problem()
    vec = random_bst(prob, 3, 1, rank_cut=1, seed=5, split=False)
    pb = PackedBST(vec, 3, 1)
    hd = hcmf_diagonal(pb, vec, prob.ops)
    po, pt = packed(prob)
    reqs = []
    for i in range(6):
        if i % 2 == 0:  # TPSCI requests
            st = workloads.energy_ordered_space(p0, 1500, R=1, seed=i)
            f, c, v, _ = pack.pack_state(st)
            reqs.append(Request(0.002 * i, i, pack.pack_ops(p0.ops, p0.bases), pack.pack_terms(p0.ham), f, c,
                                workloads.davidson_guess(f.shape[0], 1, seed=i), tol=1e-7,
                                precision="fp64" if i % 4 == 0 else "fp32", shape="tpsci"))
        else:  # BST requests
            R = 1 + i % 2
            guess = np.zeros((pb.core_total, R))
            for r, k in enumerate(np.argsort(hd)[:R]):
                guess[k, r] = 1.0
            guess += 0.05 * np.random.default_rng(i).standard_normal(guess.shape) / np.sqrt(pb.core_total)
            reqs.append(Request(0.002 * i, i, po, pt, None, None, guess, tol=1e-7,
                                precision="fp64" if i % 4 == 1 else "fp32", shape="bst", bst=pb, bst_hd=hd))
    alone = []
    for r in reqs:
        srv = SolveServer(slots=1)
        alone.append(srv.run([Request(0.0, r.rid, r.packed_ops, r.packed_terms, r.focks, r.cfgs, r.guess, r.tol,
                                      r.precision, r.max_iter, r.shape, bst=r.bst, bst_hd=r.bst_hd)])[0])
        srv.close()
    srv = NativeSolveServer(slots=3, lanes=1) if native else SolveServer(slots=3)
    mixed = srv.run(reqs)
    srv.close()
    assert [m.rid for m in mixed] == [r.rid for r in reqs]
    for a, m in zip(alone, mixed):
        tol = 1e-9 if m.shape == "tpsci" else 1e-8
        np.testing.assert_allclose(m.energies, a.energies, rtol=0, atol=tol)
        assert m.residuals.max() < 1e-7
