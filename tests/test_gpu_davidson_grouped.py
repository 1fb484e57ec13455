"""fcg_davidson_grouped: independent Davidson solves in lockstep with grouped sigma builds give
each problem the same eigenpairs as its solve alone (and as a dense diagonalisation)."""
import numpy as np
import pytest

import oracle
from fermicg_gb300 import pack, workloads
from fermicg_gb300.gpu import GpuSigma, davidson_grouped

pytestmark = pytest.mark.gpu


def _problems(n, max_cluster=4):
    out = []
    for i in range(n):
        prob, st = workloads.config3_instance(i, max_cluster=max_cluster, n_cfg_range=(300, 1500))
        f, c, v, _ = pack.pack_state(st)
        po, pt = pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham)
        g = GpuSigma(0)
        g.set_ops(po)
        g.set_terms(pt)
        g.state_set(f, c)
        R = v.shape[1]
        guess = workloads.davidson_guess(f.shape[0], R, seed=i, lowest=np.argsort(g.diagonal())[:R])
        H = oracle.Oracle(po, pt).build_H(f, c)
        out.append((g, guess, np.linalg.eigvalsh(0.5 * (H + H.T))[:R]))
    return out


@pytest.mark.parametrize("precision,tol_e", [("fp64", 1e-9), ("fp32", 1e-6)])
def test_grouped_solves_equal_solo_solves(precision, tol_e):
    probs = _problems(6)
    gpus = [p[0] for p in probs]
    res = davidson_grouped(gpus, [p[1] for p in probs], tol=1e-7, max_iter=300, precision=precision)
    for (g, guess, ref), (e, X, r, it) in zip(probs, res):
        assert np.abs(e - ref).max() < tol_e, (e, ref)
        assert r.max() < 1e-7 and it > 0
        np.testing.assert_allclose(X.T @ X, np.eye(len(e)), atol=1e-10)
        e1, X1, r1, it1 = g.davidson(guess, tol=1e-7, max_iter=300, precision=precision)
        assert np.abs(e - e1).max() < 1e-10
        # same eigenvectors up to sign (the spectra here are not degenerate)
        np.testing.assert_allclose(np.abs(np.sum(X * X1, axis=0)), 1.0, atol=1e-8)
    for g in gpus:
        g.close()


def test_grouped_single_problem_is_fcg_davidson():
    (g, guess, ref), = _problems(1)
    e, X, r, it = davidson_grouped([g], [guess], tol=1e-8, max_iter=300)[0]
    e1, X1, r1, it1 = g.davidson(guess, tol=1e-8, max_iter=300)
    assert np.abs(e - ref).max() < 1e-9
    assert np.abs(e - e1).max() < 1e-11 and it == it1
    g.close()


def test_grouped_rejects_a_context_twice():
    (g, guess, ref), = _problems(1)
    with pytest.raises(Exception):
        davidson_grouped([g, g], [guess, guess])
    g.close()


def test_a_failing_problem_is_named_and_the_contexts_stay_usable():
    from fermicg_gb300.gpu import FcgError
    probs = _problems(3)
    gpus = [p[0] for p in probs]
    guesses = [p[1].copy() for p in probs]
    guesses[1][:] = np.nan  # no usable initial direction: the solve of problem 1 fails
    with pytest.raises(FcgError, match="problem 1"):
        davidson_grouped(gpus, guesses, tol=1e-7, max_iter=300)
    for g, guess, ref in probs:  # every context still solves alone, on its own stream
        e, X, r, it = g.davidson(guess, tol=1e-7, max_iter=300)
        assert np.abs(e - ref).max() < 1e-9
    res = davidson_grouped([gpus[0], gpus[2]], [probs[0][1], probs[2][1]], tol=1e-7, max_iter=300)
    assert np.abs(res[1][0] - probs[2][2]).max() < 1e-9
    # a failure of the first problem is named too
    guesses = [p[1].copy() for p in probs]
    guesses[0][:] = np.nan
    with pytest.raises(FcgError, match=r"problem 0\)"):
        davidson_grouped(gpus, guesses, tol=1e-7, max_iter=300)
    for g in gpus:
        g.close()


def test_lanes_of_a_large_group_equal_solo_solves():
    """64 problems: the group runs as two lanes (a stream and host thread each); every
    problem's energies equal its solve alone, with and without stored blocks."""
    gpus, guesses = [], []
    for i in range(64):
        prob, st = workloads.config3_instance(i, max_cluster=4, n_cfg_range=(150, 400))
        f, c, v, _ = pack.pack_state(st)
        g = GpuSigma(0)
        g.set_ops(pack.pack_ops(prob.ops, prob.bases))
        g.set_terms(pack.pack_terms(prob.ham))
        g.state_set(f, c)
        R = v.shape[1]
        gpus.append(g)
        guesses.append(workloads.davidson_guess(f.shape[0], R, seed=100 + i, lowest=np.argsort(g.diagonal())[:R]))
    for stored in (False, True):
        if stored:
            for g in gpus:
                g.cache_hamiltonian()
        res = davidson_grouped(gpus, guesses, tol=1e-7, max_iter=300, precision="fp32")
        assert gpus[0].stats()["group_launches"] > 0
        for g, gu, (e, X, r, it) in zip(gpus, guesses, res):
            e1, X1, r1, it1 = g.davidson(gu, tol=1e-7, max_iter=300, precision="fp32")
            assert r.max() < 1e-7 and np.abs(e - e1).max() < 1e-9
    for g in gpus:
        g.close()
