"""Device Davidson and the GPU TPSCI driver vs the oracle and the reference's goldens."""
import numpy as np
import pytest

import oracle
from fermicg_gb300 import pack
from fermicg_gb300.gpu import GpuSigma
from fermicg_gb300.state import TPSCIstate
from helpers import config1_subspace, packed

pytestmark = pytest.mark.gpu


def _dense_lowest(prob, st, R):
    po, pt = packed(prob)
    f, c, v, _ = pack.pack_state(st)
    H = oracle.Oracle(po, pt).build_H(f, c)
    return np.linalg.eigvalsh(0.5 * (H + H.T))[:R]


@pytest.mark.parametrize("precision,tol_e", [("fp64", 1e-9), ("fp32", 1e-6)])
def test_davidson_matches_dense_eigenvalues(precision, tol_e):
    """Energies within 1e-9 (FP64) / 1 uEh (mixed: FP32 sigma + FP64 refinement) of a dense solve."""
    prob, st = config1_subspace(1500, 4)
    ref = _dense_lowest(prob, st, 4)
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    f, c, v, _ = pack.pack_state(st)
    g.state_set(f, c)
    guess = np.zeros_like(v)
    hd = g.diagonal()
    for r, i in enumerate(np.argsort(hd)[:4]):
        guess[i, r] = 1.0
    e, X, res, it = g.davidson(guess, tol=1e-7, max_iter=300, precision=precision)
    assert np.abs(e - ref).max() < tol_e, (e, ref)
    assert res.max() < 1e-7
    # Ritz vectors are orthonormal eigenvectors
    np.testing.assert_allclose(X.T @ X, np.eye(4), atol=1e-10)


def _h12():
    from test_golden import _h12_problem
    return _h12_problem()


def test_gpu_tpsci_h12_matches_reference_energies():
    """test/test_tpsci.jl "tpsci h12 64bit": e0 and e0+e2 of 7 roots within 1e-8, on the GPU."""
    from fermicg_gb300.tpsci import GpuTPSCI
    ints, z, m, b, ops, H = _h12()
    R, N = m["nroots"], len(m["clusters"])
    st = TPSCIstate(N, R)
    ref = tuple(map(tuple, m["init_fspace"]))
    row = np.zeros(R)
    row[0] = 1.0
    st[(ref, (0,) * N)] = row
    for i, ex in enumerate(m["excitons"]):
        row = np.zeros(R)
        row[i + 1] = 1.0
        st[(ref, tuple(ex))] = row
    kw = m["tpsci_kwargs"]
    T = GpuTPSCI(ops, b, H)
    e0, v0 = T.tpsci_ci(st, thresh_cipsi=kw["thresh_cipsi"], thresh_foi=kw["thresh_foi"],
                        thresh_asci=kw.get("thresh_asci"), conv_thresh=kw["conv_thresh"], ci_conv=1e-9)
    np.testing.assert_allclose(np.abs(e0), np.abs(np.array(m["e0"])), atol=1e-8, rtol=0)
    e2 = T.pt2_energy(v0, thresh_foi=m["pt2_thresh_foi"])
    np.testing.assert_allclose(np.abs(e0 + e2), np.abs(np.array(m["e0_plus_e2"])), atol=1e-8, rtol=0)
    # compute_pt1_wavefunction on the GPU vs the oracle, same input vectors: same FOIS keys,
    # amplitudes and e2 within 1e-10
    from oracle.tpsci import OracleTPSCI
    e2g, vg = T.pt1_wavefunction(v0, thresh_foi=m["pt2_thresh_foi"])
    e2o, vo = OracleTPSCI(ops, b, H).pt1_wavefunction(v0, thresh_foi=m["pt2_thresh_foi"])
    np.testing.assert_allclose(e2g, e2o, atol=1e-10, rtol=0)
    dg, do = vg.as_dict(), vo.as_dict()
    assert set(dg) == set(do)
    for k, x in do.items():
        np.testing.assert_allclose(dg[k], x, atol=1e-10, rtol=1e-10)
    T.close()


def test_davidson_seven_roots_from_padded_guess():
    """The solve of the second H12 TPSCI iteration: 7 roots, previous eigenvectors padded with
    zeros for the new configurations (the oracle driver produces the space)."""
    from oracle.tpsci import OracleTPSCI, _add, _copy, _zero
    from fermicg_gb300.state import TPSCIstate as TS
    ints, z, m, b, ops, H = _h12()
    R, N = m["nroots"], len(m["clusters"])
    st = TS(N, R)
    ref = tuple(map(tuple, m["init_fspace"]))
    row = np.zeros(R)
    row[0] = 1.0
    st[(ref, (0,) * N)] = row
    for i, ex in enumerate(m["excitons"]):
        row = np.zeros(R)
        row[i + 1] = 1.0
        st[(ref, tuple(ex))] = row
    kw = m["tpsci_kwargs"]
    T = OracleTPSCI(ops, b, H)
    e1, v1 = T.tpsci_ci(st, thresh_cipsi=kw["thresh_cipsi"], thresh_foi=kw["thresh_foi"], max_iter=2,
                        conv_thresh=0.0)
    # v1 is the 2nd-iteration variational vector; rebuild its padded guess
    f, c, v, _ = pack.pack_state(v1)
    po, pt = pack.pack_ops(ops, b), pack.pack_terms(H)
    Hd = oracle.Oracle(po, pt).build_H(f, c)
    ref_e = np.linalg.eigvalsh(0.5 * (Hd + Hd.T))[:R]
    g = GpuSigma(0)
    g.set_ops(po)
    g.set_terms(pt)
    g.state_set(f, c)
    guess = np.zeros_like(v)
    guess[:R] = np.eye(R)
    e, X, res, it = g.davidson(guess, tol=1e-9, max_iter=300)
    assert np.all(np.isfinite(X))
    assert np.abs(e - ref_e).max() < 1e-9, (e, ref_e)
