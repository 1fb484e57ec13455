"""The BST compressed first-order interacting space on the GPU (fcg_bst_fois) against the
oracle's restatement of build_compressed_1st_order_state, and FOIS-PT2 on the GPU against the
reference's golden (test/test_bst.jl: do_fois_pt2 on the H12 CMF state, thresh_foi = 1e-3)."""
import numpy as np
import pytest

from oracle import bst_fois as F
from test_golden import _h12_problem

pytestmark = pytest.mark.gpu


def _dense(t, r=0):
    return F.transform_modes(t["core"][r], [f.T for f in t["factors"]])


def _compare(fo, fg, R, tol):
    """Same target blocks, same ranks, same dense tensors (factor rotations are free)."""
    assert set(fo) == set(fg)
    for k in fo:
        assert [f.shape[1] for f in fo[k]["factors"]] == [f.shape[1] for f in fg[k]["factors"]], k
        for r in range(R):
            a, c = _dense(fo[k], r), _dense(fg[k], r)
            assert np.abs(a - c).max() <= tol * max(1.0, np.abs(a).max()), (k, r)


@pytest.fixture(scope="module")
def h12():
    from fermicg_gb300 import bst_fois as G
    ints, z, m, b, ops, H = _h12_problem()
    g = G.GpuBSTFois(ops, b, H)
    yield m, b, ops, H, g
    g.close()


def test_fois_cmf_h12_matches_oracle(h12):
    from fermicg_gb300 import bst_fois as G
    m, b, ops, H, g = h12
    N = len(m["clusters"])
    vec, P, Q = F.cmf_bst(b, m["init_fspace"], R=1)
    fo = F.build_compressed_1st_order_state(vec, P, Q, ops, H, N, 1, thresh=1e-3, norb=[len(c) for c in m["clusters"]])
    gv, gP, gQ = G.cmf_state(b, m["init_fspace"], R=1)
    assert gP == P and gQ == Q
    fg = g.fois(gv, gP, gQ, thresh=1e-3)
    assert len(fg) > 100
    _compare(fo, fg, 1, 1e-10)
    assert g.H.stats()["bst_fois_items"] > len(fg)


def test_fois_pt2_h12_matches_reference(h12):
    """do_fois_pt2(v_cmf; thresh_foi = 1e-3): E(PT2) = -18.326971095822113 (reference: 1e-8)."""
    from fermicg_gb300 import bst_fois as G
    m, b, ops, H, g = h12
    gv, gP, gQ = G.cmf_state(b, m["init_fspace"], R=1)
    e, psi1 = g.do_fois_pt2(gv, gP, gQ, thresh_foi=1e-3)
    assert abs(e[0] - (-18.326971095822113)) < 1e-8, e
    assert len(psi1) > 0
    assert g.cg_info[0][1]  # the Hylleraas conjugate gradient converged


def test_fois_two_roots_multiblock_matches_oracle(h12):
    """A 12-block, 2-root state (the CMF block and first-order blocks, second root seeded
    random) expanded at thresh 1e-2: every term type on ranks > 1, on both roots."""
    from fermicg_gb300 import bst_fois as G
    m, b, ops, H, g = h12
    N = len(m["clusters"])
    norb = [len(c) for c in m["clusters"]]
    vec, P, Q = F.cmf_bst(b, m["init_fspace"], R=1)
    fo1 = F.build_compressed_1st_order_state(vec, P, Q, ops, H, N, 1, thresh=1e-3, norb=norb)
    rng = np.random.default_rng(5)
    psi = {}
    for k, t in list(vec.items()) + list(fo1.items())[:11]:
        psi[k] = {"core": [t["core"][0], rng.standard_normal(t["core"][0].shape) * 0.1], "factors": t["factors"]}
    assert any(max(f.shape[1] for f in t["factors"]) > 1 for t in psi.values())
    fo = F.build_compressed_1st_order_state(psi, P, Q, ops, H, N, 2, thresh=1e-2, norb=norb)
    fg = g.fois(psi, P, Q, thresh=1e-2)
    _compare(fo, fg, 2, 1e-9)


def test_fois_everything_below_threshold_is_empty(h12):
    from fermicg_gb300 import bst_fois as G
    m, b, ops, H, g = h12
    gv, gP, gQ = G.cmf_state(b, m["init_fspace"], R=1)
    assert g.fois(gv, gP, gQ, thresh=1e6) == {}


def test_fois_cmf_32_orbitals_matches_oracle():
    """The 32-orbital, 8-cluster x 4 problem (local bases of 16 states per sector, all eight
    Tucker modes): the CMF state's FOIS at thresh 1e-3, block by block against the oracle."""
    from fermicg_gb300 import bst_fois as G
    from fermicg_gb300 import workloads
    prob = workloads.config2_problem(0)
    N = len(prob.clusters)
    vec, P, Q = F.cmf_bst(prob.bases, prob.init_fspace, R=1)
    fo = F.build_compressed_1st_order_state(vec, P, Q, prob.ops, prob.ham, N, 1, thresh=1e-3,
                                           norb=[len(c) for c in prob.clusters])
    g = G.GpuBSTFois(prob.ops, prob.bases, prob.ham)
    try:
        fg = g.fois(vec, P, Q, thresh=1e-3)
        assert g.H.stats()["bst_fois_items"] > 5000
    finally:
        g.close()
    assert len(fg) > 1000
    _compare(fo, fg, 1, 1e-9)


def test_bst_sigma_between_two_states_matches_oracle(h12):
    """fcg_bst_set_between: build_sigma! between two different BST states (the CMF block and a
    FOIS with two roots), both directions, against the oracle's build_sigma!."""
    from fermicg_gb300 import bst_fois as G
    from oracle import bst as OB
    m, b, ops, H, g = h12
    N = len(m["clusters"])
    vec, P, Q = F.cmf_bst(b, m["init_fspace"], R=1)
    fo = F.build_compressed_1st_order_state(vec, P, Q, ops, H, N, 1, thresh=1e-3, norb=[len(c) for c in m["clusters"]])
    rng = np.random.default_rng(11)
    ref = {k: {"core": [t["core"][0], 0.5 * t["core"][0]], "factors": t["factors"]} for k, t in vec.items()}
    fois = {k: {"core": [t["core"][0], rng.standard_normal(t["core"][0].shape)], "factors": t["factors"]}
            for k, t in fo.items()}
    J = G.JointSigma(g.H, ref, fois, 2, between=True)
    hx_ref, hx_fois = J.apply(G._vector(ref, 2), None)          # <X|H|0>
    h0_ref, _ = J.apply(None, G._vector(fois, 2))                # <0|H|X>
    assert np.abs(hx_ref).max() == 0.0                           # no reference-reference couplings
    sx = OB.build_sigma(OB.zero_like(fois, 2), ref, ops, H, N, 2)
    s0 = OB.build_sigma(OB.zero_like(ref, 2), fois, ops, H, N, 2)
    np.testing.assert_allclose(hx_fois, G._vector(sx, 2), atol=1e-11)
    np.testing.assert_allclose(h0_ref, G._vector(s0, 2), atol=1e-11)
