"""The oracle's BST compressed first-order interacting space against the reference's golden:
test/test_bst.jl "BST": do_fois_pt2(v_cmf, thresh_foi=1e-3) on the H12 fixture,
E(PT2) = -18.326971095822113 (asserted there to 1e-8).  This pins build_compressed_1st_order_state,
form_sigma_block_expand (1B-4B), the HOSVD compressions, nonorth_add, project_out! and the
Hylleraas solve together."""
import numpy as np

from oracle import bst_fois as F
from test_golden import _h12_problem


def test_fois_pt2_h12_matches_reference():
    ints, z, m, b, ops, H = _h12_problem()
    N = len(m["clusters"])
    vec, P, Q = F.cmf_bst(b, m["init_fspace"], R=1)
    e, psi1, n1 = F.do_fois_pt2(vec, P, Q, ops, H, N, 1, thresh_foi=1e-3, norb=[len(c) for c in m["clusters"]])
    assert abs(e[0] - (-18.326971095822113)) < 1e-8, e
    assert n1 > 0 and len(psi1) > 0


def test_tucker_compress_and_nonorth_add():
    """compress keeps singular values above thresh; nonorth_add of two Tuckers equals the sum
    of their dense tensors."""
    rng = np.random.default_rng(0)
    dims = (4, 3, 5)

    def rand_tucker(ranks):
        f = [np.linalg.qr(rng.standard_normal((d, r)))[0] for d, r in zip(dims, ranks)]
        return {"core": [rng.standard_normal(ranks)], "factors": f}

    def dense(t):
        return F.transform_modes(t["core"][0], [f.T for f in t["factors"]])

    a, c = rand_tucker((2, 2, 3)), rand_tucker((3, 1, 2))
    s = F.nonorth_add_tuckers([a, c])
    np.testing.assert_allclose(dense(s), dense(a) + dense(c), atol=1e-12)
    t = F.compress_tucker(s, 1e-12)
    np.testing.assert_allclose(dense(t), dense(a) + dense(c), atol=1e-10)
    assert F.tucker_len(F.compress_tucker(s, 1e9)) == 0
