"""GPU closed sigma and diagonal vs the CPU oracle, through the C ABI."""
import numpy as np
import pytest

import oracle
from fermicg_gb300 import pack, workloads
from fermicg_gb300.gpu import GpuSigma
from helpers import small_full, config1_subspace, packed, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10   # relative, FP64 sigma (the parity bar for float64 builds)
FP32_TOL = 2e-5    # relative, mixed (FP32 contraction + FP32 accumulation)


def _gpu_for(prob, st):
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    f, c, v, _ = pack.pack_state(st)
    g.state_set(f, c)
    return g, po, pt, f, c


@pytest.mark.parametrize("R", [1, 3])
def test_closed_sigma_full_space_fp64(R):
    prob, st = small_full()
    g, po, pt, f, c = _gpu_for(prob, st)
    O = oracle.Oracle(po, pt)
    x = np.random.default_rng(R).standard_normal((len(st), R))
    ref = O.sigma_closed(f, c, x)
    out = g.sigma_closed(x, "fp64")
    assert rel_err(out, ref) < FP64_TOL
    out32 = g.sigma_closed(x, "fp32")
    assert rel_err(out32, ref) < FP32_TOL


def test_closed_sigma_config1_subspace_fp64_and_fp32():
    prob, st = config1_subspace(3000, 4)
    g, po, pt, f, c = _gpu_for(prob, st)
    O = oracle.Oracle(po, pt)
    x = st.get_vector()
    ref = O.sigma_closed(f, c, x)
    out = g.sigma_closed(x, "fp64")
    assert rel_err(out, ref) < FP64_TOL
    s = g.stats()
    assert s["n_triples"] > 0 and s["kernel_launches"] >= 1
    out32 = g.sigma_closed(x, "fp32")
    assert rel_err(out32, ref) < FP32_TOL


def test_closed_sigma_is_hermitian_on_subspace():
    prob, st = config1_subspace(3000, 4)
    g, po, pt, f, c = _gpu_for(prob, st)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((len(st), 1))
    y = rng.standard_normal((len(st), 1))
    hx = g.sigma_closed(x)
    hy = g.sigma_closed(y)
    assert abs(float(y[:, 0] @ hx[:, 0] - x[:, 0] @ hy[:, 0])) < 1e-9 * abs(float(y[:, 0] @ hx[:, 0]))


def test_diagonal_matches_oracle():
    prob, st = config1_subspace(3000, 4)
    g, po, pt, f, c = _gpu_for(prob, st)
    O = oracle.Oracle(po, pt)
    np.testing.assert_allclose(g.diagonal(), O.diagonal_H(f, c), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(g.diagonal("Hcmf"), O.diagonal_op(f, c, pack.op_id_of("Hcmf")), rtol=1e-13,
                               atol=1e-13)


def test_empty_and_single_row_states():
    prob, st = config1_subspace(3000, 4)
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    f, c, v, _ = pack.pack_state(st)
    with pytest.raises(Exception):
        g.state_set(f[:0], c[:0])
    g.state_set(f[:1], c[:1])
    O = oracle.Oracle(po, pt)
    x = np.array([[0.7]])
    np.testing.assert_allclose(g.sigma_closed(x), O.sigma_closed(f[:1], c[:1], x), rtol=1e-12)


def _canon(of, oc, ov):
    """Rows of an open sigma as (sorted uint64 keys, values in key order)."""
    f = of.reshape(len(of), -1).astype(np.uint64)
    c = oc.astype(np.uint64)
    k1 = np.zeros(len(of), dtype=np.uint64)
    for j in range(f.shape[1]):
        k1 = (k1 << np.uint64(4)) | f[:, j]
    k2 = np.zeros(len(of), dtype=np.uint64)
    for j in range(c.shape[1]):
        k2 = (k2 << np.uint64(8)) | c[:, j]
    order = np.lexsort((k2, k1))
    return np.stack([k1[order], k2[order]], axis=1), ov[order]


def _assert_open_equal(out, ref):
    ko, vo = _canon(*out)
    kr, vr = _canon(*ref)
    assert ko.shape == kr.shape, (ko.shape, kr.shape)
    assert np.array_equal(ko, kr)
    scale = np.abs(vr).max()
    assert np.abs(vo - vr).max() <= 1e-10 * scale


@pytest.mark.parametrize("thresh", [0.0, 1e-4])
def test_open_sigma_full_space_matches_oracle(thresh):
    """open_matvec_thread: FOIS sigma key set and values vs the oracle (prescreen off)."""
    prob, st = small_full()
    g, po, pt, f, c = _gpu_for(prob, st)
    O = oracle.Oracle(po, pt)
    x = np.random.default_rng(11).standard_normal((len(st), 2))
    _assert_open_equal(g.sigma_open(x, thresh), O.sigma_open(f, c, x, thresh))


@pytest.mark.parametrize("n_cfg,thresh,nbody", [(120, 1e-5, 4), (400, 1e-3, 4), (400, 1e-4, 2)])
def test_open_sigma_config1_subspace_matches_oracle(n_cfg, thresh, nbody):
    prob, st = config1_subspace(n_cfg, 2)
    g, po, pt, f, c = _gpu_for(prob, st)
    O = oracle.Oracle(po, pt)
    x = st.get_vector()
    ref = O.sigma_open(f, c, x, thresh, nbody=nbody)
    assert len(ref[0]) > len(st)
    _assert_open_equal(g.sigma_open(x, thresh, nbody=nbody), ref)
    s = g.stats()
    assert s["open_jobs_kept"] <= s["open_jobs"]


@pytest.mark.parametrize("R", [5, 7])
def test_closed_sigma_many_roots(R):
    """Root counts outside the specialised kernels (generic path) on uneven cluster sizes."""
    prob = workloads.build_problem(10, [2, 2, 4, 2], [(1, 1), (1, 1), (2, 2), (1, 0)], 8, 4, max_roots=1000)
    st = workloads.energy_ordered_space(prob, 600, R=R, seed=2)
    g, po, pt, f, c = _gpu_for(prob, st)
    O = oracle.Oracle(po, pt)
    x = st.get_vector()
    ref = O.sigma_closed(f, c, x)
    assert rel_err(g.sigma_closed(x, "fp64"), ref) < FP64_TOL
    assert rel_err(g.sigma_closed(x, "fp32"), ref) < FP32_TOL
    np.testing.assert_allclose(g.diagonal(), O.diagonal_H(f, c), rtol=1e-12, atol=1e-12)


def test_closed_sigma_config1_30k_matches_oracle():
    """The headline problem's space at 3e4 configurations (about 5e7 triples): FP64 and FP32
    sigma against the oracle's full tps_ci_matvec restatement, R = 4."""
    prob, st = config1_subspace(30000, 4)
    g, po, pt, f, c = _gpu_for(prob, st)
    O = oracle.Oracle(po, pt)
    x = st.get_vector()
    ref = O.sigma_closed(f, c, x)
    assert g.stats()["n_triples"] > 10_000_000
    assert rel_err(g.sigma_closed(x, "fp64"), ref) < FP64_TOL
    assert rel_err(g.sigma_closed(x, "fp32"), ref) < FP32_TOL
    # the same through stored Hamiltonian blocks
    g.cache_hamiltonian()
    assert rel_err(g.sigma_closed(x, "fp64"), ref) < FP64_TOL
    assert rel_err(g.sigma_closed(x, "fp32"), ref) < FP32_TOL


def test_state_rows_then_diagonal_open_sigma_and_a_planned_sigma():
    """fcg_state_rows sets rows and sectors only: the diagonal and the open sigma work on it,
    and the first closed sigma builds the plan (same result as after fcg_state_set); the
    allocation-free sigma refuses a state without a plan."""
    import torch
    from fermicg_gb300.gpu import FcgError
    prob, st = config1_subspace(3000, 4)
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    f, c, v, _ = pack.pack_state(st)
    O = oracle.Oracle(po, pt)
    g.state_set(f, c, plan=False)
    assert g.stats()["n_triples"] == 0
    np.testing.assert_allclose(g.diagonal(), O.diagonal_H(f, c), rtol=1e-12, atol=1e-12)
    d_c = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(v).T)).cuda()
    with pytest.raises(FcgError, match="plan"):
        g.sigma_closed_noalloc(d_c.data_ptr(), d_c.data_ptr(), 4, "fp64")
    _assert_open_equal(g.sigma_open(v[:, :2], 1e-3), O.sigma_open(f, c, v[:, :2], 1e-3))
    assert rel_err(g.sigma_closed(v, "fp64"), O.sigma_closed(f, c, v)) < FP64_TOL
    assert g.stats()["n_triples"] > 0
