"""GPU closed sigma and diagonal vs the CPU oracle, through the C ABI."""
import numpy as np
import pytest

import oracle
from fermicg_gb300 import pack, workloads
from fermicg_gb300.gpu import GpuSigma
from helpers import small_full, config1_subspace, packed, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10   # relative, FP64 sigma (spec parity bar)
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


def _open_dict(of, oc, ov):
    return {(of[i].tobytes(), oc[i].tobytes()): ov[i] for i in range(len(of))}


@pytest.mark.parametrize("thresh", [0.0, 1e-4])
def test_open_sigma_full_space_matches_oracle(thresh):
    """open_matvec_thread: FOIS sigma key set and values vs the oracle (prescreen off)."""
    prob, st = small_full()
    g, po, pt, f, c = _gpu_for(prob, st)
    O = oracle.Oracle(po, pt)
    x = np.random.default_rng(11).standard_normal((len(st), 2))
    ref = _open_dict(*O.sigma_open(f, c, x, thresh))
    out = _open_dict(*g.sigma_open(x, thresh))
    assert set(out) == set(ref)
    scale = max(np.abs(v).max() for v in ref.values())
    for k, v in ref.items():
        np.testing.assert_allclose(out[k], v, rtol=0, atol=1e-10 * scale)


@pytest.mark.parametrize("thresh,nbody", [(1e-5, 4), (1e-3, 4), (1e-4, 2)])
def test_open_sigma_config1_subspace_matches_oracle(thresh, nbody):
    prob, st = config1_subspace(400, 2)
    g, po, pt, f, c = _gpu_for(prob, st)
    O = oracle.Oracle(po, pt)
    x = st.get_vector()
    ref = _open_dict(*O.sigma_open(f, c, x, thresh, nbody=nbody))
    out = _open_dict(*g.sigma_open(x, thresh, nbody=nbody))
    assert len(ref) > len(st)
    assert set(out) == set(ref)
    scale = max(np.abs(v).max() for v in ref.values())
    for k, v in ref.items():
        np.testing.assert_allclose(out[k], v, rtol=0, atol=1e-10 * scale)
    s = g.stats()
    assert s["open_jobs_kept"] <= s["open_jobs"]
