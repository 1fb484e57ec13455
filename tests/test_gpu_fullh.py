"""build_full_H_parallel and compute_expectation_value_parallel on the GPU (fcg_build_full_h,
fcg_expectation) against the oracle's dense H, float64 within 1e-12 relative."""
import numpy as np
import pytest

import oracle
from fermicg_gb300 import pack, workloads
from helpers import packed, rel_err, small_full

pytestmark = pytest.mark.gpu


def _gpu(prob, f, c):
    from fermicg_gb300.gpu import GpuSigma
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    g.state_set(f, c)
    return g, po, pt


def test_full_h_matches_oracle_on_full_space():
    prob, st = small_full()
    f, c, v, _ = pack.pack_state(st)
    g, po, pt = _gpu(prob, f, c)
    H = g.build_full_h()
    ref = oracle.Oracle(po, pt).build_H(f, c)
    assert H.shape == ref.shape
    assert rel_err(H, ref) < 1e-12
    assert rel_err(H, H.T) < 1e-12


def test_full_h_on_energy_ordered_subspace_and_expectation():
    prob = workloads.config0_problem(0)
    st = workloads.energy_ordered_space(prob, 700, R=3, seed=4)
    f, c, v, _ = pack.pack_state(st)
    g, po, pt = _gpu(prob, f, c)
    H = g.build_full_h()
    ref = oracle.Oracle(po, pt).build_H(f, c)
    assert rel_err(H, ref) < 1e-12
    e = g.expectation(v)
    want = np.einsum("ir,ij,jr->r", v, ref, v)
    assert np.abs(e - want).max() < 1e-11 * max(1.0, np.abs(want).max())
    e32 = g.expectation(v, "fp32")
    assert np.abs(e32 - want).max() < 1e-5 * max(1.0, np.abs(want).max())
