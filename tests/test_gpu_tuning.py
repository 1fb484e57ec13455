"""The closed-sigma kernel tuner (fcg_set_tuning / fcg_tuning): every candidate gives the
oracle's sigma, the automatic choice is one of them, and a second state of the same shape
takes the choice from the process's shape cache."""
import numpy as np
import pytest

import oracle
from fermicg_gb300 import pack
from fermicg_gb300.gpu import FcgError, GpuSigma
from helpers import config1_subspace, packed, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 2e-5


def _gpu(n_cfg=3000, R=4):
    prob, st = config1_subspace(n_cfg, R)
    po, pt = packed(prob)
    g = GpuSigma(0)
    g.set_ops(po)
    g.set_terms(pt)
    f, c, v, _ = pack.pack_state(st)
    g.state_set(f, c)
    return g, oracle.Oracle(po, pt).sigma_closed(f, c, v), v


def test_every_candidate_matches_the_oracle():
    g, ref, v = _gpu()
    for cand in range(4):
        g.set_tuning(cand)
        assert rel_err(g.sigma_closed(v, "fp64"), ref) < FP64_TOL, cand
        assert rel_err(g.sigma_closed(v, "fp32"), ref) < FP32_TOL, cand
        t = g.tuning()
        assert t["fp64"] == cand and t["fp32"] == cand
    with pytest.raises(FcgError):
        g.set_tuning(4)
    g.close()


def test_automatic_choice_and_shape_cache():
    g, ref, v = _gpu(2500, 2)
    v2 = v[:, :2]
    ref2 = ref[:, :2]
    assert g.tuning()["fp32"] == -1  # not tuned before the first sigma
    out = g.sigma_closed(v2, "fp32")  # first sigma: times the candidates, keeps the fastest
    assert rel_err(out, ref2) < FP32_TOL
    t = g.tuning()
    assert t["fp32"] in range(4)
    assert all(ms > 0 for ms in t["candidate_ms"]["fp32"])
    assert rel_err(g.sigma_closed(v2, "fp32"), ref2) < FP32_TOL
    assert rel_err(g.sigma_closed(v2, "fp64"), ref2) < FP64_TOL
    assert g.tuning()["fp64"] in range(4)
    # a second context with the same shape: the choice comes from the shape cache
    h, _, _ = _gpu(2500, 2)
    hits = h.stats()["tune_cache_hits"]
    assert rel_err(h.sigma_closed(v2, "fp32"), ref2) < FP32_TOL
    assert h.stats()["tune_cache_hits"] == hits + 1
    assert h.tuning()["fp32"] == t["fp32"]
    g.close()
    h.close()
