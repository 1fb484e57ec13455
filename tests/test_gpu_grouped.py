"""Grouped closed sigma (fcg_sigma_closed_grouped): independent problems of uneven sizes
and root counts in one launch must give each problem's own sigma -- FP64 within 1e-12
relative of the per-context sigma (same contraction, only the order of atomic additions
differs), FP32 within 2e-5 -- and one member is checked against the oracle."""
import numpy as np
import pytest

import oracle
from fermicg_gb300 import pack, workloads
from helpers import rel_err

pytestmark = pytest.mark.gpu


def _instances(n, max_cluster=4):
    from fermicg_gb300.gpu import GpuSigma
    import torch
    out = []
    for i in range(n):
        prob, st = workloads.config3_instance(i, max_cluster=max_cluster)
        f, c, v, _ = pack.pack_state(st)
        g = GpuSigma(0)
        g.set_problem(prob.ops, prob.bases, prob.ham)
        g.state_set(f, c)
        R = v.shape[1]
        dc = torch.from_numpy(np.asfortranarray(v).T.copy()).cuda()  # (R, n) == column-major (n, R)
        ds = torch.empty_like(dc)
        out.append((prob, f, c, v, g, dc, ds, R))
    return out


def test_grouped_matches_individual_and_oracle():
    import torch
    from fermicg_gb300.gpu import sigma_closed_grouped
    items = _instances(12)
    assert len({it[7] for it in items}) > 1  # uneven root counts
    assert len({it[1].shape[0] for it in items}) > 1  # uneven sizes
    for prec, tol in (("fp64", 1e-12), ("fp32", 2e-5)):
        sigma_closed_grouped([it[4] for it in items], [it[5].data_ptr() for it in items],
                             [it[6].data_ptr() for it in items], [it[7] for it in items], prec)
        torch.cuda.synchronize()
        grouped = [it[6].clone() for it in items]
        for k, (prob, f, c, v, g, dc, ds, R) in enumerate(items):
            g.sigma_closed_device(dc.data_ptr(), ds.data_ptr(), R, "fp64")
            torch.cuda.synchronize()
            assert rel_err(grouped[k].cpu().numpy(), ds.cpu().numpy()) < tol, (prec, k)
    # one member against the oracle
    prob, f, c, v, g, dc, ds, R = items[3]
    po, pt = pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham)
    ref = oracle.Oracle(po, pt).sigma_closed(f, c, v)
    sigma_closed_grouped([it[4] for it in items], [it[5].data_ptr() for it in items],
                         [it[6].data_ptr() for it in items], [it[7] for it in items], "fp64")
    torch.cuda.synchronize()
    got = items[3][6].cpu().numpy().T  # (n, R)
    assert rel_err(got, ref) < 1e-10


def test_grouped_rejects_bad_groups():
    from fermicg_gb300.gpu import FcgError, sigma_closed_grouped
    items = _instances(2)
    gs = [it[4] for it in items]
    with pytest.raises(FcgError):  # the same context twice
        sigma_closed_grouped([gs[0], gs[0]], [items[0][5].data_ptr()] * 2, [items[0][6].data_ptr()] * 2,
                             [items[0][7]] * 2)
    with pytest.raises(FcgError):  # root count out of range
        sigma_closed_grouped(gs, [it[5].data_ptr() for it in items], [it[6].data_ptr() for it in items], [0, 1])
