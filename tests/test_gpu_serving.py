"""Serving loop: concurrent Davidson solves give the same result alone and in the mix."""
import numpy as np
import pytest

from fermicg_gb300 import pack, workloads
from fermicg_gb300.serving import Request, SolveServer, latency_summary

pytestmark = pytest.mark.gpu


def _request(rid, prob, n_cfg, R, seed, arrival, precision="fp64"):
    st = workloads.energy_ordered_space(prob, n_cfg, R=R, seed=seed)
    f, c, v, _ = pack.pack_state(st)
    guess = np.zeros_like(v)
    guess[:R] = np.eye(R)  # lowest configurations first (energy-ordered space)
    return Request(arrival, rid, pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham), f, c, guess,
                   tol=1e-7, precision=precision, shape=f"{prob.meta['norb']}o")


def test_results_alone_equal_results_in_the_mix():
    p0 = workloads.build_problem(12, [3, 3, 3, 3], [(2, 1), (1, 2), (2, 1), (1, 2)], 36, 3, max_roots=1000)
    p1 = workloads.build_problem(16, [4, 4, 4, 4], [(2, 2)] * 4, 24, 4, max_roots=12, delta_elec=2)
    reqs = [_request(i, p0 if i % 2 == 0 else p1, 1500 if i % 2 == 0 else 3000, 1 + (i % 3), i, 0.002 * i)
            for i in range(8)]
    alone = []
    for r in reqs:
        srv = SolveServer(slots=1)
        alone.append(srv.run([Request(0.0, r.rid, r.packed_ops, r.packed_terms, r.focks, r.cfgs, r.guess, r.tol,
                                      r.precision, r.max_iter, r.shape)])[0])
        srv.close()
    srv = SolveServer(slots=4)
    mixed = srv.run(reqs)
    srv.close()
    assert len(mixed) == len(reqs)
    for a, m in zip(alone, mixed):
        assert a.rid == m.rid
        np.testing.assert_allclose(m.energies, a.energies, rtol=0, atol=1e-9)
        assert m.residuals.max() < 1e-7
    s = latency_summary(mixed)
    assert s["p99_s"] >= s["p50_s"] > 0
