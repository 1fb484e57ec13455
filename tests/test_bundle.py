"""Problem bundles (.npz): a saved and reloaded problem gives the same packed operators,
terms and state, and the oracle's sigma from the reloaded arrays equals the original."""
import numpy as np

import oracle
from fermicg_gb300 import pack, workloads
from fermicg_gb300.bundle import load_bundle, save_bundle
from helpers import packed


def test_bundle_round_trip(tmp_path):
    prob = workloads.build_problem(8, [2, 2, 2, 2], [(1, 1)] * 4, 8, 3, max_roots=1000)
    st = workloads.energy_ordered_space(prob, 300, R=2, seed=1)
    path = tmp_path / "prob.npz"
    save_bundle(path, prob, st)
    b = load_bundle(path)
    po, pt = packed(prob)
    f, c, v, _ = pack.pack_state(st)
    assert np.array_equal(b.ops.table, po.table) and np.array_equal(b.ops.data, po.data)
    assert np.array_equal(b.terms.table, pt.table) and np.array_equal(b.terms.ints, pt.ints)
    assert np.array_equal(b.terms.transfers, pt.transfers)
    assert np.array_equal(b.state[0], f) and np.array_equal(b.state[1], c) and np.array_equal(b.state[2], v)
    assert b.clusters == prob.clusters and b.init_fspace == [tuple(x) for x in prob.init_fspace]
    assert np.array_equal(b.h2, prob.ints.h2) and b.meta["seed"] == 3
    s0 = oracle.Oracle(po, pt).sigma_closed(f, c, v)
    s1 = oracle.Oracle(b.ops, b.terms).sigma_closed(*b.state)
    assert np.array_equal(s0, s1)
