"""The closed-sigma join on the device (fcg_set_planner(1), the default) against the host
planner (fcg_set_planner(0)): the permutation pool, the term-sector records, the lane jobs
and the warp-chunk table are bit-identical, the counts agree, and sigma through either plan
matches the oracle."""
import numpy as np
import pytest

import oracle
from fermicg_gb300 import pack, workloads
from fermicg_gb300.gpu import GpuSigma
from fermicg_gb300.terms import ClusteredOperator
from helpers import config1_subspace, packed, rel_err, small_full

pytestmark = pytest.mark.gpu

KEYS = ("perm", "ts", "jobs", "chunk_lo", "chunk_val")
COUNTS = ("n_work_items", "n_triples", "flops_reference", "flops_executed")


def _both(po, pt, f, c):
    g = GpuSigma(0)
    g.set_ops(po)
    g.set_terms(pt)
    g.set_planner(False)
    g.state_set(f, c)
    host = g.plan_arrays()
    sh = g.stats()
    g.set_planner(True)
    dev = g.plan_arrays()
    sd = g.stats()
    assert sh["join_on_device"] == 0 and sd["join_on_device"] == 1
    for k in KEYS:
        assert host[k].shape == dev[k].shape, k
        assert np.array_equal(host[k], dev[k]), k
    assert host["items"] == dev["items"]
    for k in COUNTS:
        assert sh[k] == sd[k], k
    return g, host


def _state(prob, st):
    po, pt = packed(prob)
    f, c, v, _ = pack.pack_state(st)
    return po, pt, f, c, v


def test_planners_agree_full_space():
    prob, st = small_full()
    po, pt, f, c, v = _state(prob, st)
    g, host = _both(po, pt, f, c)
    assert host["items"] > 0 and len(host["jobs"]) % 32 == 0
    x = np.random.default_rng(0).standard_normal((len(f), 2))
    assert rel_err(g.sigma_closed(x, "fp64"), oracle.Oracle(po, pt).sigma_closed(f, c, x)) < 1e-10


@pytest.mark.parametrize("n_cfg", [3000, 30000])
def test_planners_agree_24_orbitals(n_cfg):
    prob, st = config1_subspace(n_cfg, 4)
    po, pt, f, c, v = _state(prob, st)
    g, host = _both(po, pt, f, c)
    x = v[:, :2].copy()
    dev_sigma = g.sigma_closed(x, "fp64")
    g.set_planner(False)
    host_sigma = g.sigma_closed(x, "fp64")
    assert rel_err(dev_sigma, host_sigma) < 1e-13
    if n_cfg == 3000:
        assert rel_err(dev_sigma, oracle.Oracle(po, pt).sigma_closed(f, c, x)) < 1e-10


def test_planners_agree_eight_clusters():
    """32 orbitals / 8 clusters of 4 (local bases of 8 states per sector): 8 clusters of
    spectator keys and up to 4-body active sets."""
    prob = workloads.build_problem(32, [4] * 8, [(2, 2)] * 8, 96, 1001, max_roots=8, delta_elec=2)
    st = workloads.energy_ordered_space(prob, 2000, R=2, seed=0)
    po, pt, f, c, v = _state(prob, st)
    _both(po, pt, f, c)


def test_planners_agree_three_orbital_clusters():
    prob = workloads.build_problem(12, [3] * 4, [(2, 1), (1, 2), (2, 1), (1, 2)], 36, 5, max_roots=1000)
    st = workloads.energy_ordered_space(prob, 1500, R=1, seed=0)
    po, pt, f, c, v = _state(prob, st)
    _both(po, pt, f, c)


@pytest.mark.parametrize("max_body", [1, 2])
def test_planners_agree_with_fewer_terms(max_body):
    """Terms up to max_body clusters: transfers whose term lists are empty, sets missing."""
    prob, st = config1_subspace(3000, 4)
    ham = ClusteredOperator(prob.ham.n_clusters)
    for tr, terms in prob.ham:
        ham.trans[tr] = [t for t in terms if t.nbody <= max_body]
    po = pack.pack_ops(prob.ops, prob.bases)
    pt = pack.pack_terms(ham)
    f, c, v, _ = pack.pack_state(st)
    g, host = _both(po, pt, f, c)
    x = v[:, :1].copy()
    assert rel_err(g.sigma_closed(x, "fp64"), oracle.Oracle(po, pt).sigma_closed(f, c, x)) < 1e-10


def test_planners_agree_on_one_row_and_one_sector():
    prob, st = config1_subspace(3000, 4)
    po, pt, f, c, v = _state(prob, st)
    _both(po, pt, f[:1].copy(), c[:1].copy())
    first = np.all(f == f[0], axis=(1, 2))
    n0 = int(np.argmin(first)) if not first.all() else len(f)
    _both(po, pt, f[:n0].copy(), c[:n0].copy())


def _corrupt(f, c, kind):
    """A copy of the rows with one (or two) planted errors."""
    f = f.copy()
    c = c.copy()
    n0 = int(np.argmin(np.all(f == f[0], axis=(1, 2))))  # first row of the second sector
    if kind == "split_sector":       # the first sector comes back after the second
        f[n0 + 1] = f[0]
        c[n0 + 1] = c[0]
    elif kind == "fock_range":
        f[n0:n0 + 1, 2, 0] = 16
    elif kind == "fock_negative":
        f[n0:n0 + 1, 1, 1] = -1
    elif kind == "state_range":
        c[7, 3] = 300
    elif kind == "cluster_size":
        f[n0, 4, 0] = 5              # 4-orbital clusters
    elif kind == "no_basis":
        f[n0, 0] = (4, 4)            # a sector outside the local bases
    elif kind == "beyond_basis":
        c[11, 2] = 200
    elif kind == "split_before_range":   # both; the earlier row wins
        f[n0 + 1] = f[0]
        c[n0 + 1] = c[0]
        f[len(f) - 1, 2, 0] = 16
    elif kind == "range_before_size":    # state range (checked first) beats an earlier size error
        f[n0, 4, 0] = 5
        c[len(c) - 1, 0] = -2
    return f, c


@pytest.mark.parametrize("kind", ["split_sector", "fock_range", "fock_negative", "state_range", "cluster_size",
                                  "no_basis", "beyond_basis", "split_before_range", "range_before_size"])
def test_bad_rows_same_message_both_planners(kind):
    prob, st = config1_subspace(3000, 4)
    po, pt, f, c, v = _state(prob, st)
    fb, cb = _corrupt(f, c, kind)
    msgs = []
    for dev in (False, True):
        g = GpuSigma(0)
        g.set_ops(po)
        g.set_terms(pt)
        g.set_planner(dev)
        with pytest.raises(Exception) as ei:
            g.state_set(fb, cb)
        msgs.append(str(ei.value))
        g.state_set(f, c)  # the context stays usable
        assert g.stats()["n_cfg"] == len(f)
    assert msgs[0] == msgs[1], msgs
    assert "Fock" in msgs[0] or "local state" in msgs[0]


def test_planners_agree_on_an_empty_join():
    """Only terms that change the Fock sector, on the rows of one sector: no ket sector exists
    for any (bra sector, transfer), so the plan has no records, work items or lane jobs, and
    sigma is zero."""
    prob, st = config1_subspace(3000, 4)
    ham = ClusteredOperator(prob.ham.n_clusters)
    for tr, terms in prob.ham:
        if any(int(x) != 0 for pair in tr for x in pair):
            ham.trans[tr] = list(terms)
    po = pack.pack_ops(prob.ops, prob.bases)
    pt = pack.pack_terms(ham)
    f, c, v, _ = pack.pack_state(st)
    n0 = int(np.argmin(np.all(f == f[0], axis=(1, 2))))
    g, host = _both(po, pt, f[:n0].copy(), c[:n0].copy())
    assert host["items"] == 0 and len(host["jobs"]) == 0 and len(host["ts"]) == 0
    assert g.stats()["n_triples"] == 0
    x = v[:n0, :2].copy()
    for prec in ("fp64", "fp32"):
        assert np.abs(g.sigma_closed(x, prec)).max() == 0.0
