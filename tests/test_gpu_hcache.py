"""Stored Hamiltonian blocks (fcg_cache_hamiltonian): closed sigmas, Davidson solves, grouped
launches and the dense H read from the blocks equal the oracle and the direct build."""
import numpy as np
import pytest

import oracle
from fermicg_gb300 import pack, workloads
from fermicg_gb300.gpu import FcgError, GpuSigma, davidson_grouped, sigma_closed_grouped
from helpers import small_full, config1_subspace, packed, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10   # relative, FP64 sigma (the parity bar for float64 builds)
FP32_TOL = 2e-5    # relative, float32 sigma


def _gpu_for(prob, st):
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    f, c, v, _ = pack.pack_state(st)
    g.state_set(f, c)
    return g, po, pt, f, c


@pytest.mark.parametrize("R", [1, 3])
def test_cached_sigma_full_space_matches_oracle(R):
    prob, st = small_full()
    g, po, pt, f, c = _gpu_for(prob, st)
    x = np.random.default_rng(R).standard_normal((len(st), R))
    ref = oracle.Oracle(po, pt).sigma_closed(f, c, x)
    direct64, direct32 = g.sigma_closed(x, "fp64"), g.sigma_closed(x, "fp32")
    nbytes = g.cache_hamiltonian()
    s = g.stats()
    assert nbytes > 0 and s["hcache_pairs"] > 0 and s["hcache_bytes"] == nbytes
    assert s["hcache_pairs"] <= s["n_triples"]
    out64, out32 = g.sigma_closed(x, "fp64"), g.sigma_closed(x, "fp32")
    assert rel_err(out64, ref) < FP64_TOL
    assert rel_err(out64, direct64) < 1e-12
    assert rel_err(out32, ref) < FP32_TOL
    # the float32 blocks are float64 sums rounded once: no worse than the direct float32 build
    assert rel_err(out32, ref) <= 2 * rel_err(direct32, ref) + 1e-7
    g.close()


def test_cached_sigma_config1_subspace_and_drop():
    prob, st = config1_subspace(3000, 4)
    g, po, pt, f, c = _gpu_for(prob, st)
    x = st.get_vector()
    ref = oracle.Oracle(po, pt).sigma_closed(f, c, x)
    g.cache_hamiltonian()
    assert rel_err(g.sigma_closed(x, "fp64"), ref) < FP64_TOL
    assert rel_err(g.sigma_closed(x, "fp32"), ref) < FP32_TOL
    # device-pointer entry points read the blocks too
    import torch
    dc = torch.from_numpy(np.asfortranarray(x).T.copy()).cuda()  # column-major n x R
    ds = torch.empty_like(dc)
    g.sigma_closed_device(dc.data_ptr(), ds.data_ptr(), x.shape[1], "fp64")
    got = ds.cpu().numpy().T
    assert rel_err(got, ref) < FP64_TOL
    assert g.cache_hamiltonian(0) == 0  # dropped: the direct build again
    assert rel_err(g.sigma_closed(x, "fp64"), ref) < FP64_TOL
    g.close()


def test_cache_budget_and_invalidation():
    prob, st = config1_subspace(2000, 2)
    g, po, pt, f, c = _gpu_for(prob, st)
    x = np.random.default_rng(3).standard_normal((len(st), 2))
    ref = oracle.Oracle(po, pt).sigma_closed(f, c, x)
    with pytest.raises(FcgError):
        g.cache_hamiltonian(1000.0)  # too small: nothing is stored
    assert g.stats()["hcache_pairs"] == 0
    assert rel_err(g.sigma_closed(x), ref) < FP64_TOL
    g.cache_hamiltonian()
    # a new state drops the blocks of the old one
    prob2, st2 = config1_subspace(1500, 2)
    f2, c2, v2, _ = pack.pack_state(st2)
    g.state_set(f2, c2)
    x2 = np.random.default_rng(4).standard_normal((len(st2), 2))
    ref2 = oracle.Oracle(po, pt).sigma_closed(f2, c2, x2)
    assert rel_err(g.sigma_closed(x2), ref2) < FP64_TOL
    g.close()


def test_davidson_and_full_h_from_the_blocks():
    prob, st = config1_subspace(2500, 2)
    g, po, pt, f, c = _gpu_for(prob, st)
    guess = workloads.davidson_guess(len(st), 2, seed=5)
    e64, X64, r64, _ = g.davidson(guess, tol=1e-8, max_iter=300, precision="fp64")
    e32, _, _, _ = g.davidson(guess, tol=1e-8, max_iter=300, precision="fp32")
    H = g.build_full_h()
    g.cache_hamiltonian()
    c64, Xc, rc, _ = g.davidson(guess, tol=1e-8, max_iter=300, precision="fp64")
    c32, _, rc32, _ = g.davidson(guess, tol=1e-8, max_iter=300, precision="fp32")
    assert np.abs(c64 - e64).max() < 1e-9 and rc.max() < 1e-8
    assert np.abs(c32 - e64).max() < 1e-9 and rc32.max() < 1e-8
    np.testing.assert_allclose(np.abs(np.sum(Xc * X64, axis=0)), 1.0, atol=1e-7)
    Hc = g.build_full_h()
    assert np.abs(Hc - H).max() < 1e-10 * np.abs(H).max()
    g.close()


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL)])
def test_grouped_launch_mixes_stored_and_direct_problems(precision, tol):
    import torch
    items = []
    for i in range(5):
        prob, st = workloads.config3_instance(i, max_cluster=4, n_cfg_range=(300, 1200))
        f, c, v, _ = pack.pack_state(st)
        po, pt = pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham)
        g = GpuSigma(0)
        g.set_ops(po)
        g.set_terms(pt)
        g.state_set(f, c)
        x = np.random.default_rng(10 + i).standard_normal((f.shape[0], v.shape[1]))
        ref = oracle.Oracle(po, pt).sigma_closed(f, c, x)
        if i % 2 == 0:
            g.cache_hamiltonian()
        dc = torch.from_numpy(np.asfortranarray(x).T.copy()).cuda()
        items.append((g, x, ref, dc, torch.empty_like(dc)))
    gs = [it[0] for it in items]
    sigma_closed_grouped(gs, [it[3].data_ptr() for it in items], [it[4].data_ptr() for it in items],
                         [it[1].shape[1] for it in items], precision)
    torch.cuda.synchronize()
    for g, x, ref, dc, ds in items:
        assert rel_err(ds.cpu().numpy().T, ref) < tol
    # grouped Davidson over the same mix equals the solo solves
    guesses = [workloads.davidson_guess(it[1].shape[0], it[1].shape[1], seed=20 + q,
                                        lowest=np.argsort(it[0].diagonal())[:it[1].shape[1]])
               for q, it in enumerate(items)]
    res = davidson_grouped(gs, guesses, tol=1e-7, max_iter=300, precision=precision)
    for (g, *_), gu, (e, X, r, it) in zip(items, guesses, res):
        e1, X1, r1, it1 = g.davidson(gu, tol=1e-7, max_iter=300, precision=precision)
        assert np.abs(e - e1).max() < 1e-9 and r.max() < 1e-7
    for g in gs:
        g.close()
