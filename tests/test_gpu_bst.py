"""BST (block-sparse Tucker) sigma on the GPU -- fcg_bst_set (cache_hamiltonian) and
fcg_bst_sigma (build_sigma!) -- against the oracle's build_sigma! on the same seeded
vectors.  FP64 within 1e-12 relative (the device sums each group's terms into one operator
before contracting, so the rounding order differs from the oracle's); FP32 within 2e-5."""
import numpy as np
import pytest

from fermicg_gb300 import workloads
from fermicg_gb300.bst import PackedBST, plan_triples, synthetic_bst
from helpers import packed, random_bst, rel_err
from oracle import bst as obst

pytestmark = pytest.mark.gpu


def _three():
    return workloads.build_problem(6, [2, 2, 2], [(1, 1), (1, 1), (1, 0)], 6, 5, max_roots=1000, cmf=False)


def _four():
    return workloads.build_problem(6, [2, 1, 2, 1], [(1, 1), (1, 0), (1, 1), (0, 1)], 6, 7, max_roots=1000,
                                   cmf=False)


def _gpu(prob):
    from fermicg_gb300.gpu import GpuSigma
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    return g


def _run(prob, vec, N, R, precision="fp64", nbody=4, g=None):
    pb = PackedBST(vec, N, R)
    g = g or _gpu(prob)
    ct = g.bst_set(pb, nbody=nbody)
    assert ct == pb.core_total
    out = g.bst_sigma(pb.cores_of(vec), precision)
    want = pb.cores_of(obst.build_sigma(obst.zero_like(vec, R), vec, prob.ops, prob.ham, N, R, nbody=nbody))
    return g, pb, out, want


def test_bst_sigma_split_blocks_fp64():
    prob = _three()
    vec = random_bst(prob, 3, 2, rank_cut=1, seed=2, split=True)
    g, pb, out, want = _run(prob, vec, 3, 2)
    assert np.abs(want).max() > 0.1
    assert rel_err(out, want) < 1e-12
    st = g.stats()
    assert st["bst_blocks"] == len(pb.keys)
    assert st["bst_groups"] <= st["bst_triples"]
    assert st["bst_flops_executed"] <= st["bst_flops_reference"]


def test_bst_sigma_full_rank_and_fp32():
    prob = _three()
    vec = random_bst(prob, 3, 3, rank_cut=0, seed=1, split=False)
    g, pb, out, want = _run(prob, vec, 3, 3)
    assert rel_err(out, want) < 1e-12
    out32 = g.bst_sigma(pb.cores_of(vec), "fp32")
    assert rel_err(out32, want) < 2e-5


def test_bst_sigma_four_clusters_4body_and_triples():
    prob = _four()
    vec = random_bst(prob, 4, 2, rank_cut=1, seed=3, split=True)
    g, pb, out, want = _run(prob, vec, 4, 2)
    assert rel_err(out, want) < 1e-12
    got = {tuple(int(x) for x in r) for r in g.bst_triples()}
    ref = {tuple(int(x) for x in r) for r in plan_triples(pb, prob.ham, ops=prob.ops)}
    assert got == ref


@pytest.mark.parametrize("nbody", [1, 2, 3])
def test_bst_sigma_nbody_limit(nbody):
    prob = _four()
    vec = random_bst(prob, 4, 1, rank_cut=1, seed=4, split=True)
    _, _, out, want = _run(prob, vec, 4, 1, nbody=nbody)
    assert rel_err(out, want) < 1e-12


def test_bst_sigma_global_workspace_path():
    """Cores of 512 elements with 16 roots: two workspace buffers per root exceed the
    shared-memory budget of the sigma kernel, so these groups run from global memory."""
    prob = workloads.build_problem(9, [3, 3, 3], [(2, 1), (1, 2), (1, 1)], 9, 11, max_roots=1000, cmf=False)
    vec = random_bst(prob, 3, 16, rank_cut=1, seed=5, split=False)
    pb = PackedBST(vec, 3, 16)
    assert 2 * 16 * int(pb.blocks[:, 1].max()) * 8 > 96 * 1024
    _, _, out, want = _run(prob, vec, 3, 16)
    assert rel_err(out, want) < 1e-12


def test_bst_sigma_hermitian_on_24_orbital_blocks():
    """24 orbitals / 6 clusters of 4 (M=16): BST blocks with up to two excited clusters
    (ranks 2-6) over the reference sector and its single charge transfers.  The projected H
    is symmetric, so x . H y = H x . y for the device sigma."""
    prob = workloads.config1_problem(0)
    ref = tuple(tuple(f) for f in prob.init_fspace)
    sectors = [ref]
    for i in range(6):
        for j in range(6):
            if i != j:
                fs = [list(f) for f in ref]
                fs[i][0] -= 1
                fs[j][0] += 1
                sectors.append(tuple(tuple(f) for f in fs))
    vec = synthetic_bst(prob, sectors, max_q=2, rank_range=(2, 6), R=2, seed=9)
    pb = PackedBST(vec, 6, 2)
    g = _gpu(prob)
    g.bst_set(pb)
    x = pb.cores_of(vec)
    rng = np.random.default_rng(1)
    y = rng.standard_normal(x.shape)
    hx = g.bst_sigma(x)
    hy = g.bst_sigma(y)
    for r in range(2):
        a, b = float(x[r] @ hy[r]), float(hx[r] @ y[r])
        assert abs(a - b) < 1e-10 * max(abs(a), 1.0)
    # linearity
    h2 = g.bst_sigma(2.0 * x - 0.5 * y)
    assert rel_err(h2, 2.0 * hx - 0.5 * hy) < 1e-12
