"""The tensor-core (tcgen05) part of the float BST sigma: GEMM-shaped groups (at least 64
bra-active rows, 16 ket-active columns, 32 spectator columns over the roots) run as 3xTF32
tiles with FP32 accumulation.  Checked against the oracle's build_sigma! on a 12-orbital
problem whose 2-cluster groups reach 144 x 144 operators, and against the device FP64 sigma
(itself oracle-checked) on the 32-orbital vector with cores up to 12^4."""
import numpy as np
import pytest

from fermicg_gb300 import workloads
from fermicg_gb300.bst import PackedBST, synthetic_bst
from helpers import packed, rel_err
from oracle import bst as obst

pytestmark = pytest.mark.gpu

FP32_TOL = 2e-5


def _gpu(prob):
    from fermicg_gb300.gpu import GpuSigma
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    return g


def test_tensor_core_groups_match_the_oracle():
    prob = workloads.build_problem(12, [4, 4, 4], [(2, 2), (2, 2), (2, 2)], 24, 21, max_roots=1000, cmf=False)
    ref = tuple(tuple(f) for f in prob.init_fspace)
    R = 4
    vec = synthetic_bst(prob, [ref], max_q=3, rank_range=(8, 12), R=R, seed=3)
    pb = PackedBST(vec, 3, R)
    g = _gpu(prob)
    g.bst_set(pb)
    x = pb.cores_of(vec)
    want = pb.cores_of(obst.build_sigma(obst.zero_like(vec, R), vec, prob.ops, prob.ham, 3, R))
    out64 = g.bst_sigma(x, "fp64")
    assert rel_err(out64, want) < 1e-12
    out32 = g.bst_sigma(x, "fp32")
    st = g.stats()
    assert st["bst_tc_groups"] > 0 and st["bst_tc_flops"] > 0 and st["bst_tc_ms"] > 0
    assert rel_err(out32, want) < FP32_TOL
    # the same groups on the CUDA cores agree, and the switch back works
    g.bst_tensor_cores(False)
    out_cc = g.bst_sigma(x, "fp32")
    assert g.stats()["bst_tc_groups"] == 0
    assert rel_err(out_cc, want) < FP32_TOL
    g.bst_tensor_cores(True)
    assert rel_err(g.bst_sigma(x, "fp32"), out32) < 1e-6
    g.close()


def test_tensor_core_sigma_at_config2_core_sizes():
    """32 orbitals, 8 clusters x 4: the reference sector with up to four excited clusters,
    Tucker ranks 4-12 (cores up to 12^4), 2 roots; two calls in a row, and linearity."""
    prob = workloads.config2_problem(0)
    secs = workloads.single_transfer_sectors(prob)
    vec = synthetic_bst(prob, secs[:1], max_q=4, rank_range=(4, 12), R=2, seed=0)
    pb = PackedBST(vec, 8, 2)
    assert int(pb.blocks[:, 1].max()) > 10000
    g = _gpu(prob)
    g.bst_set(pb)
    x = pb.cores_of(vec)
    ref = g.bst_sigma(x, "fp64")
    for _ in range(2):
        out = g.bst_sigma(x, "fp32")
        assert g.stats()["bst_tc_groups"] > 100
        assert rel_err(out, ref) < FP32_TOL
    y = np.random.default_rng(2).standard_normal(x.shape)
    hy = g.bst_sigma(y, "fp32")
    assert rel_err(g.bst_sigma(x - 0.5 * y, "fp32"), out - 0.5 * hy) < 1e-5
    g.close()


def test_config2_sigma_sampled_blocks_match_the_oracle():
    """The FP64 and FP32 sigma on the config-2-sized vector (every launch path: warp chunks,
    the CTA-per-group workspace buckets, the global-workspace groups taken largest first, the
    tensor-core groups on the second stream) against the oracle's build_sigma! for a sample of
    bra blocks: the largest cores and an even spread of the rest."""
    prob = workloads.config2_problem(0)
    secs = workloads.single_transfer_sectors(prob)
    R = 2
    vec = synthetic_bst(prob, secs[:1], max_q=4, rank_range=(4, 12), R=R, seed=0)
    pb = PackedBST(vec, 8, R)
    g = _gpu(prob)
    g.bst_set(pb)
    x = pb.cores_of(vec)
    out64 = g.bst_sigma(x, "fp64")
    out32 = g.bst_sigma(x, "fp32")
    sizes = pb.blocks[:, 1]
    pick = set(np.argsort(-sizes)[:3].tolist()) | set(range(0, len(pb.keys), max(1, len(pb.keys) // 5)))
    sample = [pb.keys[i] for i in sorted(pick)]
    want = obst.build_sigma({k: obst.zero_like({k: vec[k]}, R)[k] for k in sample}, vec, prob.ops, prob.ham, 8, R)
    for k in sample:
        i = pb.index[k]
        o, n = int(pb.blocks[i, 0]), int(pb.blocks[i, 1])
        ref = np.stack([np.asarray(want[k]["core"][r]).reshape(-1, order="F") for r in range(R)])
        scale = max(float(np.abs(ref).max()), 1e-300)
        assert float(np.abs(out64[:, o:o + n] - ref).max()) / scale < 1e-10
        assert float(np.abs(out32[:, o:o + n] - ref).max()) / scale < FP32_TOL
    g.close()
