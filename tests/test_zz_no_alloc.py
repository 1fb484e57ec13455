"""The allocation-free closed sigma (fcg_sigma_closed_noalloc) against the regular
device entry point, through the C ABI.

fcg_sigma_closed_noalloc serves callers that cannot call cudaMalloc/cudaFree while they
solve (a pool allocator that owns the device memory, a fixed memory budget, or streams
that must not be stalled by cudaFree's device-wide synchronisation).  Its working copies
of C and sigma live in a fixed device array inside the library, shared by every call, so
two calls in a row must not see each other's leftovers.  This file is collected last so a
stop-at-first-failure run has already run every other test.
"""
import numpy as np
import pytest

from fermicg_gb300 import pack
from fermicg_gb300.gpu import FcgError, GpuSigma
from helpers import config1_subspace, packed, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 2e-5


def _ctx(n_cfg=2000, R=4):
    prob, st = config1_subspace(n_cfg, R)
    g = GpuSigma(0)
    po, pt = packed(prob)
    g.set_ops(po)
    g.set_terms(pt)
    f, c, v, _ = pack.pack_state(st)
    g.state_set(f, c)
    return g, v


def _dev(torch, a):
    # column-major (n, R) float64 on the device: a (R, n) contiguous tensor
    return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL)])
def test_noalloc_matches_device_entry_point_on_two_calls(precision, tol):
    torch = pytest.importorskip("torch")
    g, v = _ctx()
    n, R = v.shape
    rng = np.random.default_rng(3)
    for call in range(2):  # two calls in a row share the fixed scratch
        x = v if call == 0 else rng.standard_normal((n, R))
        d_c = _dev(torch, x)
        d_ref = torch.zeros_like(d_c)
        d_out = torch.full_like(d_c, float("nan"))
        g.sigma_closed_device(d_c.data_ptr(), d_ref.data_ptr(), R, precision)
        g.sigma_closed_noalloc(d_c.data_ptr(), d_out.data_ptr(), R, precision)
        torch.cuda.synchronize()
        ref = d_ref.cpu().numpy().T
        out = d_out.cpu().numpy().T
        assert np.all(np.isfinite(out))
        assert rel_err(out, ref) < tol, (call, rel_err(out, ref))


def test_noalloc_fp64_then_fp32_and_stored_blocks():
    """An FP64 call, then an FP32 call on the same scratch (the float copies overlay the
    double ones), then both again after the state's Hamiltonian blocks are stored (the
    stored-block launch path): each against the regular device entry point."""
    torch = pytest.importorskip("torch")
    g, v = _ctx()
    n, R = v.shape
    d_c = _dev(torch, np.random.default_rng(5).standard_normal((n, R)))
    for stored in (False, True):
        if stored:
            g.cache_hamiltonian()
        for precision, tol in (("fp64", FP64_TOL), ("fp32", FP32_TOL)):
            d_ref = torch.zeros_like(d_c)
            d_out = torch.full_like(d_c, float("nan"))
            g.sigma_closed_device(d_c.data_ptr(), d_ref.data_ptr(), R, precision)
            g.sigma_closed_noalloc(d_c.data_ptr(), d_out.data_ptr(), R, precision)
            torch.cuda.synchronize()
            ref = d_ref.cpu().numpy().T
            out = d_out.cpu().numpy().T
            assert np.all(np.isfinite(out))
            assert rel_err(out, ref) < tol, (stored, precision, rel_err(out, ref))


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    g, v = _ctx(n_cfg=600, R=4)
    R = 16
    assert v.shape[0] * R <= 2 ** 20  # in range: accepted
    d_c = torch.zeros((R, v.shape[0]), dtype=torch.float64, device="cuda")
    d_s = torch.zeros_like(d_c)
    g.sigma_closed_noalloc(d_c.data_ptr(), d_s.data_ptr(), R, "fp64")
    g2, v2 = _ctx(n_cfg=70000, R=4)
    d_c2 = torch.zeros((16, v2.shape[0]), dtype=torch.float64, device="cuda")
    with pytest.raises(FcgError, match="exceeds its fixed scratch"):
        g2.sigma_closed_noalloc(d_c2.data_ptr(), d_c2.data_ptr(), 16, "fp64")
