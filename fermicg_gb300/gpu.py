"""ctypes binding of the in-tree CUDA library (include/fcg_gpu.h).

This is the Python mirror of the reference's sigma entry points:
  tps_ci_matvec(ci_vector, cluster_ops, clustered_ham)   src/tpsci_outer.jl:462
  compute_diagonal(ci_vector, cluster_ops, H | "Hcmf")    src/tpsci_outer.jl:694/722
all running on the GPU through libfcg_gpu.so.  There is no CPU fallback: if
the library is missing or no GPU is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import pack
from .local_fci import N_OPS

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libfcg_gpu.so")

# closed-sigma kernel candidates of the library's tuner (index -> description)
TUNE_CANDIDATES = ["4 (float) / 3 (double) CTAs per SM, ~4 waves of warp chunks",
                   "3 (float) / 2 (double) CTAs per SM, ~4 waves of warp chunks",
                   "4 (float) / 3 (double) CTAs per SM, ~16 waves of warp chunks",
                   "3 (float) / 2 (double) CTAs per SM, ~16 waves of warp chunks"]

FCG_FP64 = 0
FCG_FP32 = 1
PRECISION = {"fp64": FCG_FP64, "fp32": FCG_FP32, "mixed": FCG_FP32}

# exported symbol -> (restype, argtypes); every name declared in include/fcg_gpu.h
_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_int64
SIGNATURES = {
    "fcg_version": (_I, []),
    "fcg_ctx_create": (_I, [_I, ctypes.POINTER(_P)]),
    "fcg_ctx_destroy": (_I, [_P]),
    "fcg_last_error": (ctypes.c_char_p, [_P]),
    "fcg_set_stream": (_I, [_P, _P]),
    "fcg_set_ops": (_I, [_P, _I, _P, _L, _P, _L, _P]),
    "fcg_set_terms": (_I, [_P, _I, _P, _L, _P, _I, _P]),
    "fcg_state_set": (_I, [_P, _L, _P, _P]),
    "fcg_state_rows": (_I, [_P, _L, _P, _P]),
    "fcg_sigma_closed": (_I, [_P, _I, _P, _P, _I]),
    "fcg_sigma_closed_device": (_I, [_P, _I, _P, _P, _I]),
    "fcg_cache_hamiltonian": (_I, [_P, ctypes.c_double, ctypes.POINTER(ctypes.c_int64)]),
    "fcg_diagonal": (_I, [_P, _I, _P]),
    "fcg_sigma_open": (_I, [_P, _I, _P, ctypes.c_double, _I, ctypes.POINTER(_L)]),
    "fcg_sigma_open_fetch": (_I, [_P, _P, _P, _P]),
    "fcg_davidson": (_I, [_P, _I, _P, _I, _I, ctypes.c_double, ctypes.c_double, _I, _I, _P, _P, _P,
                          ctypes.POINTER(_I)]),
    "fcg_sigma_closed_noalloc": (_I, [_P, _I, _P, _P, _I]),
    "fcg_get_stats": (_I, [_P, _P]),
    "fcg_set_tuning": (_I, [_P, _I]),
    "fcg_set_planner": (_I, [_P, _I]),
    "fcg_plan_sizes": (_I, [_P, _P]),
    "fcg_plan_copy": (_I, [_P, _I, _P, _L]),
    "fcg_bst_tensor_cores": (_I, [_P, _I]),
    "fcg_bst_davidson": (_I, [_P, _I, _P, _P, _I, _I, ctypes.c_double, ctypes.c_double, _I, _P, _P, _P,
                              ctypes.POINTER(_I)]),
    "fcg_submit_bst": (_I, [_P, _P, _I, _P, _P, _I, _I, ctypes.c_double, ctypes.c_double, _I, ctypes.POINTER(_L)]),
    "fcg_tuning": (_I, [_P, _P, _P]),
    "fcg_bst_set": (_I, [_P, _I, _L, _P, _P, _P, _L, _P, ctypes.POINTER(_L)]),
    "fcg_bst_sigma": (_I, [_P, _I, _P, _P, _I]),
    "fcg_bst_set_between": (_I, [_P, _I, _L, _L, _P, _P, _P, _L, _P, ctypes.POINTER(_L)]),
    "fcg_bst_sigma_device": (_I, [_P, _I, _P, _P, _I]),
    "fcg_bst_triples": (_I, [_P, _P]),
    "fcg_sigma_closed_grouped": (_I, [_I, _P, _P, _P, _P, _I]),
    "fcg_davidson_grouped": (_I, [_I, _P, _P, _P, _I, _I, ctypes.c_double, ctypes.c_double, _I, _I, _P, _P, _P,
                                  _P]),
    "fcg_server_create": (_I, [_I, _I, _I, ctypes.c_double, ctypes.POINTER(_P)]),
    "fcg_server_destroy": (_I, [_P]),
    "fcg_submit": (_I, [_P, _P, _I, _P, _I, _I, ctypes.c_double, ctypes.c_double, _I, _I, ctypes.POINTER(_L)]),
    "fcg_poll": (_I, [_P, _L, ctypes.POINTER(_I)]),
    "fcg_wait": (_I, [_P, _L, _I, _P, _P, _P, ctypes.POINTER(_I)]),
    "fcg_expectation": (_I, [_P, _I, _P, _P, _I]),
    "fcg_build_full_h": (_I, [_P, _P]),
    "fcg_bst_fois": (_I, [_P, _I, _I, ctypes.c_double, _I, _L, _P, _P, _P, _L, _P, _P, _P, ctypes.POINTER(_L),
                          ctypes.POINTER(_L), ctypes.POINTER(_L)]),
    "fcg_bst_fois_get": (_I, [_P, _P, _P, _P, _P, _P]),
}


class Stats(ctypes.Structure):
    _fields_ = [("n_cfg", ctypes.c_int64), ("n_sectors", ctypes.c_int64), ("n_work_items", ctypes.c_int64),
                ("n_triples", ctypes.c_int64), ("flops_reference", ctypes.c_int64),
                ("flops_executed", ctypes.c_int64), ("dressed_elements", ctypes.c_int64),
                ("plan_seconds", ctypes.c_double), ("last_kernel_ms", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("open_jobs", ctypes.c_int64),
                ("open_jobs_kept", ctypes.c_int64), ("open_contractions", ctypes.c_int64),
                ("davidson_sigma_calls", ctypes.c_int64), ("bst_blocks", ctypes.c_int64),
                ("bst_triples", ctypes.c_int64), ("bst_groups", ctypes.c_int64),
                ("bst_cache_elements", ctypes.c_int64), ("bst_flops_reference", ctypes.c_int64),
                ("bst_flops_executed", ctypes.c_int64), ("bst_cache_seconds", ctypes.c_double),
                ("bst_plan_seconds", ctypes.c_double), ("bst_fois_items", ctypes.c_int64),
                ("bst_fois_seconds", ctypes.c_double), ("group_rounds", ctypes.c_int64),
                ("group_launches", ctypes.c_int64), ("group_setup_seconds", ctypes.c_double),
                ("group_step_seconds", ctypes.c_double), ("group_issue_seconds", ctypes.c_double),
                ("group_wait_seconds", ctypes.c_double), ("hcache_pairs", ctypes.c_int64),
                ("hcache_bytes", ctypes.c_int64), ("hcache_seconds", ctypes.c_double),
                ("open_expand_ms", ctypes.c_double), ("open_flops_reference", ctypes.c_int64),
                ("open_bytes", ctypes.c_int64), ("tune_seconds", ctypes.c_double),
                ("tune_cache_hits", ctypes.c_int64), ("bst_tc_groups", ctypes.c_int64),
                ("bst_tc_flops", ctypes.c_int64), ("bst_tc_mma_flops", ctypes.c_int64), ("bst_tc_ms", ctypes.c_double),
                ("join_seconds", ctypes.c_double), ("join_on_device", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libfcg_gpu.so (built by fermicg_gb300.build.build()); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library not built: {path} (run fermicg_gb300.build.build())")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class FcgError(RuntimeError):
    pass


class GpuSigma:
    """One device context holding cluster ops, the clustered Hamiltonian and a state index."""

    def __init__(self, device: int = 0):
        self.L = load_library()
        h = ctypes.c_void_p()
        rc = self.L.fcg_ctx_create(device, ctypes.byref(h))
        if rc != 0:
            raise FcgError(f"fcg_ctx_create failed ({rc}): no usable CUDA device {device}")
        self.h = h
        self._keep = []
        self.N = None
        self.n_cfg = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.fcg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            msg = self.L.fcg_last_error(self.h)
            raise FcgError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def set_stream(self, stream_ptr: int | None):
        """Run later calls on an external cudaStream_t (e.g. torch's current stream)."""
        self._check(self.L.fcg_set_stream(self.h, ctypes.c_void_p(stream_ptr or 0)), "fcg_set_stream")

    # --- uploads ------------------------------------------------------------
    def set_ops(self, packed_ops: "pack.PackedOps"):
        tab = np.ascontiguousarray(packed_ops.table, dtype=np.int64)
        dat = np.ascontiguousarray(packed_ops.data, dtype=np.float64)
        norb = np.ascontiguousarray(packed_ops.cluster_norb, dtype=np.int32)
        self.N = int(packed_ops.n_clusters)
        self._check(self.L.fcg_set_ops(self.h, self.N, _ptr(norb), tab.shape[0], _ptr(tab), dat.size, _ptr(dat)),
                    "fcg_set_ops")

    def set_terms(self, packed_terms: "pack.PackedTerms"):
        tab = np.ascontiguousarray(packed_terms.table, dtype=np.int32)
        ints = np.ascontiguousarray(packed_terms.ints, dtype=np.float64)
        tr = np.ascontiguousarray(packed_terms.transfers, dtype=np.int16)
        self._check(self.L.fcg_set_terms(self.h, tab.shape[0], _ptr(tab), ints.size, _ptr(ints), tr.shape[0],
                                         _ptr(tr)), "fcg_set_terms")

    def set_problem(self, ops, bases, ham):
        self.set_ops(pack.pack_ops(ops, bases))
        self.set_terms(pack.pack_terms(ham))

    def state_set(self, focks, cfgs, plan: bool = True):
        """The state's rows (TPSCIstate order) and, with plan (default), its closed-sigma plan;
        plan=False sets only the rows and sectors (fcg_state_rows: diagonals, open sigma),
        and the first closed sigma builds the plan."""
        f = np.ascontiguousarray(focks, dtype=np.int16)
        c = np.ascontiguousarray(cfgs, dtype=np.int16)
        fn = self.L.fcg_state_set if plan else self.L.fcg_state_rows
        self._check(fn(self.h, f.shape[0], _ptr(f), _ptr(c)), "fcg_state_set" if plan else "fcg_state_rows")
        self.n_cfg = f.shape[0]

    # --- sigma --------------------------------------------------------------
    def sigma_closed(self, coeffs, precision="fp64"):
        """tps_ci_matvec: coeffs (n_cfg, R) host array -> sigma (n_cfg, R) float64."""
        c = np.asfortranarray(coeffs, dtype=np.float64)
        n, R = c.shape
        if n != self.n_cfg:
            raise ValueError("coefficient rows do not match the state")
        sig = np.zeros((n, R), dtype=np.float64, order="F")
        self._check(self.L.fcg_sigma_closed(self.h, R, _ptr(c), _ptr(sig), PRECISION[precision]),
                    "fcg_sigma_closed")
        return np.ascontiguousarray(sig)

    def sigma_closed_device(self, d_c_ptr: int, d_sigma_ptr: int, R: int, precision="fp64"):
        """Device-pointer variant (column-major n_cfg x R float64 buffers on this GPU)."""
        self._check(self.L.fcg_sigma_closed_device(self.h, R, ctypes.c_void_p(d_c_ptr), ctypes.c_void_p(d_sigma_ptr),
                                                   PRECISION[precision]), "fcg_sigma_closed_device")

    def cache_hamiltonian(self, max_bytes: float = 64e9) -> int:
        """Store the state's Hamiltonian blocks on the device (fcg_cache_hamiltonian); later
        closed sigmas, Davidson solves and grouped launches of this state read them.  Returns
        the bytes they take; max_bytes <= 0 drops them."""
        b = ctypes.c_int64(0)
        self._check(self.L.fcg_cache_hamiltonian(self.h, float(max_bytes), ctypes.byref(b)), "fcg_cache_hamiltonian")
        return int(b.value)

    def sigma_closed_noalloc(self, d_c_ptr: int, d_sigma_ptr: int, R: int, precision="fp64"):
        """Allocation-free device-pointer sigma (fixed 16 MiB scratch; n_cfg * R <= 2**20)."""
        self._check(self.L.fcg_sigma_closed_noalloc(self.h, R, ctypes.c_void_p(d_c_ptr), ctypes.c_void_p(d_sigma_ptr),
                                                    PRECISION[precision]), "fcg_sigma_closed_noalloc")

    def expectation(self, coeffs, precision="fp64"):
        """compute_expectation_value_parallel: c_r^T H c_r per root (coeffs (n_cfg, R))."""
        c = np.asfortranarray(coeffs, dtype=np.float64)
        n, R = c.shape
        if n != self.n_cfg:
            raise ValueError("coefficient rows do not match the state")
        e = np.zeros(R)
        self._check(self.L.fcg_expectation(self.h, R, _ptr(c), _ptr(e), PRECISION[precision]), "fcg_expectation")
        return e

    def build_full_h(self):
        """build_full_H_parallel on the state: dense (n_cfg, n_cfg) float64."""
        H = np.zeros((self.n_cfg, self.n_cfg), order="F")
        self._check(self.L.fcg_build_full_h(self.h, _ptr(H)), "fcg_build_full_h")
        return H

    def diagonal(self, op: str | None = None):
        """compute_diagonal: op None = all zero-transfer terms; else an op string ("Hcmf", "H")."""
        oid = -1 if op is None else pack.op_id_of(op)
        hd = np.zeros(self.n_cfg)
        self._check(self.L.fcg_diagonal(self.h, oid, _ptr(hd)), "fcg_diagonal")
        return hd

    def sigma_open(self, coeffs, thresh, nbody=4):
        """open_matvec_thread: (fock (m,N,2) int16, cfg (m,N) int16, coeff (m,R)) of the FOIS sigma.
        coeff is column-major as the library writes it (no second copy of m*R doubles)."""
        c = np.asfortranarray(coeffs, dtype=np.float64)
        n, R = c.shape
        if n != self.n_cfg:
            raise ValueError("coefficient rows do not match the state")
        m = ctypes.c_int64(0)
        self._check(self.L.fcg_sigma_open(self.h, R, _ptr(c), float(thresh), int(nbody), ctypes.byref(m)),
                    "fcg_sigma_open")
        m = m.value
        of = np.empty((m, self.N, 2), dtype=np.int16)
        oc = np.empty((m, self.N), dtype=np.int16)
        ov = np.empty((m, R), dtype=np.float64, order="F")
        self._check(self.L.fcg_sigma_open_fetch(self.h, _ptr(of), _ptr(oc), _ptr(ov)), "fcg_sigma_open_fetch")
        return of, oc, ov

    def davidson(self, v0, max_iter=100, max_ss_vecs=12, tol=1e-8, lindep=1e-12, precision="fp64",
                 precond=True):
        """Block Davidson on the device (tps_ci_davidson): returns (energies, vectors, residuals, iters)."""
        v = np.asfortranarray(v0, dtype=np.float64)
        n, R = v.shape
        if n != self.n_cfg:
            raise ValueError("guess rows do not match the state")
        e = np.zeros(R)
        res = np.zeros(R)
        out = np.zeros((n, R), order="F")
        it = ctypes.c_int(0)
        self._check(self.L.fcg_davidson(self.h, R, _ptr(v), int(max_iter), int(max_ss_vecs), float(tol),
                                        float(lindep), PRECISION[precision], int(bool(precond)), _ptr(e),
                                        _ptr(out), _ptr(res), ctypes.byref(it)), "fcg_davidson")
        return e, np.ascontiguousarray(out), res, it.value

    # --- block-sparse Tucker ---------------------------------------------------
    def bst_set(self, packed_bst, nbody=4):
        """cache_hamiltonian for a BST structure (fermicg_gb300.bst.PackedBST); returns core_total."""
        pb = packed_bst
        N = pb.N
        fock = np.ascontiguousarray(np.array([[list(f) for f in k[0]] for k in pb.keys], dtype=np.int16)
                                    .reshape(-1, N, 2))
        blocks = np.ascontiguousarray(pb.blocks[:, 5:5 + 3 * N], dtype=np.int64)
        foff = np.ascontiguousarray(pb.factor_off, dtype=np.int64)
        fac = np.ascontiguousarray(pb.factors, dtype=np.float64)
        ct = ctypes.c_int64(0)
        self._check(self.L.fcg_bst_set(self.h, int(nbody), blocks.shape[0], _ptr(fock), _ptr(blocks), _ptr(foff),
                                       fac.size, _ptr(fac), ctypes.byref(ct)), "fcg_bst_set")
        self.bst_core_total = ct.value
        return ct.value

    def bst_set_raw(self, fock, blocks, factor_off, factors, nbody=4):
        """fcg_bst_set on arrays in its own layout (blocks [n][3N] = {rank, start, len})."""
        f = np.ascontiguousarray(fock, dtype=np.int16)
        bl = np.ascontiguousarray(blocks, dtype=np.int64)
        fo = np.ascontiguousarray(factor_off, dtype=np.int64)
        fa = np.ascontiguousarray(factors, dtype=np.float64)
        ct = ctypes.c_int64(0)
        self._check(self.L.fcg_bst_set(self.h, int(nbody), bl.shape[0], _ptr(f), _ptr(bl), _ptr(fo), fa.size, _ptr(fa),
                                       ctypes.byref(ct)), "fcg_bst_set")
        self.bst_core_total = ct.value
        return ct.value

    def bst_set_between_raw(self, n_first, fock, blocks, factor_off, factors, nbody=4):
        """fcg_bst_set_between: only couplings between blocks [0, n_first) and the rest."""
        f = np.ascontiguousarray(fock, dtype=np.int16)
        bl = np.ascontiguousarray(blocks, dtype=np.int64)
        fo = np.ascontiguousarray(factor_off, dtype=np.int64)
        fa = np.ascontiguousarray(factors, dtype=np.float64)
        ct = ctypes.c_int64(0)
        self._check(self.L.fcg_bst_set_between(self.h, int(nbody), int(n_first), bl.shape[0], _ptr(f), _ptr(bl),
                                               _ptr(fo), fa.size, _ptr(fa), ctypes.byref(ct)), "fcg_bst_set_between")
        self.bst_core_total = ct.value
        return ct.value

    def bst_sigma(self, cores, precision="fp64"):
        """build_sigma!: cores (R, core_total) -> sigma cores (R, core_total) float64."""
        c = np.ascontiguousarray(cores, dtype=np.float64)
        R = c.shape[0]
        if c.shape[1] != self.bst_core_total:
            raise ValueError("core length does not match the BST structure")
        out = np.zeros_like(c)
        self._check(self.L.fcg_bst_sigma(self.h, R, _ptr(c), _ptr(out), PRECISION[precision]), "fcg_bst_sigma")
        return out

    def bst_davidson(self, v0, hdiag=None, max_iter=200, max_ss_vecs=12, tol=1e-6, lindep=1e-12,
                     precision="fp64"):
        """The BST ci_solve Davidson on the device over the cores of the last bst_set: v0
        (core_total, R); hdiag (core_total,) preconditioner diagonal or None.  Returns
        (energies, vectors (core_total, R), residuals, iterations)."""
        v = np.asfortranarray(v0, dtype=np.float64)
        n, R = v.shape
        if n != self.bst_core_total:
            raise ValueError("guess rows do not match the BST structure")
        hd = None if hdiag is None else np.ascontiguousarray(hdiag, dtype=np.float64)
        if hd is not None and hd.shape != (n,):
            raise ValueError("hdiag must have core_total entries")
        e, res = np.zeros(R), np.zeros(R)
        out = np.zeros((n, R), order="F")
        it = ctypes.c_int(0)
        self._check(self.L.fcg_bst_davidson(self.h, R, _ptr(v), _ptr(hd) if hd is not None else None, int(max_iter),
                                            int(max_ss_vecs), float(tol), float(lindep), PRECISION[precision],
                                            _ptr(e), _ptr(out), _ptr(res), ctypes.byref(it)), "fcg_bst_davidson")
        return e, np.ascontiguousarray(out), res, it.value

    def bst_sigma_device(self, d_cores_ptr: int, d_sigma_ptr: int, R: int, precision="fp64"):
        self._check(self.L.fcg_bst_sigma_device(self.h, R, ctypes.c_void_p(d_cores_ptr), ctypes.c_void_p(d_sigma_ptr),
                                                PRECISION[precision]), "fcg_bst_sigma_device")

    def bst_triples(self):
        n = self.stats()["bst_triples"]
        out = np.zeros((n, 4), dtype=np.int32)
        self._check(self.L.fcg_bst_triples(self.h, _ptr(out)), "fcg_bst_triples")
        return out

    def bst_fois(self, fock, blocks, factor_off, factors, cores, spaces, thresh, nbody=4, compress_twice=True):
        """build_compressed_1st_order_state on the device (fcg_bst_fois).  Inputs in the
        fcg_bst_set layout (blocks [n][3N] = {rank, start, len}), cores (R, core_total), spaces
        int32 [N][nmax+1][nmax+1][4].  Returns (fock, blocks, factor_off, factors, cores)."""
        f = np.ascontiguousarray(fock, dtype=np.int16)
        bl = np.ascontiguousarray(blocks, dtype=np.int64)
        fo = np.ascontiguousarray(factor_off, dtype=np.int64)
        fa = np.ascontiguousarray(factors, dtype=np.float64)
        co = np.ascontiguousarray(cores, dtype=np.float64)
        sp = np.ascontiguousarray(spaces, dtype=np.int32)
        R = co.shape[0]
        nb, ct, nf = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
        self._check(self.L.fcg_bst_fois(self.h, R, int(nbody), float(thresh), int(bool(compress_twice)), bl.shape[0],
                                        _ptr(f), _ptr(bl), _ptr(fo), fa.size, _ptr(fa), _ptr(co), _ptr(sp),
                                        ctypes.byref(nb), ctypes.byref(ct), ctypes.byref(nf)), "fcg_bst_fois")
        N = self.N
        of = np.zeros((nb.value, N, 2), dtype=np.int16)
        ob = np.zeros((nb.value, 3 * N), dtype=np.int64)
        oo = np.zeros((nb.value, N), dtype=np.int64)
        ofa = np.zeros(max(nf.value, 1))
        oc = np.zeros((R, max(ct.value, 1)))
        self._check(self.L.fcg_bst_fois_get(self.h, _ptr(of), _ptr(ob), _ptr(oo), _ptr(ofa), _ptr(oc)),
                    "fcg_bst_fois_get")
        return of, ob, oo, ofa[:nf.value], oc[:, :ct.value]

    def bst_tensor_cores(self, enable: bool = True):
        """float BST sigma: GEMM-shaped groups on the tcgen05 tensor cores (default) or not."""
        self._check(self.L.fcg_bst_tensor_cores(self.h, int(bool(enable))), "fcg_bst_tensor_cores")

    def set_planner(self, on_device: bool = True):
        """Closed-sigma join on the device (default) or on the host (its reference); the
        state's plan is rebuilt on its next use.  Both give bit-identical plans."""
        self._check(self.L.fcg_set_planner(self.h, int(bool(on_device))), "fcg_set_planner")

    def plan_arrays(self):
        """The state's closed-sigma plan as numpy arrays: permutation pool (int32), term-sector
        records (72-byte rows, uint8), lane jobs (16-byte rows, uint8), warp-chunk first warp
        tasks and first stored values (int64); and the work-item count."""
        sz = np.zeros(5, dtype=np.int64)
        self._check(self.L.fcg_plan_sizes(self.h, _ptr(sz)), "fcg_plan_sizes")
        out = {}
        for which, name, dt, width in ((0, "perm", np.int32, 1), (1, "ts", np.uint8, 72), (2, "jobs", np.uint8, 16),
                                       (3, "chunk_lo", np.int64, 1), (4, "chunk_val", np.int64, 1)):
            n = int(sz[which if which < 4 else 3])
            a = np.zeros((n, width) if width > 1 else n, dtype=dt)
            self._check(self.L.fcg_plan_copy(self.h, which, _ptr(a), a.nbytes), "fcg_plan_copy")
            out[name] = a
        out["items"] = int(sz[4])
        return out

    def set_tuning(self, mode: int = -1):
        """Closed-sigma kernel candidate: -1 times the candidates on the first sigma of each
        precision (default), 0..3 forces one."""
        self._check(self.L.fcg_set_tuning(self.h, int(mode)), "fcg_set_tuning")

    def tuning(self):
        """{"fp64": candidate, "fp32": candidate (-1: not tuned yet), "candidate_ms": {...}}"""
        ch = (ctypes.c_int * 2)()
        ms = (ctypes.c_float * 8)()
        self._check(self.L.fcg_tuning(self.h, ch, ms), "fcg_tuning")
        return {"fp64": ch[0], "fp32": ch[1], "candidate_ms": {"fp64": list(ms[:4]), "fp32": list(ms[4:])},
                "candidates": TUNE_CANDIDATES}

    def stats(self):
        s = Stats()
        self._check(self.L.fcg_get_stats(self.h, ctypes.byref(s)), "fcg_get_stats")
        return s.as_dict()


def sigma_closed_grouped(gpus, d_c_ptrs, d_sigma_ptrs, roots, precision="fp64"):
    """Closed sigmas of independent problems (one GpuSigma each, state set) in one grouped
    launch; device buffers column-major (n_cfg, R) float64.  Returns the leading context's
    stats (kernel time of the grouped launch)."""
    n = len(gpus)
    if not (len(d_c_ptrs) == len(d_sigma_ptrs) == len(roots) == n) or n == 0:
        raise ValueError("one buffer pair and root count per context")
    L = gpus[0].L
    hs = (ctypes.c_void_p * n)(*[g.h.value for g in gpus])
    rs = (ctypes.c_int * n)(*[int(r) for r in roots])
    cs = (ctypes.c_void_p * n)(*[int(p) for p in d_c_ptrs])
    ss = (ctypes.c_void_p * n)(*[int(p) for p in d_sigma_ptrs])
    gpus[0]._check(L.fcg_sigma_closed_grouped(n, hs, rs, cs, ss, PRECISION[precision]), "fcg_sigma_closed_grouped")
    return gpus[0].stats()


def davidson_grouped(gpus, guesses, max_iter=100, max_ss_vecs=12, tol=1e-8, lindep=1e-12, precision="fp64",
                     precond=True):
    """Davidson solves of independent problems (one GpuSigma each, state set) in lockstep, their
    sigma builds grouped per iteration (fcg_davidson_grouped).  guesses: one (n_cfg, R) array
    per problem.  Returns a list of (energies, vectors, residuals, iterations)."""
    n = len(gpus)
    if len(guesses) != n or n == 0:
        raise ValueError("one guess per context")
    L = gpus[0].L
    vs = [np.asfortranarray(v, dtype=np.float64) for v in guesses]
    for g, v in zip(gpus, vs):
        if v.shape[0] != g.n_cfg:
            raise ValueError("guess rows do not match the state")
    es = [np.zeros(v.shape[1]) for v in vs]
    rs = [np.zeros(v.shape[1]) for v in vs]
    xs = [np.zeros(v.shape, order="F") for v in vs]
    its = (ctypes.c_int * n)()
    P = ctypes.c_void_p
    gpus[0]._check(L.fcg_davidson_grouped(
        n, (P * n)(*[g.h.value for g in gpus]), (ctypes.c_int * n)(*[v.shape[1] for v in vs]),
        (P * n)(*[v.ctypes.data for v in vs]), int(max_iter), int(max_ss_vecs), float(tol), float(lindep),
        PRECISION[precision], int(bool(precond)), (P * n)(*[e.ctypes.data for e in es]),
        (P * n)(*[x.ctypes.data for x in xs]), (P * n)(*[r.ctypes.data for r in rs]), its), "fcg_davidson_grouped")
    return [(es[q], np.ascontiguousarray(xs[q]), rs[q], its[q]) for q in range(n)]


def tps_ci_matvec(state, gpu: GpuSigma, precision="fp64"):
    """sigma = H c for a TPSCIstate already indexed on `gpu` (tpsci_outer.jl:462)."""
    return gpu.sigma_closed(state.get_vector(), precision)


assert N_OPS == 24
