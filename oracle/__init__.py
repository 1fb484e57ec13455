"""CPU oracle for the TPSCI sigma build -- TEST INFRASTRUCTURE, not product.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker / timed CPU reference.  The product
(fermicg_gb300 + its CUDA library) never imports it.

The C++ restatement lives in oracle.cpp (see its header for the reference
file:line map).  `fci.py` holds an independent determinant-FCI check.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liboracle.so")
_lib = None


def build(force=False):
    """Compile oracle.cpp with g++ -O3 -fopenmp into oracle/_build/liboracle.so."""
    src = os.path.join(_HERE, "oracle.cpp")
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= os.path.getmtime(src):
        return _SO
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _SO + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp])
    os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.oracle_set_problem.restype = ctypes.c_int
        L.oracle_set_problem.argtypes = [ctypes.c_int, P, ctypes.c_int, i64, P, P, ctypes.c_int, P, P,
                                         ctypes.c_int, P]
        L.oracle_sigma_closed.argtypes = [ctypes.c_int, i64, P, P, ctypes.c_int, P, P, i64, i64, ctypes.c_int]
        L.oracle_diagonal_H.argtypes = [ctypes.c_int, i64, P, P, P]
        L.oracle_build_H.argtypes = [ctypes.c_int, i64, P, P, P]
        L.oracle_diagonal_op.argtypes = [ctypes.c_int, i64, P, P, ctypes.c_int, P]
        L.oracle_sigma_open.argtypes = [ctypes.c_int, i64, P, P, ctypes.c_int, P, ctypes.c_double, ctypes.c_int, i64, i64,
                                        ctypes.c_int]
        L.oracle_sigma_open.restype = i64
        L.oracle_open_fetch.argtypes = [ctypes.c_int, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """Holds the packed problem (numpy buffers must outlive the C side)."""

    def __init__(self, pops, pterms):
        from fermicg_gb300.local_fci import N_OPS  # op-id table shared with the packer
        self._keep = []
        L = lib()
        self.N = int(pops.n_clusters)
        opb = np.ascontiguousarray(pops.table, dtype=np.int64)
        opd = np.ascontiguousarray(pops.data, dtype=np.float64)
        trm = np.ascontiguousarray(pterms.table, dtype=np.int32)
        ints = np.ascontiguousarray(pterms.ints, dtype=np.float64)
        trans = np.ascontiguousarray(pterms.transfers, dtype=np.int16)
        norb = np.ascontiguousarray(pops.cluster_norb, dtype=np.int32)
        self._keep = [opb, opd, trm, ints, trans, norb]
        rc = L.oracle_set_problem(self.N, _p(norb), N_OPS, opb.shape[0], _p(opb), _p(opd), trm.shape[0], _p(trm),
                                  _p(ints), trans.shape[0], _p(trans))
        if rc < 0:
            raise RuntimeError("oracle_set_problem failed")
        self.h = rc

    def sigma_closed(self, focks, cfgs, coeffs, rows=None, n_threads=0):
        """tps_ci_matvec; coeffs (n_cfg, R) -> sigma (n_cfg, R)."""
        n, R = coeffs.shape
        f = np.ascontiguousarray(focks, dtype=np.int16)
        c = np.ascontiguousarray(cfgs, dtype=np.int16)
        cf = np.asfortranarray(coeffs, dtype=np.float64)
        sig = np.zeros((n, R), dtype=np.float64, order="F")
        r0, r1 = (0, n) if rows is None else rows
        rc = lib().oracle_sigma_closed(self.h, n, _p(f), _p(c), R, _p(cf), _p(sig), r0, r1, n_threads)
        if rc != 0:
            raise RuntimeError("oracle_sigma_closed failed")
        return np.ascontiguousarray(sig)

    def build_H(self, focks, cfgs):
        """Dense H over the configurations (build_full_H)."""
        n = focks.shape[0]
        f = np.ascontiguousarray(focks, dtype=np.int16)
        c = np.ascontiguousarray(cfgs, dtype=np.int16)
        H = np.zeros((n, n))
        if lib().oracle_build_H(self.h, n, _p(f), _p(c), _p(H)) != 0:
            raise RuntimeError("oracle_build_H failed")
        return H

    def diagonal_H(self, focks, cfgs):
        n = focks.shape[0]
        f = np.ascontiguousarray(focks, dtype=np.int16)
        c = np.ascontiguousarray(cfgs, dtype=np.int16)
        hd = np.zeros(n)
        lib().oracle_diagonal_H(self.h, n, _p(f), _p(c), _p(hd))
        return hd

    def diagonal_op(self, focks, cfgs, op_id):
        n = focks.shape[0]
        f = np.ascontiguousarray(focks, dtype=np.int16)
        c = np.ascontiguousarray(cfgs, dtype=np.int16)
        hd = np.zeros(n)
        rc = lib().oracle_diagonal_op(self.h, n, _p(f), _p(c), op_id, _p(hd))
        if rc != 0:
            raise RuntimeError("missing diagonal block")
        return hd

    def sigma_open(self, focks, cfgs, coeffs, thresh, nbody=4, rows=None, n_threads=0):
        """open_matvec_thread (prescreen off): returns dict (fock, cfg) -> coeff row."""
        n, R = coeffs.shape
        f = np.ascontiguousarray(focks, dtype=np.int16)
        c = np.ascontiguousarray(cfgs, dtype=np.int16)
        cf = np.asfortranarray(coeffs, dtype=np.float64)
        r0, r1 = (0, n) if rows is None else rows
        m = lib().oracle_sigma_open(self.h, n, _p(f), _p(c), R, _p(cf), float(thresh), nbody, r0, r1, n_threads)
        if m < 0:
            raise RuntimeError("oracle_sigma_open failed")
        of = np.zeros((m, self.N, 2), dtype=np.int16)
        oc = np.zeros((m, self.N), dtype=np.int16)
        ov = np.zeros((m, R), dtype=np.float64)
        lib().oracle_open_fetch(self.h, _p(of), _p(oc), _p(ov))
        return of, oc, ov
