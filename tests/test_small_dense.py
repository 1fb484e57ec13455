"""Host linear algebra of the device Davidson (csrc/small_dense.h) against numpy: the
Rayleigh-Ritz eigensolver and the Cholesky factor inverse used for the new directions."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("sd") / "libsd.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", os.path.join(ROOT, "tests", "small_dense_shim.cpp"),
                    "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    dp = ctypes.POINTER(ctypes.c_double)
    L.sd_symeig.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_int]
    L.sd_chol_inverse.argtypes = [ctypes.c_int, dp, ctypes.c_int, ctypes.c_double, dp]
    L.sd_spd_condition.argtypes = [ctypes.c_int, dp, ctypes.c_int]
    L.sd_spd_condition.restype = ctypes.c_double
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def symeig(L, A, nvec=-1):
    k = A.shape[0]
    nv = k if nvec < 0 else nvec
    a = np.asfortranarray(A.copy())
    w = np.zeros(max(k, 1))
    Z = np.zeros(max(k * nv, 1))
    rc = L.sd_symeig(k, _p(a), _p(w), _p(Z), nvec)
    return rc, w[:k], Z[:k * nv].reshape((k, nv), order="F")


@pytest.mark.parametrize("k", [1, 2, 3, 5, 12, 48, 97, 200])
def test_symeig_random(lib, k):
    rng = np.random.default_rng(k)
    B = rng.standard_normal((k, k))
    A = (B + B.T) / 2 + np.diag(np.arange(k) * 0.3)
    rc, w, Z = symeig(lib, A)
    assert rc == 0
    wr = np.linalg.eigvalsh(A)
    scale = max(1.0, np.abs(wr).max())
    assert np.abs(w - wr).max() < 1e-12 * scale * k
    assert np.abs(Z.T @ Z - np.eye(k)).max() < 1e-12 * k
    assert np.abs(A @ Z - Z * w).max() < 1e-12 * scale * k


@pytest.mark.parametrize("case", ["zero", "identity", "diagonal", "degenerate", "tridiagonal", "lower_only"])
def test_symeig_structured(lib, case):
    k = 20
    rng = np.random.default_rng(5)
    if case == "zero":
        A = np.zeros((k, k))
    elif case == "identity":
        A = np.eye(k) * 3.0
    elif case == "diagonal":
        A = np.diag(rng.standard_normal(k))
    elif case == "degenerate":  # eigenvalues 1 (x10) and -2 (x10) in a random basis
        Q, _ = np.linalg.qr(rng.standard_normal((k, k)))
        A = Q @ np.diag([1.0] * 10 + [-2.0] * 10) @ Q.T
    elif case == "tridiagonal":
        A = np.diag(rng.standard_normal(k)) + np.diag(np.ones(k - 1), 1) + np.diag(np.ones(k - 1), -1)
    else:
        B = rng.standard_normal((k, k))
        A = (B + B.T) / 2
    A_in = A.copy()
    if case == "lower_only":  # only the lower triangle is read
        A_in = np.tril(A) + np.triu(np.full((k, k), 1e9), 1)
    rc, w, Z = symeig(lib, A_in)
    assert rc == 0
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - np.linalg.eigvalsh(A)).max() < 1e-12 * max(1.0, np.abs(A).max()) * k
    assert np.abs(Z.T @ Z - np.eye(k)).max() < 1e-12 * k
    assert np.abs(A @ Z - Z * w).max() < 1e-11 * max(1.0, np.abs(A).max())


@pytest.mark.parametrize("k,nvec", [(48, 4), (200, 16), (30, 1), (7, 0)])
def test_symeig_lowest_vectors(lib, k, nvec):
    rng = np.random.default_rng(k + nvec)
    B = rng.standard_normal((k, k))
    A = (B + B.T) / 2
    rc, w, Z = symeig(lib, A, nvec)
    assert rc == 0 and Z.shape == (k, nvec)
    wr, Zr = np.linalg.eigh(A)
    assert np.abs(w - wr).max() < 1e-12 * k * max(1.0, np.abs(wr).max())
    if nvec:
        assert np.abs(Z.T @ Z - np.eye(nvec)).max() < 1e-12 * k
        assert np.abs(A @ Z - Z * w[:nvec]).max() < 1e-12 * k * max(1.0, np.abs(wr).max())


def test_symeig_nonfinite_reports(lib):
    A = np.eye(4)
    A[2, 1] = np.nan
    rc, _, _ = symeig(lib, A)
    assert rc == 1


def test_chol_inverse(lib):
    rng = np.random.default_rng(3)
    m = 6
    X = rng.standard_normal((40, m))
    G = np.asfortranarray(X.T @ X)
    Ri = np.zeros((m, m), order="F")
    good = lib.sd_chol_inverse(m, _p(G), m, 1e-8, _p(Ri))
    assert good == m
    Q = X @ Ri
    assert np.abs(Q.T @ Q - np.eye(m)).max() < 1e-12
    assert np.allclose(np.triu(Ri), Ri)
    # a dependent column stops the factorisation there
    X2 = np.hstack([X[:, :3], X[:, :1] + X[:, 1:2], X[:, 3:]])
    G2 = np.asfortranarray(X2.T @ X2)
    Ri2 = np.zeros((m + 1, m + 1), order="F")
    good2 = lib.sd_chol_inverse(m + 1, _p(G2), m + 1, 1e-8, _p(Ri2))
    assert good2 == 3


def test_spd_condition(lib):
    G = np.asfortranarray(np.diag([1.0, 10.0, 100.0]))
    assert abs(lib.sd_spd_condition(3, _p(G), 3) - 100.0) < 1e-9
    G2 = np.asfortranarray(np.diag([1.0, 0.0]))
    assert lib.sd_spd_condition(2, _p(G2), 2) == float("inf")


# ---- the cooperative Tucker routines of csrc/tucker_small.cuh, run with one thread ----------
def _coop(lib):
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)
    lib.sd_coop_jacobi.argtypes = [ctypes.c_int, dp, dp, dp, ip]
    lib.sd_coop_mode_gram.argtypes = [dp, ip, ctypes.c_int, ctypes.c_int, dp]
    lib.sd_coop_mode_product_t.argtypes = [dp, ip, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, dp]
    return lib


@pytest.mark.parametrize("n,case", [(1, "rand"), (2, "rand"), (7, "rand"), (36, "rand"), (64, "rand"),
                                    (20, "degenerate"), (12, "zero")])
def test_coop_jacobi(lib, n, case):
    L = _coop(lib)
    rng = np.random.default_rng(n)
    if case == "rand":
        B = rng.standard_normal((n, n))
        A = B @ B.T
    elif case == "degenerate":
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        A = Q @ np.diag([2.0] * (n // 2) + [0.5] * (n - n // 2)) @ Q.T
    else:
        A = np.zeros((n, n))
    a = np.asfortranarray(A.copy())
    w = np.zeros(n)
    V = np.zeros((n, n), order="F")
    perm = np.zeros(n, dtype=np.int32)
    L.sd_coop_jacobi(n, _p(a), _p(w), _p(V), perm.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    ws = w[perm]
    assert np.all(np.diff(ws) <= 1e-12 * max(1.0, abs(ws).max()))
    np.testing.assert_allclose(np.sort(ws), np.linalg.eigvalsh(A), atol=1e-11 * max(1.0, np.abs(A).max()))
    Vs = V[:, perm]
    np.testing.assert_allclose(Vs.T @ Vs, np.eye(n), atol=1e-12)
    np.testing.assert_allclose(A @ Vs, Vs * ws, atol=1e-10 * max(1.0, np.abs(A).max()))


def test_coop_mode_gram_and_product(lib):
    L = _coop(lib)
    rng = np.random.default_rng(2)
    dims = np.array([3, 4, 5], dtype=np.int32)
    T = rng.standard_normal(tuple(dims))
    a = np.asfortranarray(T).reshape(-1, order="F").copy()
    for m in range(3):
        d = dims[m]
        G = np.zeros((d, d), order="F")
        L.sd_coop_mode_gram(_p(a), dims.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 3, m, _p(G))
        Mm = np.moveaxis(T, m, 0).reshape(d, -1)
        np.testing.assert_allclose(G, Mm @ Mm.T, atol=1e-12)
        k = 2
        M = np.asfortranarray(rng.standard_normal((d, k)))
        out = np.zeros(int(np.prod(dims)) // d * k)
        L.sd_coop_mode_product_t(_p(a), dims.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 3, m, _p(M), d, k,
                                 _p(out))
        ref = np.moveaxis(np.tensordot(T, M, axes=([m], [0])), -1, m)
        np.testing.assert_allclose(out.reshape(ref.shape, order="F"), ref, atol=1e-12)
