"""TPSCI driver on the GPU sigma build.

tpsci_ci (src/tpsci.jl:39-363, incremental-sigma branch), compute_pt2_energy
(src/tpsci_pt2_energy.jl:10-233) and compute_pt1_wavefunction
(src/tpsci_pt1_wavefunction.jl:11-83), with every sigma-sized operation on the device:
the variational solve is the device Davidson (fcg_davidson, the tps_ci_davidson
solve), the FOIS sigma is fcg_sigma_open, the PT denominators are fcg_diagonal("Hcmf"),
<0|H0|0> is a closed sigma of the 1-body "Hcmf" operator.  The TPSCIstate bookkeeping
(sparse adds, overlaps, clipping) is host work, as it is in the reference.
"""
from __future__ import annotations

import numpy as np

from . import pack
from .gpu import FcgError, GpuSigma
from .state import (TPSCIstate, add_state, clip, copy_state, minus_state, overlap, project_out,
                    state_from_rows, times_matrix, zero_state)
from .terms import extract_1body_operator


class GpuTPSCI:
    def __init__(self, ops, bases, ham, device: int = 0, precision: str = "fp64", store_blocks: float = 16e9):
        """store_blocks: largest stored Hamiltonian (bytes) a variational solve may keep on
        the device (fcg_cache_hamiltonian); a larger one, or 0, solves with the direct build."""
        self.N = ham.n_clusters
        self.precision = precision
        self.store_blocks = store_blocks
        self.H = GpuSigma(device)
        self.H.set_problem(ops, bases, ham)
        self.H0 = GpuSigma(device)
        self.H0.set_problem(ops, bases, extract_1body_operator(ham, "Hcmf"))
        self._indexed = {}

    def close(self):
        self.H.close()
        self.H0.close()

    # ---- primitives ----------------------------------------------------------------------
    def _index(self, ctx, s: TPSCIstate):
        f, c, v, _ = pack.pack_state(s)
        ctx.state_set(f, c)
        return v

    def solve(self, s: TPSCIstate, tol=1e-8, max_iter=200, max_ss_vecs=12, lindep=1e-12):
        """Lowest R eigenpairs of H within s's configurations (tps_ci_davidson)."""
        v = self._index(self.H, s)
        if self.store_blocks > 0:  # every sigma of this solve reads the stored blocks
            try:
                self.H.cache_hamiltonian(self.store_blocks)
            except FcgError:
                pass
        e, X, res, it = self.H.davidson(v, max_iter=max_iter, max_ss_vecs=max_ss_vecs, tol=tol, lindep=lindep,
                                        precision=self.precision)
        self.H.cache_hamiltonian(0)
        out = copy_state(s)
        out.set_vector(X)
        return e, out, res

    def expectation0(self, s: TPSCIstate):
        """<v_r|H0|v_r> with H0 = sum_c Hcmf_c (compute_expectation_value_parallel)."""
        v = self._index(self.H0, s)
        hv = self.H0.sigma_closed(v, "fp64")
        return np.einsum("ir,ir->r", v, hv)

    def open_sigma(self, s: TPSCIstate, thresh: float, nbody: int = 4) -> TPSCIstate:
        v = self._index(self.H, s)
        of, oc, ov = self.H.sigma_open(v, thresh, nbody)
        return state_from_rows(self.N, s.R, of, oc, ov)

    def diagonal_cmf(self, s: TPSCIstate):
        if len(s) == 0:
            return np.zeros(0)
        self._index(self.H, s)
        return self.H.diagonal("Hcmf")

    # ---- drivers -------------------------------------------------------------------------
    def tpsci_ci(self, ci_vector: TPSCIstate, thresh_cipsi=1e-2, thresh_foi=1e-6, thresh_asci=None, max_iter=10,
                 conv_thresh=1e-4, nbody=4, ci_conv=1e-8, ci_max_iter=200, ci_max_ss_vecs=12,
                 ci_lindep_thresh=1e-12, log=None):
        R = ci_vector.R
        vec_var = copy_state(ci_vector)
        vec_pt = copy_state(ci_vector)
        zero_state(vec_pt)
        e0_last = np.zeros(R)
        vec_asci_old = TPSCIstate(self.N, R)
        sig_old = TPSCIstate(self.N, R)
        e0 = None
        for it in range(1, max_iter + 1):
            if it > 1:
                zero_state(vec_pt)
                add_state(vec_var, vec_pt)
            e0, vec_var, _ = self.solve(vec_var, tol=ci_conv, max_iter=ci_max_iter, max_ss_vecs=ci_max_ss_vecs,
                                        lindep=ci_lindep_thresh)
            efock = self.expectation0(vec_var)
            vec_asci = copy_state(vec_var)
            if thresh_asci is not None:
                clip(vec_asci, thresh_asci)
            S = overlap(vec_asci_old, vec_asci)
            sig = times_matrix(sig_old, S)
            del_v0 = minus_state(vec_asci, times_matrix(vec_asci_old, S))
            vec_asci_old = copy_state(vec_asci)
            del_sig = self.open_sigma(del_v0, thresh_foi, nbody)
            add_state(sig, del_sig)
            sig_old = copy_state(sig)
            project_out(sig, vec_asci)
            hd = self.diagonal_cmf(sig)
            sig_v = sig.get_vector() if len(sig) else np.zeros((0, R))
            norms = np.linalg.norm(vec_asci.get_vector(), axis=0)
            v_pt = np.zeros_like(sig_v)
            e2 = np.zeros(R)
            for r in range(R):
                denom = 1.0 / (efock[r] / (norms[r] * norms[r]) - hd)
                v_pt[:, r] = denom * sig_v[:, r]
                e2[r] = float(np.sum(sig_v[:, r] * v_pt[:, r]))
            vec_pt = copy_state(sig)
            if len(vec_pt):
                vec_pt.set_vector(v_pt)
            clip(vec_pt, thresh_cipsi)
            if log is not None:
                log.append(dict(it=it, dim=len(vec_var), foi=len(sig), e0=e0.copy(), e2=e2.copy()))
            if np.max(np.abs(e0_last - e0)) < conv_thresh:
                break
            e0_last = e0.copy()
        return e0, vec_var

    def pt2_energy(self, ci_vector: TPSCIstate, thresh_foi=1e-9, nbody=4):
        """compute_pt2_energy with H0 = Hcmf: sum_x sigma_x^2 / (E0 - Hd_x) over the FOIS."""
        v = copy_state(ci_vector)
        V = v.get_vector()
        Q, _ = np.linalg.qr(V)
        Q = Q * np.sign(np.sum(Q * V, axis=0))
        v.set_vector(Q)
        e0 = self.expectation0(v)
        sig = self.open_sigma(v, thresh_foi, nbody)
        project_out(sig, v)
        hd = self.diagonal_cmf(sig)
        sv = sig.get_vector()
        return np.array([np.sum(sv[:, r] ** 2 / (e0[r] - hd)) for r in range(v.R)])

    def pt1_wavefunction(self, ci_vector: TPSCIstate, thresh_foi=1e-8, nbody=4, E0=None):
        """compute_pt1_wavefunction with H0 = Hcmf: the FOIS sigma with the variational
        configurations removed, divided by (E0_r / |v_r|^2 - Hd); returns (e2, PT1 state).
        E0 = <v_r|H0|v_r> unless given (src/tpsci_pt1_wavefunction.jl:11-83)."""
        R = ci_vector.R
        norms = np.linalg.norm(ci_vector.get_vector(), axis=0)
        sig = self.open_sigma(ci_vector, thresh_foi, nbody)
        project_out(sig, ci_vector)
        hd = self.diagonal_cmf(sig)
        if E0 is None:
            E0 = self.expectation0(ci_vector)
        sig_v = sig.get_vector() if len(sig) else np.zeros((0, R))
        v_pt = np.zeros_like(sig_v)
        e2 = np.zeros(R)
        for r in range(R):
            denom = 1.0 / (E0[r] / (norms[r] * norms[r]) - hd)
            v_pt[:, r] = denom * sig_v[:, r]
            e2[r] = float(np.sum(sig_v[:, r] * v_pt[:, r]))
        if len(sig):
            sig.set_vector(v_pt)
        return e2, sig
