"""TPSCI driver on the GPU sigma build.

tpsci_ci (src/tpsci.jl:39-363, incremental-sigma branch), compute_pt2_energy
(src/tpsci_pt2_energy.jl:10-233) and compute_pt1_wavefunction
(src/tpsci_pt1_wavefunction.jl:11-83), with every sigma-sized operation on the device:
the variational solve is the device Davidson (fcg_davidson, the tps_ci_davidson
solve), the FOIS sigma is fcg_sigma_open, the PT denominators are fcg_diagonal("Hcmf"),
<0|H0|0> is a closed sigma of the 1-body "Hcmf" operator.  The TPSCIstate bookkeeping
(sparse adds, overlaps, clipping) is host work, as it is in the reference; it runs on the
array form FlatTPSCI (vectorised, the same row order as TPSCIstate), since first-order
spaces reach millions of configurations.  Inputs and results are TPSCIstates.
"""
from __future__ import annotations

import numpy as np

from .gpu import FcgError, GpuSigma
from .state import FlatTPSCI, SectorRegistry, TPSCIstate
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
        self.reg = SectorRegistry(self.N, [max(v.shape[1] for v in b.basis.values()) for b in bases])

    def close(self):
        self.H.close()
        self.H0.close()

    # ---- primitives (FlatTPSCI in, FlatTPSCI out) ----------------------------------------
    def _flat(self, s) -> FlatTPSCI:
        return s if isinstance(s, FlatTPSCI) else FlatTPSCI.from_state(self.reg, s)

    def _index(self, ctx, s: FlatTPSCI, plan: bool = True):
        f, c, v = s.rows()
        ctx.state_set(np.ascontiguousarray(f), np.ascontiguousarray(c), plan=plan)
        return v

    def solve(self, s, tol=1e-8, max_iter=200, max_ss_vecs=12, lindep=1e-12):
        """Lowest R eigenpairs of H within s's configurations (tps_ci_davidson)."""
        fs = self._flat(s)
        v = self._index(self.H, fs)
        if self.store_blocks > 0:  # every sigma of this solve reads the stored blocks
            try:
                self.H.cache_hamiltonian(self.store_blocks)
            except FcgError:
                pass
        e, X, res, it = self.H.davidson(v, max_iter=max_iter, max_ss_vecs=max_ss_vecs, tol=tol, lindep=lindep,
                                        precision=self.precision)
        out = fs.copy()
        out.set_vector(X)
        return e, (out if isinstance(s, FlatTPSCI) else out.to_state()), res

    def expectation0(self, s):
        """<v_r|H0|v_r> with H0 = sum_c Hcmf_c (compute_expectation_value_parallel)."""
        v = self._index(self.H0, self._flat(s))
        hv = self.H0.sigma_closed(v, "fp64")
        return np.einsum("ir,ir->r", v, hv)

    def open_sigma(self, s, thresh: float, nbody: int = 4):
        fs = self._flat(s)
        v = self._index(self.H, fs, plan=False)  # the open sigma needs the rows and sectors only
        of, oc, ov = self.H.sigma_open(v, thresh, nbody)
        out = FlatTPSCI.from_rows(self.reg, fs.R, of, oc, ov)
        return out if isinstance(s, FlatTPSCI) else out.to_state()

    def diagonal_cmf(self, s):
        fs = self._flat(s)
        if len(fs) == 0:
            return np.zeros(0)
        self._index(self.H, fs, plan=False)  # compute_diagonal needs the rows and sectors only
        return self.H.diagonal("Hcmf")

    # ---- drivers -------------------------------------------------------------------------
    def tpsci_ci(self, ci_vector: TPSCIstate, thresh_cipsi=1e-2, thresh_foi=1e-6, thresh_asci=None, max_iter=10,
                 conv_thresh=1e-4, nbody=4, ci_conv=1e-8, ci_max_iter=200, ci_max_ss_vecs=12,
                 ci_lindep_thresh=1e-12, log=None):
        R = ci_vector.R
        vec_var = self._flat(ci_vector)
        vec_pt = vec_var.copy()
        vec_pt.zero()
        e0_last = np.zeros(R)
        vec_asci_old = FlatTPSCI(self.reg, R)
        sig_old = FlatTPSCI(self.reg, R)
        e0 = None
        for it in range(1, max_iter + 1):
            if it > 1:
                vec_pt.zero()
                vec_var.add(vec_pt)
            e0, vec_var, _ = self.solve(vec_var, tol=ci_conv, max_iter=ci_max_iter, max_ss_vecs=ci_max_ss_vecs,
                                        lindep=ci_lindep_thresh)
            efock = self.expectation0(vec_var)
            vec_asci = vec_var.copy()
            if thresh_asci is not None:
                vec_asci.clip(thresh_asci)
            S = vec_asci_old.overlap(vec_asci)
            sig = sig_old.times_matrix(S)
            del_v0 = vec_asci.minus(vec_asci_old.times_matrix(S))
            vec_asci_old = vec_asci.copy()
            del_sig = self.open_sigma(del_v0, thresh_foi, nbody)
            sig.add(del_sig)
            sig_old = sig.copy()
            sig.project_out(vec_asci)
            hd = self.diagonal_cmf(sig)
            sig_v = sig.get_vector() if len(sig) else np.zeros((0, R))
            norms = np.linalg.norm(vec_asci.get_vector(), axis=0)
            v_pt = np.zeros_like(sig_v)
            e2 = np.zeros(R)
            # A configuration whose Hcmf diagonal equals E0/|v|^2 exactly (degenerate local states,
            # e.g. the spin-flipped partner of the reference) gets an infinite (sigma != 0) or NaN
            # (sigma == 0) first-order coefficient, as 1.0 ./ (...) gives in the reference
            # (src/tpsci.jl:323); clip! keeps such a row (no |c| < thresh holds), so it always enters
            # the variational space, here as there.  Only the floating-point warning is silenced.
            with np.errstate(divide="ignore", invalid="ignore"):
                for r in range(R):
                    denom = 1.0 / (efock[r] / (norms[r] * norms[r]) - hd)
                    v_pt[:, r] = denom * sig_v[:, r]
                    e2[r] = float(np.sum(sig_v[:, r] * v_pt[:, r]))
            vec_pt = sig.copy()
            if len(vec_pt):
                vec_pt.set_vector(v_pt)
            vec_pt.clip(thresh_cipsi)
            if log is not None:
                log.append(dict(it=it, dim=len(vec_var), foi=len(sig), e0=e0.copy(), e2=e2.copy()))
            if np.max(np.abs(e0_last - e0)) < conv_thresh:
                break
            e0_last = e0.copy()
        return e0, vec_var.to_state()

    def pt2_energy(self, ci_vector: TPSCIstate, thresh_foi=1e-9, nbody=4):
        """compute_pt2_energy with H0 = Hcmf: sum_x sigma_x^2 / (E0 - Hd_x) over the FOIS."""
        v = self._flat(ci_vector).copy()
        V = v.get_vector()
        Q, _ = np.linalg.qr(V)
        Q = Q * np.sign(np.sum(Q * V, axis=0))
        v.set_vector(Q)
        e0 = self.expectation0(v)
        sig = self.open_sigma(v, thresh_foi, nbody)
        sig.project_out(v)
        hd = self.diagonal_cmf(sig)
        sv = sig.get_vector()
        return np.array([np.sum(sv[:, r] ** 2 / (e0[r] - hd)) for r in range(v.R)])

    def pt1_wavefunction(self, ci_vector: TPSCIstate, thresh_foi=1e-8, nbody=4, E0=None):
        """compute_pt1_wavefunction with H0 = Hcmf: the FOIS sigma with the variational
        configurations removed, divided by (E0_r / |v_r|^2 - Hd); returns (e2, PT1 state).
        E0 = <v_r|H0|v_r> unless given (src/tpsci_pt1_wavefunction.jl:11-83)."""
        R = ci_vector.R
        fv = self._flat(ci_vector)
        norms = np.linalg.norm(fv.get_vector(), axis=0)
        sig = self.open_sigma(fv, thresh_foi, nbody)
        sig.project_out(fv)
        hd = self.diagonal_cmf(sig)
        if E0 is None:
            E0 = self.expectation0(fv)
        sig_v = sig.get_vector() if len(sig) else np.zeros((0, R))
        v_pt = np.zeros_like(sig_v)
        e2 = np.zeros(R)
        for r in range(R):
            denom = 1.0 / (E0[r] / (norms[r] * norms[r]) - hd)
            v_pt[:, r] = denom * sig_v[:, r]
            e2[r] = float(np.sum(sig_v[:, r] * v_pt[:, r]))
        if len(sig):
            sig.set_vector(v_pt)
        return e2, sig.to_state()
