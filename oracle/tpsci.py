"""CPU restatement of the TPSCI driver -- TEST INFRASTRUCTURE ONLY.

tpsci_ci (src/tpsci.jl:39-363), incremental-sigma branch, with the direct
solver (tps_ci_direct, src/tpsci_outer.jl:165-300, exact dense eigensolve),
and compute_pt2_energy (src/tpsci_pt2_energy.jl:10-233).  Every sigma, dense H,
diagonal and FOIS sigma comes from the C++ oracle.  Used to pin the oracle
against the reference's TPSCI energies (test/test_tpsci.jl) and as the checker
of the GPU TPSCI driver.
"""
from __future__ import annotations

import numpy as np

from fermicg_gb300 import pack
from fermicg_gb300.state import TPSCIstate
from fermicg_gb300.terms import extract_1body_operator

from . import Oracle


# ---- TPSCIstate algebra (src/type_TPSCIstate.jl) ------------------------------------------

def _copy(s: TPSCIstate) -> TPSCIstate:
    out = TPSCIstate(s.n_clusters, s.R)
    for f, cs in s.data.items():
        if cs:
            out.data[f] = {c: v.copy() for c, v in cs.items()}
    return out


def _add(s1: TPSCIstate, s2: TPSCIstate):
    """add! (type_TPSCIstate.jl:617)"""
    for f, cs in s2.data.items():
        if f in s1.data:
            d = s1.data[f]
            for c, v in cs.items():
                if c in d:
                    d[c] = d[c] + v
                else:
                    d[c] = v.copy()
        else:
            s1.data[f] = {c: v.copy() for c, v in cs.items()}


def _scale(s, a):
    for cs in s.data.values():
        for c in cs:
            cs[c] = cs[c] * a


def _times(s: TPSCIstate, C) -> TPSCIstate:
    """A * C (type_TPSCIstate.jl:456)"""
    out = _copy(s)
    if len(out):
        out.set_vector(s.get_vector() @ C)
    return out


def _minus(A, B):
    """A - B (type_TPSCIstate.jl:478): copy of -B, then add A"""
    C = _copy(B)
    _scale(C, -1.0)
    _add(C, A)
    return C


def _overlap(v1, v2):
    """overlap (type_TPSCIstate.jl:416)"""
    R = v2.R
    S = np.zeros((R, R))
    for f, cs in v2.data.items():
        if f not in v1.data:
            continue
        d1 = v1.data[f]
        for c, v in cs.items():
            if c in d1:
                S += np.outer(d1[c], v)
    return S


def _project_out(v, w):
    """project_out! (tpsci_outer.jl:869)"""
    for f, cs in w.data.items():
        if f in v.data:
            for c in cs:
                v.data[f].pop(c, None)
            if not v.data[f]:
                del v.data[f]


def _clip(s, thresh):
    """clip! (type_TPSCIstate.jl:589)"""
    for f in list(s.data):
        cs = s.data[f]
        for c in list(cs):
            if np.all(np.abs(cs[c]) < thresh):
                del cs[c]
        if not cs:
            del s.data[f]


def _zero(s):
    for cs in s.data.values():
        for c in cs:
            cs[c] = np.zeros(s.R)


def _sorted_by_sector(s: TPSCIstate) -> TPSCIstate:
    return s  # TPSCIstate rows are already grouped by sector (dict of dicts)


def _from_open(N, R, of, oc, ov):
    out = TPSCIstate(N, R)
    for i in range(len(of)):
        f = tuple((int(a), int(b)) for a, b in of[i])
        out.add_fockconfig(f)
        out.data[f][tuple(int(x) for x in oc[i])] = ov[i].copy()
    return out


class OracleTPSCI:
    def __init__(self, ops, bases, ham):
        self.N = ham.n_clusters
        self.O = Oracle(pack.pack_ops(ops, bases), pack.pack_terms(ham))
        self.O0 = Oracle(pack.pack_ops(ops, bases), pack.pack_terms(extract_1body_operator(ham, "Hcmf")))
        self.hcmf = pack.op_id_of("Hcmf")

    def _flat(self, s):
        f, c, v, _ = pack.pack_state(s)
        return f, c, v

    def expectation(self, s, zeroth=False):
        """compute_expectation_value_parallel (tpsci_outer.jl:601): <v_r|H|v_r> per root."""
        f, c, v = self._flat(s)
        O = self.O0 if zeroth else self.O
        hv = O.sigma_closed(f, c, v)
        return np.einsum("ir,ir->r", v, hv)

    def open_sigma(self, s, thresh, nbody=4):
        f, c, v = self._flat(s)
        of, oc, ov = self.O.sigma_open(f, c, v, thresh, nbody=nbody)
        return _from_open(self.N, s.R, of, oc, ov)

    def direct(self, s):
        """tps_ci_direct: lowest R eigenpairs of the dense H over the configurations."""
        f, c, v = self._flat(s)
        H = self.O.build_H(f, c)
        w, V = np.linalg.eigh(0.5 * (H + H.T))
        out = _copy(s)
        out.set_vector(V[:, :s.R])
        return w[:s.R].copy(), out

    def tpsci_ci(self, ci_vector, thresh_cipsi=1e-2, thresh_foi=1e-6, thresh_asci=None, max_iter=10,
                 conv_thresh=1e-4, nbody=4, log=None):
        """tpsci_ci (tpsci.jl:39-363), incremental = true, direct solver."""
        R = ci_vector.R
        vec_var = _copy(ci_vector)
        vec_pt = _copy(ci_vector)
        _zero(vec_pt)
        e0_last = np.zeros(R)
        vec_asci_old = TPSCIstate(self.N, R)
        sig_old = TPSCIstate(self.N, R)
        e0 = e2 = None
        for it in range(1, max_iter + 1):
            if it > 1:
                _zero(vec_pt)
                _add(vec_var, vec_pt)
            e0, vec_var = self.direct(vec_var)
            efock = self.expectation(vec_var, zeroth=True)
            vec_asci = _copy(vec_var)
            if thresh_asci is not None:
                _clip(vec_asci, thresh_asci)
            S = _overlap(vec_asci_old, vec_asci)
            sig = _times(sig_old, S)
            del_v0 = _minus(vec_asci, _times(vec_asci_old, S))
            vec_asci_old = _copy(vec_asci)
            del_sig = self.open_sigma(del_v0, thresh_foi, nbody)
            _add(sig, del_sig)
            sig_old = _copy(sig)
            _project_out(sig, vec_asci)
            f, c, sig_v = self._flat(sig)
            hd = self.O.diagonal_op(f, c, self.hcmf) if len(sig) else np.zeros(0)
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
            vec_pt = _copy(sig)
            if len(vec_pt):
                vec_pt.set_vector(v_pt)
            _clip(vec_pt, thresh_cipsi)
            if log is not None:
                log.append(dict(it=it, dim=len(vec_var), foi=len(sig), e0=e0.copy(), e2=e2.copy()))
            if np.max(np.abs(e0_last - e0)) < conv_thresh:
                break
            e0_last = e0.copy()
        return e0, vec_var

    def pt2_energy(self, ci_vector, thresh_foi=1e-9, nbody=4):
        """compute_pt2_energy (tpsci_pt2_energy.jl:10-233) with H0 = Hcmf."""
        v = _copy(ci_vector)
        V = v.get_vector()
        Q, _ = np.linalg.qr(V)  # orthonormalize! is Gram-Schmidt; same span, signs fixed below
        Q = Q * np.sign(np.sum(Q * V, axis=0))
        v.set_vector(Q)
        e0 = self.expectation(v, zeroth=True)
        sig = self.open_sigma(v, thresh_foi, nbody)
        _project_out(sig, v)
        f, c, sv = self._flat(sig)
        hd = self.O.diagonal_op(f, c, self.hcmf)
        return np.array([np.sum(sv[:, r] ** 2 / (e0[r] - hd)) for r in range(v.R)])

    def pt1_wavefunction(self, ci_vector, thresh_foi=1e-8, nbody=4, E0=None):
        """compute_pt1_wavefunction (tpsci_pt1_wavefunction.jl:11-83) with H0 = Hcmf:
        v_pt = sigma / (E0_r / |v_r|^2 - Hd) on the FOIS minus the variational configurations,
        e2_r = sum sigma_r * v_pt_r; returns (e2, PT1 state)."""
        R = ci_vector.R
        norms = np.linalg.norm(ci_vector.get_vector(), axis=0)
        sig = self.open_sigma(ci_vector, thresh_foi, nbody)
        _project_out(sig, ci_vector)
        f, c, sig_v = self._flat(sig)
        hd = self.O.diagonal_op(f, c, self.hcmf) if len(sig) else np.zeros(0)
        if E0 is None:
            E0 = self.expectation(ci_vector, zeroth=True)
        v_pt = np.zeros_like(sig_v)
        e2 = np.zeros(R)
        for r in range(R):
            denom = 1.0 / (E0[r] / (norms[r] * norms[r]) - hd)
            v_pt[:, r] = denom * sig_v[:, r]
            e2[r] = float(np.sum(sig_v[:, r] * v_pt[:, r]))
        if len(sig):
            sig.set_vector(v_pt)
        return e2, sig
