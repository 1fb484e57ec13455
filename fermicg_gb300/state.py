"""TPSCIstate: the sparse tensor-product-state vector.

Restates the data model of type_TPSCIstate.jl:11-14: an insertion-ordered
map FockConfig -> (insertion-ordered map ClusterConfig -> R coefficients).
The flat row order (get_vector, type_TPSCIstate.jl:139-149) is fock-sector
insertion order, then config insertion order within the sector; rows of one
sector are therefore contiguous, which the device layout relies on.

Local state indices are 0-based here (the reference's ClusterConfig is
1-based Int16); conversion happens at the Julia boundary.
"""
from __future__ import annotations

import numpy as np


class TPSCIstate:
    def __init__(self, n_clusters: int, R: int = 1, dtype=np.float64):
        self.n_clusters = n_clusters
        self.R = R
        self.dtype = dtype
        self.data = {}  # fock tuple -> {config tuple -> np.ndarray(R)}

    # --- construction -----------------------------------------------------
    def add_fockconfig(self, fock):
        fock = tuple((int(a), int(b)) for a, b in fock)
        if fock not in self.data:
            self.data[fock] = {}
        return fock

    def __setitem__(self, key, value):
        fock, cfg = key
        fock = self.add_fockconfig(fock)
        self.data[fock][tuple(int(x) for x in cfg)] = np.asarray(value, dtype=self.dtype).reshape(self.R).copy()

    def __len__(self):
        return sum(len(v) for v in self.data.values())

    def copy_structure(self, R=None):
        out = TPSCIstate(self.n_clusters, self.R if R is None else R, self.dtype)
        for f, cfgs in self.data.items():
            out.data[f] = {c: np.zeros(out.R, dtype=self.dtype) for c in cfgs}
        return out

    # --- flat views -------------------------------------------------------
    def get_vector(self):
        """(n_cfg, R) coefficients in row order (type_TPSCIstate.jl:139)."""
        n = len(self)
        v = np.zeros((n, self.R), dtype=self.dtype)
        i = 0
        for cfgs in self.data.values():
            for c in cfgs.values():
                v[i] = c
                i += 1
        return v

    def set_vector(self, v):
        """type_TPSCIstate.jl:172-190"""
        v = np.asarray(v).reshape(len(self), -1)
        if v.shape[1] != self.R:
            raise ValueError("root count mismatch")
        i = 0
        for cfgs in self.data.values():
            for c in cfgs:
                cfgs[c] = v[i].astype(self.dtype).copy()
                i += 1

    def flat(self):
        """Flat index arrays: focks (n_cfg, N, 2) int16, configs (n_cfg, N) int16,
        coeffs (n_cfg, R), and the sector table (list of (fock, start, count))."""
        n = len(self)
        N = self.n_clusters
        focks = np.zeros((n, N, 2), dtype=np.int16)
        cfgs = np.zeros((n, N), dtype=np.int16)
        coeffs = np.zeros((n, self.R), dtype=self.dtype)
        sectors = []
        i = 0
        for f, cs in self.data.items():
            start = i
            fa = np.array(f, dtype=np.int16)
            for c, v in cs.items():
                focks[i] = fa
                cfgs[i] = c
                coeffs[i] = v
                i += 1
            sectors.append((f, start, i - start))
        return focks, cfgs, coeffs, sectors

    @staticmethod
    def from_flat(n_clusters, focks, cfgs, coeffs):
        coeffs = np.asarray(coeffs)
        R = coeffs.shape[1]
        s = TPSCIstate(n_clusters, R, coeffs.dtype)
        for i in range(len(cfgs)):
            f = tuple((int(a), int(b)) for a, b in focks[i])
            s.add_fockconfig(f)
            s.data[f][tuple(int(x) for x in cfgs[i])] = coeffs[i].copy()
        return s

    def keys(self):
        for f, cs in self.data.items():
            for c in cs:
                yield f, c

    def as_dict(self):
        return {(f, c): v for f, cs in self.data.items() for c, v in cs.items()}


# ---- host-side TPSCIstate algebra (src/type_TPSCIstate.jl, src/tpsci_outer.jl) ------------

def copy_state(s: TPSCIstate) -> TPSCIstate:
    """deepcopy (type_TPSCIstate.jl:491): empty sectors are dropped."""
    out = TPSCIstate(s.n_clusters, s.R, s.dtype)
    for f, cs in s.data.items():
        if cs:
            out.data[f] = {c: v.copy() for c, v in cs.items()}
    return out


def add_state(s1: TPSCIstate, s2: TPSCIstate):
    """add! (type_TPSCIstate.jl:617): s1 += s2, new configurations appended."""
    for f, cs in s2.data.items():
        d = s1.data.setdefault(f, {})
        for c, v in cs.items():
            if c in d:
                d[c] = d[c] + v
            else:
                d[c] = v.copy()


def scale_state(s: TPSCIstate, a: float):
    for cs in s.data.values():
        for c in cs:
            cs[c] = cs[c] * a


def times_matrix(s: TPSCIstate, C) -> TPSCIstate:
    """A * C (type_TPSCIstate.jl:456)."""
    out = copy_state(s)
    if len(out):
        out.set_vector(s.get_vector() @ C)
    return out


def minus_state(A: TPSCIstate, B: TPSCIstate) -> TPSCIstate:
    """A - B (type_TPSCIstate.jl:478)."""
    C = copy_state(B)
    scale_state(C, -1.0)
    add_state(C, A)
    return C


def overlap(v1: TPSCIstate, v2: TPSCIstate):
    """R x R overlap over the shared configurations (type_TPSCIstate.jl:416)."""
    S = np.zeros((v2.R, v2.R))
    for f, cs in v2.data.items():
        d1 = v1.data.get(f)
        if not d1:
            continue
        for c, v in cs.items():
            if c in d1:
                S += np.outer(d1[c], v)
    return S


def project_out(v: TPSCIstate, w: TPSCIstate):
    """project_out! (tpsci_outer.jl:869): drop w's configurations from v."""
    for f, cs in w.data.items():
        if f in v.data:
            d = v.data[f]
            for c in cs:
                d.pop(c, None)
            if not d:
                del v.data[f]


def clip(s: TPSCIstate, thresh: float):
    """clip! (type_TPSCIstate.jl:589): drop configurations with every |c| < thresh."""
    for f in list(s.data):
        cs = s.data[f]
        for c in list(cs):
            if np.all(np.abs(cs[c]) < thresh):
                del cs[c]
        if not cs:
            del s.data[f]


def zero_state(s: TPSCIstate):
    for cs in s.data.values():
        for c in cs:
            cs[c] = np.zeros(s.R, dtype=s.dtype)


def state_from_rows(n_clusters, R, focks, cfgs, coeffs) -> TPSCIstate:
    out = TPSCIstate(n_clusters, R)
    for i in range(len(cfgs)):
        f = tuple((int(a), int(b)) for a, b in focks[i])
        out.data.setdefault(f, {})[tuple(int(x) for x in cfgs[i])] = np.array(coeffs[i], dtype=np.float64)
    return out
