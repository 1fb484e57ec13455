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


# ---- array form of the same vector, for first-order spaces of millions of rows -------------

class SectorRegistry:
    """Fock sectors of one problem, numbered as first seen, with the mixed-radix key of a
    configuration: key = sector id * prod(radix) + sum_c cfg_c * prod(radix[:c]), radix_c the
    largest local dimension of cluster c over all its sectors."""

    def __init__(self, n_clusters: int, radix):
        self.N = n_clusters
        self.radix = np.asarray(radix, dtype=np.int64)
        self.stride = np.concatenate([[1], np.cumprod(self.radix)[:-1]]).astype(np.int64)
        self.span = int(np.prod(self.radix))
        self.ids = {}      # fock tuple -> id
        self.focks = []    # id -> (N, 2) int16

    def sector_ids(self, focks):
        """ids of the (n, N, 2) int16 Fock rows (new sectors registered in first-row order)."""
        focks = np.ascontiguousarray(focks, dtype=np.int16).reshape(-1, self.N * 2)
        if len(focks) == 0:
            return np.zeros(0, dtype=np.int64)
        if self.N <= 8 and focks.min() >= 0 and focks.max() <= 15:  # 4 bits per entry: one uint64 per row
            packed = np.zeros(len(focks), dtype=np.uint64)
            for j in range(2 * self.N):
                packed |= focks[:, j].astype(np.uint64) << np.uint64(4 * j)
            u, first, inv = np.unique(packed, return_index=True, return_inverse=True)
        else:
            u, first, inv = np.unique(focks.view(np.dtype((np.void, focks.dtype.itemsize * focks.shape[1]))).ravel(),
                                      return_index=True, return_inverse=True)
        uid = np.empty(len(u), dtype=np.int64)
        for j in np.argsort(first, kind="stable"):
            f = focks[first[j]]
            t = tuple((int(f[2 * c]), int(f[2 * c + 1])) for c in range(self.N))
            if t not in self.ids:
                if (len(self.focks) + 1) * self.span >= (1 << 62):
                    raise OverflowError("configuration keys exceed 62 bits")
                self.ids[t] = len(self.focks)
                self.focks.append(np.asarray(t, dtype=np.int16))
            uid[j] = self.ids[t]
        return uid[inv.ravel()]

    def keys(self, sec, cfgs):
        return sec * self.span + (np.asarray(cfgs, dtype=np.int64) * self.stride).sum(axis=1)


class FlatTPSCI:
    """A TPSCIstate as arrays: sector id, configuration and R coefficients per row, in any
    physical order, with the bookkeeping that gives TPSCIstate's row order -- sectors in
    insertion order (a sector that loses its last row is deleted, and goes to the end when
    it comes back), configurations in insertion order within their sector.  The operations
    below are those of the TPSCIstate functions of the same names, vectorised."""

    def __init__(self, reg: SectorRegistry, R: int):
        self.reg, self.R = reg, R
        self.sec = np.zeros(0, dtype=np.int64)
        self.cfg = np.zeros((0, reg.N), dtype=np.int16)
        self.coef = np.zeros((0, R))
        self.ins = np.zeros(0, dtype=np.int64)   # insertion counter of each row
        self.rank = {}                           # sector id -> insertion rank of the sector
        self.next_ins = 0
        self.next_rank = 0
        self._key = None
        self._ks = None     # (argsort of the keys, the sorted keys), while the keys stay as they are
        self._canon = True  # the physical rows are in TPSCIstate row order

    # -- construction and views ----------------------------------------------------------
    @staticmethod
    def from_rows(reg, R, focks, cfgs, coeffs):
        """Rows in the given order (distinct configurations), as appended to an empty state."""
        s = FlatTPSCI(reg, R)
        s._append(reg.sector_ids(focks), np.asarray(cfgs, dtype=np.int16).reshape(-1, reg.N),
                  np.asarray(coeffs, dtype=np.float64).reshape(-1, R))
        return s

    @staticmethod
    def from_state(reg, st: TPSCIstate):
        f, c, v, _ = st.flat()
        return FlatTPSCI.from_rows(reg, st.R, f, c, v)

    def to_state(self) -> TPSCIstate:
        f, c, v = self.rows()
        return TPSCIstate.from_flat(self.reg.N, f, c, v) if len(f) else TPSCIstate(self.reg.N, self.R)

    def __len__(self):
        return len(self.sec)

    def key(self):
        if self._key is None:
            self._key = self.reg.keys(self.sec, self.cfg)
        return self._key

    def order(self):
        """physical rows in TPSCIstate row order"""
        if len(self.sec) == 0:
            return np.zeros(0, dtype=np.int64)
        if self._canon:  # already in row order
            return np.arange(len(self.sec), dtype=np.int64)
        rank = np.zeros(len(self.reg.focks), dtype=np.int64)
        for sid, r in self.rank.items():
            rank[sid] = r
        if len(self.ins) == 0 or int(self.ins.max()) < (1 << 40):  # one sort key: rank, then insertion
            return np.argsort((rank[self.sec] << 40) | self.ins, kind="stable")
        return np.lexsort((self.ins, rank[self.sec]))

    def canonicalize(self):
        """reorder the physical rows into TPSCIstate row order"""
        if self._canon:
            return
        o = self.order()
        self.sec, self.cfg, self.coef, self.ins = self.sec[o], self.cfg[o], self.coef[o], self.ins[o]
        self._key = None if self._key is None else self._key[o]
        self._ks = None
        self._canon = True

    def rows(self):
        """(focks (n, N, 2) int16, cfgs (n, N) int16, coeffs (n, R)) in row order"""
        self.canonicalize()
        focks = np.stack(self.reg.focks)[self.sec] if len(self.sec) else np.zeros((0, self.reg.N, 2), np.int16)
        return focks, self.cfg.copy(), self.coef.copy()

    def get_vector(self):
        self.canonicalize()
        return self.coef.copy()

    def set_vector(self, v):
        self.canonicalize()
        v = np.asarray(v, dtype=np.float64).reshape(len(self), -1)
        if v.shape[1] != self.R:
            raise ValueError("root count mismatch")
        self.coef = v.copy()

    # -- bookkeeping -------------------------------------------------------------------------
    def _append(self, sec, cfg, coef):
        """new rows (configurations not present), in the given order"""
        if len(sec) == 0:
            return
        # sectors that (re)appear get ranks in first-row order; sector ids are small, so the
        # present ones come from a count, and the first rows are only sought for new ones
        present = np.flatnonzero(np.bincount(sec))
        new = [sid for sid in present.tolist() if sid not in self.rank]
        if new:
            u, first = np.unique(sec, return_index=True)
            for sid in u[np.argsort(first, kind="stable")].tolist():
                if sid not in self.rank:
                    self.rank[sid] = self.next_rank
                    self.next_rank += 1
        n = len(sec)
        self._canon = False  # new rows go to the end physically; row order is restored on demand
        self.sec = np.concatenate([self.sec, sec])
        self.cfg = np.concatenate([self.cfg, cfg])
        self.coef = np.concatenate([self.coef, coef])
        self.ins = np.concatenate([self.ins, self.next_ins + np.arange(n, dtype=np.int64)])
        self.next_ins += n
        self._key = None
        self._ks = None

    def _keep(self, mask):
        """keep the rows of mask; sectors left without rows are deleted"""
        self.sec, self.cfg, self.coef, self.ins = self.sec[mask], self.cfg[mask], self.coef[mask], self.ins[mask]
        self._key = None if self._key is None else self._key[mask]
        self._ks = None
        live = set(np.flatnonzero(np.bincount(self.sec)).tolist()) if len(self.sec) else set()
        self.rank = {s: r for s, r in self.rank.items() if s in live}

    def _find(self, keys):
        """physical row of each key, -1 where absent"""
        k = self.key()
        if len(k) == 0:
            return np.full(len(keys), -1, dtype=np.int64)
        if self._ks is None:
            o = np.argsort(k, kind="stable")
            self._ks = (o, k[o])
        o, ks = self._ks
        p = np.searchsorted(ks, keys)
        p = np.minimum(p, len(ks) - 1)
        hit = ks[p] == keys
        return np.where(hit, o[p], -1)

    def copy(self):
        """copy_state (empty sectors are not kept: a state never holds one)"""
        s = FlatTPSCI(self.reg, self.R)
        s.sec, s.cfg, s.coef, s.ins = self.sec.copy(), self.cfg.copy(), self.coef.copy(), self.ins.copy()
        s.rank, s.next_ins, s.next_rank = dict(self.rank), self.next_ins, self.next_rank
        s._key = None if self._key is None else self._key.copy()
        s._ks = None if self._ks is None else (self._ks[0].copy(), self._ks[1].copy())
        s._canon = self._canon
        return s

    # -- TPSCIstate algebra ------------------------------------------------------------------
    def zero(self):
        """zero_state"""
        self.coef = np.zeros_like(self.coef)

    def scale(self, a: float):
        self.coef = self.coef * a

    def add(self, other: "FlatTPSCI"):
        """add_state: self += other, new configurations appended in other's row order"""
        if len(other) == 0:
            return
        o = other.order()
        keys = other.key()[o]
        pos = self._find(keys)
        hit = pos >= 0
        if hit.any():  # distinct rows (other's keys are distinct)
            self.coef[pos[hit]] += other.coef[o][hit]
        new = o[~hit]
        self._append(other.sec[new], other.cfg[new], other.coef[new])

    def times_matrix(self, C) -> "FlatTPSCI":
        out = self.copy()
        if len(out):
            out.coef = self.coef @ np.asarray(C)
        return out

    def minus(self, B: "FlatTPSCI") -> "FlatTPSCI":
        """minus_state(self, B) = self - B, in B's row order then self's new rows"""
        C = B.copy()
        C.scale(-1.0)
        C.add(self)
        return C

    def overlap(self, v2: "FlatTPSCI"):
        """overlap(self, v2): R x R over the shared configurations"""
        S = np.zeros((v2.R, v2.R))
        if len(self) == 0 or len(v2) == 0:
            return S
        pos = self._find(v2.key())
        hit = pos >= 0
        return self.coef[pos[hit]].T @ v2.coef[hit]

    def project_out(self, w: "FlatTPSCI"):
        """project_out: drop w's configurations"""
        if len(self) == 0 or len(w) == 0:
            return
        self._keep(w._find(self.key()) < 0)

    def clip(self, thresh: float):
        """clip: drop configurations with every |c| < thresh"""
        if len(self):
            self._keep(~np.all(np.abs(self.coef) < thresh, axis=1))
