"""Flat, pointer-and-size form of ClusterOps / ClusteredOperator / TPSCIstate.

This is the layout that crosses the C ABI (include/fcg_gpu.h) and that the CPU
oracle reads.  Everything is plain numpy arrays:

op blocks  (one row per TDM block, `OPB_*` columns, int64):
    cluster, op_id, fb_a, fb_b, fk_a, fk_b, n_idx, m_bra, m_ket, offset
    data: float64 blob; block element (pidx, I, J) at offset + pidx + n_idx*(I + m_bra*J)
    (the reference's column-major (n_orbidx, I, J) layout, build_local_quantities.jl:176-188;
    "H"/"Hcmf" blocks have n_idx = 1).
terms      (one row per ClusteredTerm, `TRM_*` columns, int32):
    nbody, transfer_id, c[4], op[4], da[4], db[4], parity[4], dim[4], ints_offset(2 x int32 lo/hi)
    ints: float64 blob, each term's ints flattened column-major (type_ClusteredTerm.jl:31-67).
transfers  (n_transfers, N, 2) int16: the TransferConfig of each group.
state      fock (n_cfg, N, 2) int16, cfg (n_cfg, N) int16 (0-based local states),
           rows in TPSCIstate order.
"""
from __future__ import annotations

import numpy as np

from .local_fci import OP_ID, OP_H, OP_HCMF, N_OPS

OPB_COLS = 10
TRM_COLS = 2 + 4 * 6 + 2


def op_id_of(name: str) -> int:
    if name == "H":
        return OP_H
    if name == "Hcmf":
        return OP_HCMF
    return OP_ID[name]


class PackedOps:
    def __init__(self, table, data, n_clusters, cluster_norb):
        self.table = table
        self.data = data
        self.n_clusters = n_clusters
        self.cluster_norb = cluster_norb

    def lookup(self):
        return {tuple(int(x) for x in r[:6]): i for i, r in enumerate(self.table)}


def pack_ops(ops, bases, dtype=np.float64) -> PackedOps:
    rows = []
    chunks = []
    off = 0
    for co in ops:
        c = co.idx
        for name, blocks in co.data.items():
            oid = op_id_of(name)
            for (fb, fk), g in blocks.items():
                g = np.asarray(g)
                if g.ndim == 2:
                    mk, mb = g.shape
                    nidx = 1
                else:
                    mk, mb, nidx = g.shape
                rows.append([c, oid, fb[0], fb[1], fk[0], fk[1], nidx, mb, mk, off])
                chunks.append(np.ascontiguousarray(g, dtype=dtype).reshape(-1))
                off += g.size
    table = np.array(rows, dtype=np.int64).reshape(-1, OPB_COLS)
    data = np.concatenate(chunks) if chunks else np.zeros(0, dtype=dtype)
    return PackedOps(table, data, len(ops), np.array([len(b.orbs) for b in bases], dtype=np.int32))


class PackedTerms:
    def __init__(self, table, ints, transfers):
        self.table = table
        self.ints = ints
        self.transfers = transfers


def pack_terms(ham, dtype=np.float64) -> PackedTerms:
    N = ham.n_clusters
    rows = []
    chunks = []
    trans = []
    off = 0
    for tid, (tr, terms) in enumerate(ham):
        trans.append(np.array(tr, dtype=np.int16))
        for t in terms:
            r = np.zeros(TRM_COLS, dtype=np.int64)
            r[0] = t.nbody
            r[1] = tid
            for i in range(4):
                if i < t.nbody:
                    r[2 + i] = t.clusters[i]
                    r[6 + i] = op_id_of(t.ops[i])
                    r[10 + i] = t.delta[i][0]
                    r[14 + i] = t.delta[i][1]
                    r[18 + i] = t.parity[i]
                    r[22 + i] = t.ints.shape[i] if (t.nbody > 1 and i < t.ints.ndim) else 1
                else:
                    r[2 + i] = -1
                    r[6 + i] = -1
                    r[22 + i] = 1
            flat = np.asarray(t.ints).reshape(-1, order="F") if t.nbody > 1 else np.zeros(0)
            r[26] = off & 0xFFFFFFFF
            r[27] = off >> 32
            rows.append(r)
            chunks.append(flat.astype(dtype))
            off += flat.size
    table = np.array(rows, dtype=np.int64).astype(np.int32).reshape(-1, TRM_COLS)
    ints = np.concatenate(chunks) if chunks else np.zeros(0, dtype=dtype)
    transfers = np.array(trans, dtype=np.int16).reshape(-1, N, 2)
    return PackedTerms(table, ints, transfers)


def pack_state(state):
    focks, cfgs, coeffs, sectors = state.flat()
    return np.ascontiguousarray(focks), np.ascontiguousarray(cfgs), coeffs, sectors
