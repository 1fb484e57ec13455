"""On-disk problem bundle: one `.npz` file with everything the sigma build needs.

FermiCG keeps problems in JLD2 files (Julia's HDF5 flavour: InCoreInts, clusters, ClusterOps,
ClusteredOperator, TPSCIstate).  The bundle stores the same data as flat arrays, in the
layouts the C ABI consumes (fermicg_gb300.pack), so a problem built once can be reloaded
and uploaded without rebuilding local bases, TDMs or terms:

    ints          h0 (scalar), h1 (n, n), h2 (n, n, n, n)
    clusters      cluster_sizes (N,), cluster_orbs (sum of sizes,) -- consecutive per cluster
    init_fspace   (N, 2)
    ops           ops_table (n_blocks, 10) int64, ops_data float64, cluster_norb (N,) int32
    terms         terms_table (n_terms, 28) int32, terms_ints float64, transfers (T, N, 2) int16
    state         (optional) state_fock (n_cfg, N, 2) int16, state_cfg (n_cfg, N) int16,
                  state_coeff (n_cfg, R) float64
    meta          meta_json: the problem's generation parameters, as JSON text
"""
from __future__ import annotations

import json

import numpy as np

from . import pack

FORMAT_VERSION = 1


def save_bundle(path, prob, state=None):
    """Write `prob` (fermicg_gb300.workloads.Problem) and optionally a TPSCIstate."""
    po = pack.pack_ops(prob.ops, prob.bases)
    pt = pack.pack_terms(prob.ham)
    arrays = {
        "format_version": np.array(FORMAT_VERSION, dtype=np.int64),
        "h0": np.array(float(prob.ints.h0)),
        "h1": np.asarray(prob.ints.h1, dtype=np.float64),
        "h2": np.asarray(prob.ints.h2, dtype=np.float64),
        "cluster_sizes": np.array([len(c) for c in prob.clusters], dtype=np.int32),
        "cluster_orbs": np.array([o for c in prob.clusters for o in c], dtype=np.int32),
        "init_fspace": np.array(prob.init_fspace, dtype=np.int16).reshape(-1, 2),
        "ops_table": po.table, "ops_data": po.data, "cluster_norb": po.cluster_norb,
        "terms_table": pt.table, "terms_ints": pt.ints, "transfers": pt.transfers,
        "meta_json": np.array(json.dumps(prob.meta, default=str)),
    }
    if state is not None:
        f, c, v, _ = pack.pack_state(state)
        arrays.update(state_fock=f, state_cfg=c, state_coeff=np.ascontiguousarray(v))
    np.savez_compressed(path, **arrays)


class Bundle:
    """A loaded bundle: `ops` / `terms` ready for GpuSigma.set_ops / set_terms (and the
    oracle), `state` = (fock, cfg, coeff) or None, plus the integrals and clusters."""

    def __init__(self, z):
        if int(z["format_version"]) != FORMAT_VERSION:
            raise ValueError(f"unsupported bundle format {int(z['format_version'])}")
        self.h0 = float(z["h0"])
        self.h1 = z["h1"]
        self.h2 = z["h2"]
        sizes = [int(s) for s in z["cluster_sizes"]]
        orbs = [int(o) for o in z["cluster_orbs"]]
        self.clusters, p = [], 0
        for s in sizes:
            self.clusters.append(orbs[p:p + s])
            p += s
        self.init_fspace = [tuple(int(x) for x in r) for r in z["init_fspace"]]
        self.ops = pack.PackedOps(z["ops_table"], z["ops_data"], len(sizes), z["cluster_norb"])
        self.terms = pack.PackedTerms(z["terms_table"], z["terms_ints"], z["transfers"])
        self.state = None
        if "state_fock" in z:
            self.state = (z["state_fock"], z["state_cfg"], z["state_coeff"])
        self.meta = json.loads(str(z["meta_json"]))


def load_bundle(path):
    with np.load(path, allow_pickle=False) as z:
        return Bundle({k: z[k] for k in z.files})
