"""The host builders and the CPU oracle, pinned to the reference's own test data.

Fixtures (tests/golden/*.npz|json) were extracted from the reference's JLD2 test
files and test scripts by tests/golden/make_goldens.py.
"""
import json
import os

import numpy as np
import pytest

import oracle
from oracle.fci import fci_energies
from fermicg_gb300 import pack
from fermicg_gb300.integrals import InCoreInts
from fermicg_gb300.local_fci import add_cmf_operators, compute_cluster_eigenbasis, compute_cluster_ops
from fermicg_gb300.state import TPSCIstate
from fermicg_gb300.terms import extract_ClusteredTerms

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    z = np.load(os.path.join(G, name + ".npz"))
    m = json.load(open(os.path.join(G, name + ".json")))
    return InCoreInts(float(z["h0"]), z["h1"], z["h2"]), z, m


def test_h6_fci_energy():
    """test/test_FCI.jl: lowest determinant-FCI energy of H6 (1a,1b) = e_fci."""
    ints, z, m = _load("h6")
    e = fci_energies(ints.h1, ints.h2, *m["fci_electrons"], k=1)
    assert abs(e[0] - float(z["e_fci"])) < 1e-10


def test_h6_cluster_basis_checksums():
    """test/test_Clusters.jl: sum of |basis vector entries| over all clusters and sectors."""
    ints, z, m = _load("h6")
    s = m["cluster_abs_sums"]
    b = compute_cluster_eigenbasis(ints, m["clusters"], max_roots=10)
    assert abs(sum(np.abs(v).sum() for cb in b for v in cb.basis.values()) - s["default_max_roots10"]) < 1e-10
    b = compute_cluster_eigenbasis(ints, m["clusters"], max_roots=s["max_roots"], init_fspace=m["init_fspace"],
                                   delta_elec=s["delta_elec"])
    assert abs(sum(np.abs(v).sum() for cb in b for v in cb.basis.values()) - s["restricted"]) < 1e-10


def test_h6_tdm_slices():
    """test/test_TDMs.jl: |TDM| slices of A, B, AA, aa, Aa, Bb, Ab blocks (1e-5, as the reference)."""
    ints, z, m = _load("h6")
    b = compute_cluster_eigenbasis(ints, m["tdm_clusters"], max_roots=m["tdm_max_roots"])
    ops = compute_cluster_ops(b, ints)
    assert len(m["tdm_slices"]) >= 7
    for t in m["tdm_slices"]:
        blk = ops[t["cluster"]].data[t["op"]][(tuple(t["fb"]), tuple(t["fk"]))]
        n = len(m["tdm_clusters"][t["cluster"]])
        pidx = sum(o * n ** i for i, o in enumerate(t["orb"]))
        sl = blk[:, :, pidx].T
        np.testing.assert_allclose(np.abs(sl), np.array(t["ref_abs"]), atol=1e-5)


def _h12_problem():
    ints, z, m = _load("h12")
    b = compute_cluster_eigenbasis(ints, m["clusters"], max_roots=m["max_roots"], init_fspace=m["init_fspace"],
                                   rdm1a=z["da"], rdm1b=z["db"])
    ops = compute_cluster_ops(b, ints)
    add_cmf_operators(ops, b, ints, z["da"], z["db"])
    H = extract_ClusteredTerms(ints, m["clusters"])
    return ints, z, m, b, ops, H


def test_h12_cmf_reference_energy():
    """generate_test_data_h12.jl / the fixture's e_cmf: <CMF|H|CMF> + h0 from the
    embedded local bases and the clustered Hamiltonian's diagonal."""
    ints, z, m, b, ops, H = _h12_problem()
    st = TPSCIstate(len(m["clusters"]), 1)
    st[(tuple(map(tuple, m["init_fspace"])), (0,) * len(m["clusters"]))] = [1.0]
    f, c, v, _ = pack.pack_state(st)
    O = oracle.Oracle(pack.pack_ops(ops, b), pack.pack_terms(H))
    assert abs(O.diagonal_H(f, c)[0] + ints.h0 - float(z["e_cmf"])) < 1e-10


def test_h12_tpsci_energies_match_reference():
    """test/test_tpsci.jl "tpsci h12 64bit": TPSCI variational energies of 7 roots and
    e0 + e2 (reference asserts 1e-8), from the oracle's tpsci_ci / PT2 restatement."""
    from oracle.tpsci import OracleTPSCI
    ints, z, m, b, ops, H = _h12_problem()
    R, N = m["nroots"], len(m["clusters"])
    st = TPSCIstate(N, R)
    ref = tuple(map(tuple, m["init_fspace"]))
    row = np.zeros(R)
    row[0] = 1.0
    st[(ref, (0,) * N)] = row
    for i, ex in enumerate(m["excitons"]):
        row = np.zeros(R)
        row[i + 1] = 1.0
        st[(ref, tuple(ex))] = row
    kw = m["tpsci_kwargs"]
    T = OracleTPSCI(ops, b, H)
    e0, v0 = T.tpsci_ci(st, thresh_cipsi=kw["thresh_cipsi"], thresh_foi=kw["thresh_foi"],
                        thresh_asci=kw.get("thresh_asci"), conv_thresh=kw["conv_thresh"])
    np.testing.assert_allclose(np.abs(e0), np.abs(np.array(m["e0"])), atol=1e-8, rtol=0)
    # compute_pt2_energy(v0, thresh_foi=1e-10): e0 + e2 (reference asserts 1e-8)
    e2 = T.pt2_energy(v0, thresh_foi=m["pt2_thresh_foi"])
    np.testing.assert_allclose(np.abs(e0 + e2), np.abs(np.array(m["e0_plus_e2"])), atol=1e-8, rtol=0)
    # compute_pt1_wavefunction on the same orthonormal vectors gives the same e2, and its
    # PT1 amplitudes reproduce it: e2_r = sum_x sigma_x,r * v_pt_x,r
    e2_pt1, v_pt = T.pt1_wavefunction(v0, thresh_foi=m["pt2_thresh_foi"])
    np.testing.assert_allclose(e2_pt1, e2, atol=1e-12, rtol=0)
    assert len(v_pt) > len(v0)
    d0 = v0.as_dict()
    assert not any(k in d0 for k in v_pt.keys())
