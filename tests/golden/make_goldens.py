"""Generate the golden fixtures under tests/golden/ from the reference's own test data.

Run with the path of a FermiCG checkout as the one (required) argument:

    python tests/golden/make_goldens.py PATH_TO_FERMICG

It reads the reference's JLD2 fixtures (test/_testdata_*.jld2) with the minimal
HDF5 reader next to this script, and the known-answer values written in the
reference's test files (test/test_FCI.jl, test/test_Clusters.jl,
test/test_TDMs.jl, test/test_tpsci.jl), and writes small .npz / .json files that
the tests load without the reference present.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from jld2_reader import JLD2File  # noqa: E402

REF = None  # the FermiCG checkout, set from the command line


def _ints(f):
    i = f["ints"]
    return float(i["h0"]), np.asarray(i["h1"], dtype=np.float64), np.asarray(i["h2"], dtype=np.float64)


def _clusters(f):
    return [[int(x) - 1 for x in c["orb_list"]] for c in f["clusters"]]


def _fspace(f):
    return [(int(t["1"]), int(t["2"])) for t in f["init_fspace"]]


def _julia_matrix(txt):
    rows = [r.strip() for r in txt.strip().split("\n") if r.strip()]
    out = []
    for r in rows:
        r = r.rstrip(";").strip()
        out.append([float(x) for x in r.split()])
    return np.array(out)


def tdm_goldens():
    """ref matrices of test/test_TDMs.jl with the op block and orbital slice they test."""
    txt = open(os.path.join(REF, "test", "test_TDMs.jl")).read()
    pat = re.compile(r"ref\d?\s*=\s*\[(.*?)\]\s*(?:#.*?\n\s*)*?test\s*=\s*cluster_ops\[(\d+)\]\[\"(\w+)\"\]"
                     r"\[\(\((\d+),\s*(\d+)\),\s*\((\d+),\s*(\d+)\)\)\]\[([\d,\s]+),:,:\]", re.S)
    out = []
    for m in pat.finditer(txt):
        mat = _julia_matrix(m.group(1))
        out.append({"cluster": int(m.group(2)) - 1, "op": m.group(3),
                    "fb": [int(m.group(4)), int(m.group(5))], "fk": [int(m.group(6)), int(m.group(7))],
                    "orb": [int(x) - 1 for x in m.group(8).split(",")], "ref_abs": np.abs(mat).tolist()})
    return out


def main():
    # ---- H6 (test_FCI.jl, test_Clusters.jl, test_TDMs.jl) -----------------------------
    f = JLD2File(os.path.join(REF, "test", "_testdata_hf_h6.jld2"))
    h0, h1, h2 = _ints(f)
    fci_txt = open(os.path.join(REF, "test", "test_FCI.jl")).read()
    na = int(re.search(r"n_elec_a\s*=\s*(\d+)", fci_txt).group(1))
    nb = int(re.search(r"n_elec_b\s*=\s*(\d+)", fci_txt).group(1))
    cl_txt = open(os.path.join(REF, "test", "test_Clusters.jl")).read()
    sums = [float(x) for x in re.findall(r"isapprox\(tst1,\s*([-\d.eE]+)", cl_txt)]
    mr = int(re.search(r"max_roots=(\d+), init_fspace=init_fspace, delta_elec=(\d+)", cl_txt).group(1))
    de = int(re.search(r"max_roots=(\d+), init_fspace=init_fspace, delta_elec=(\d+)", cl_txt).group(2))
    tdm_txt = open(os.path.join(REF, "test", "test_TDMs.jl")).read()
    tdm_cl = re.findall(r"clusters\s*=\s*\[(\(\d+:\d+\)(?:,\s*\(\d+:\d+\))*)\]", tdm_txt)[-1]
    tdm_clusters = [list(range(int(a) - 1, int(b))) for a, b in re.findall(r"\((\d+):(\d+)\)", tdm_cl)]
    np.savez(os.path.join(HERE, "h6.npz"), h0=h0, h1=h1, h2=h2, e_fci=float(f["e_fci"]))
    meta = {
        "source": "reference test/_testdata_hf_h6.jld2, test/test_FCI.jl, test/test_Clusters.jl, test/test_TDMs.jl",
        "clusters": _clusters(f), "init_fspace": _fspace(f),
        "fci_electrons": [na, nb],
        "cluster_abs_sums": {"default_max_roots10": sums[0], "max_roots": mr, "delta_elec": de,
                             "restricted": sums[1]},
        "tdm_clusters": tdm_clusters, "tdm_max_roots": 100,
        "tdm_slices": tdm_goldens(),
    }
    json.dump(meta, open(os.path.join(HERE, "h6.json"), "w"), indent=1)

    # ---- H12 (test_tpsci.jl "tpsci h12 64bit") -----------------------------------------
    f = JLD2File(os.path.join(REF, "test", "_testdata_cmf_h12_64bit.jld2"))
    h0, h1, h2 = _ints(f)
    d1 = f["d1"]
    np.savez(os.path.join(HERE, "h12.npz"), h0=h0, h1=h1, h2=h2, da=np.asarray(d1["a"]), db=np.asarray(d1["b"]),
             e_cmf=float(f["e_cmf"]))
    tp = open(os.path.join(REF, "test", "test_tpsci.jl")).read()
    block = tp[tp.index('@testset "tpsci h12 64bit"'):tp.index('@testset "tpsci h12 32bit"')]
    block = "\n".join(l for l in block.split("\n") if not l.strip().startswith("#"))
    refs = re.findall(r"ref\s*=\s*\[(.*?)\]", block, re.S)
    e0 = [float(x) for x in refs[0].split()]
    e02 = [float(x) for x in refs[1].split()]
    call = block[block.index("FermiCG.tpsci_ci("):]
    call = call[:call.index(");")]
    kw = dict(re.findall(r"(thresh_cipsi|thresh_foi|conv_thresh|ci_conv|thresh_asci)=([-\d.eE]+)", call))
    pt2 = re.search(r"compute_pt2_energy\(.*?thresh_foi=([-\d.eE]+)\)", block).group(1)
    excit = [[int(x) - 1 for x in m.split(",")] for m in re.findall(r"ClusterConfig\(\[([\d,]+)\]\)\]\s*=", block)]
    gen = open(os.path.join(REF, "test", "generate_test_data_h12.jl")).read()
    json.dump({
        "source": "reference test/_testdata_cmf_h12_64bit.jld2, test/test_tpsci.jl, test/generate_test_data_h12.jl",
        "clusters": _clusters(f), "init_fspace": _fspace(f),
        "max_roots": int(re.search(r"max_roots\s*=\s*(\d+)", gen).group(1)),
        "nroots": len(e0), "excitons": excit,
        "tpsci_kwargs": {k: float(v) for k, v in kw.items()}, "pt2_thresh_foi": float(pt2),
        "e0": e0, "e0_plus_e2": e02,
    }, open(os.path.join(HERE, "h12.json"), "w"), indent=1)
    print("wrote", sorted(x for x in os.listdir(HERE) if x.endswith((".npz", ".json"))))


if __name__ == "__main__":
    if len(sys.argv) != 2 or not os.path.isdir(os.path.join(sys.argv[1], "test")):
        sys.exit("usage: python tests/golden/make_goldens.py PATH_TO_FERMICG  (a checkout with test/*.jld2)")
    REF = sys.argv[1]
    main()
