"""Build of the in-tree CUDA library fermicg_gb300/_build/libfcg_gpu.so (sm_103a only)."""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfcg_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["fcg_gpu.cu", "open_sigma.cu", "davidson.cu", "bst.cu", "bst_fois.cu", "dplan.cu", "plan.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def build(force: bool = False, verbose: bool = False) -> str:
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, "fcg_internal.h"), os.path.join(CSRC, "fcg_ctx.cuh"),
                   os.path.join(CSRC, "small_dense.h"), os.path.join(CSRC, "tucker_small.cuh"),
                   os.path.join(CSRC, "tcgen05.cuh"), os.path.join(CSRC, "dprim.cuh"),
                   os.path.join(os.path.dirname(HERE), "include", "fcg_gpu.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp"] + ARCH
    objs = []
    cmds = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        cmds.append([nvcc, "-c", s, "-o", o] + common)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(len(cmds)) as ex:
        list(ex.map(run, cmds))
    tmp = LIB + f".tmp{os.getpid()}"
    run([nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
