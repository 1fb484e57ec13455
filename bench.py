"""Benchmark: TPSCI closed sigma builds/s (tps_ci_matvec) on one GB300, mixed vs FP64.

Workload: 24 orbitals / 24 electrons, 6 clusters x 4 orbitals, K=72 seeded Cholesky
integrals, M=16 lowest local states per Fock sector (sectors within 2 electrons of
(2,2)), an energy-ordered variational space of 100,000 TPS configurations, 4 roots.
A step is one sigma build sigma = H C over that space.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is device-resident throughput (inputs in HBM, L2 flushed between steps);
`e2e` goes through the C ABI with pinned host buffers (H2D of C and D2H of sigma
inside the timed region).  The reference arm times the CPU oracle (a restatement
of the reference's Julia loops) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TPSCI sigma builds/s (mixed FP32 vs FP64), config 24o/6 clusters/1e5 TPS configs/4 roots"
WORKLOAD = "tpsci_closed_sigma_24o_6x4_M16_1e5cfg_R4"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-cfg", type=int, default=100000)
    ap.add_argument("--roots", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    ap.add_argument("--no-serving", dest="serving", action="store_false", help="skip the solve-latency stream")
    ap.add_argument("--no-bst", dest="bst", action="store_false", help="skip the block-sparse Tucker sigma leg")
    ap.add_argument("--bst-only", action="store_true", help="run only the block-sparse Tucker sigma leg")
    ap.add_argument("--bst-sectors", type=int, default=5, help="first K Fock sectors of the BST vector (0 = all)")
    ap.add_argument("--bst-maxq", type=int, default=4, help="most clusters in their excited range per Tucker block")
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip the grouped launch of 256 uneven problems")
    ap.add_argument("--batched-only", action="store_true", help="run only the grouped-launch leg")
    ap.add_argument("--instances", type=int, default=256, help="problems of the grouped-launch leg")
    ap.add_argument("--no-stored", dest="stored", action="store_false",
                    help="skip the stored-Hamiltonian-block timings and solve variants")
    ap.add_argument("--no-open", dest="open", action="store_false", help="skip the open (FOIS) sigma leg")
    ap.add_argument("--open-only", action="store_true", help="run only the open (FOIS) sigma leg")
    ap.add_argument("--no-fois", dest="fois", action="store_false", help="skip the BST first-order space leg")
    ap.add_argument("--no-tpsci", dest="tpsci", action="store_false", help="skip the tpsci_ci driver leg")
    ap.add_argument("--tpsci-only", action="store_true", help="run only the tpsci_ci driver leg")
    ap.add_argument("--fois-only", action="store_true", help="run only the BST first-order space leg")
    ap.add_argument("--no-davidson", dest="davidson", action="store_false", help="skip the per-shape solve timings")
    ap.add_argument("--serving-only", action="store_true", help="run only the solve-stream leg (both servers)")
    ap.add_argument("--davidson-only", action="store_true",
                    help="run only the per-shape Davidson solve timings of the serving shapes")
    ap.add_argument("--open-cfg", type=int, default=10000, help="variational configurations of the open sigma leg")
    return ap.parse_args()


def bench_config(n_cfg, R, world):
    """The workload description both arms print (identical dicts for the same workload)."""
    return {"workload": WORKLOAD, "n_cfg": int(n_cfg), "roots": int(R), "parallelism": f"replicas{world}",
            "l2": "flushed (256 MiB write) before every timed GPU step"}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x: float, world: int) -> float:
    """The largest x over the ranks of the process group (x itself on one rank): a timed
    region counts as long as its slowest replica."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def build_workload(n_cfg, R):
    from fermicg_gb300 import pack, workloads
    prob = workloads.config1_problem(seed=0)
    st = workloads.energy_ordered_space(prob, n_cfg, R=R, seed=0)
    po, pt = pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham)
    f, c, v, _ = pack.pack_state(st)
    return prob, st, po, pt, f, c, v


def cpu_reference(po, pt, f, c, v, budget_s, threads):
    """Time the oracle's tps_ci_matvec restatement (all host threads): a 1/16 row sample
    first; the full build when it fits the budget, else a larger evenly spaced sample.
    Returns (sigma builds/s for the full space, description of what was timed, the full
    sigma (n_cfg, R) when the whole build ran, else None)."""
    import oracle
    O = oracle.Oracle(po, pt)
    n = f.shape[0]

    def run(nblk, frac):
        rows = max(1, int(n * frac / nblk))
        t0 = time.perf_counter()
        done = 0
        for b in range(nblk):
            s0 = (b * n) // nblk
            O.sigma_closed(f, c, v, rows=(s0, min(n, s0 + rows)), n_threads=threads)
            done += min(n, s0 + rows) - s0
        return time.perf_counter() - t0, done

    dt, done = run(16, 1.0 / 16)
    est_full = dt * n / done
    if est_full < budget_s:
        sig, dt = cpu_full_build(O, f, c, v, threads)
        return 1.0 / dt, f"full build, all {n} bra rows, {dt:.2f} s", sig
    frac = min(1.0, budget_s / est_full)
    dt, done = run(16, frac)
    return (done / (dt * n), f"{done} of {n} bra rows in 16 evenly spaced blocks, {dt:.1f} s, scaled to the full "
            "build", None)


def cpu_full_build(O, f, c, v, threads):
    """One whole tps_ci_matvec of the oracle's restatement: (sigma, seconds)."""
    t0 = time.perf_counter()
    sig = O.sigma_closed(f, c, v, n_threads=threads)
    return sig, time.perf_counter() - t0


def _shape_12o(seed):
    from fermicg_gb300 import workloads
    return workloads.build_problem(12, [3] * 4, [(2, 1), (1, 2), (2, 1), (1, 2)], 36, seed, max_roots=1000)


def _shape_24o(seed):
    from fermicg_gb300 import workloads
    return workloads.build_problem(24, [4] * 6, [(2, 2)] * 6, 72, seed, max_roots=16, delta_elec=2)


def _shape_32o(seed):
    from fermicg_gb300 import workloads
    return workloads.build_problem(32, [4] * 8, [(2, 2)] * 8, 96, seed, max_roots=8, delta_elec=2)


def _shape_32o_bst(seed):
    """A config-2-shaped request: the 32-orbital / 8-cluster x 4 problem (local bases of 16
    states per sector), BST blocks of the reference sector with at most two excited clusters,
    Tucker ranks 4-12."""
    from fermicg_gb300 import workloads
    return workloads.build_problem(32, [4] * 8, [(2, 2)] * 8, 96, seed, max_roots=16, delta_elec=2)


SERVING_SHAPES = [  # (name, builder(seed), n_cfg (TPSCI) or None (BST), roots, share of the serving stream)
    ("12o_4x3_full", _shape_12o, 2000, 1, 0.6),
    ("24o_6x4_M16", _shape_24o, 10000, 4, 0.3),
    ("32o_8x4_bst_q2", _shape_32o_bst, None, 2, 0.1),
]

# the per-shape Davidson timings also cover the earlier TPSCI request of the 32-orbital shape
DAVIDSON_SHAPES = [
    ("12o_4x3_full", _shape_12o, 2000, 1),
    ("24o_6x4_M16", _shape_24o, 10000, 4),
    ("32o_8x4_M8", lambda seed: _shape_32o(seed), 5000, 2),
]


def _bst_request_parts(prob, R, seed):
    """(PackedOps, PackedTerms, PackedBST, guess (core_total, R), preconditioner diagonal) of a
    BST solve of the reference sector of `prob` (at most two excited clusters, ranks 4-12)."""
    from fermicg_gb300 import pack
    from fermicg_gb300.bst import PackedBST, hcmf_diagonal, synthetic_bst
    ref = tuple(tuple(f) for f in prob.init_fspace)
    vec = synthetic_bst(prob, [ref], max_q=2, rank_range=(4, 12), R=R, seed=seed)
    pb = PackedBST(vec, len(prob.clusters), R)
    hd = hcmf_diagonal(pb, vec, prob.ops)
    rng = np.random.default_rng(seed)
    guess = 0.05 * rng.standard_normal((pb.core_total, R)) / np.sqrt(pb.core_total)
    for r, k in enumerate(np.argsort(hd)[:R]):
        guess[k, r] += 1.0
    return pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham), pb, guess, hd


def headline_solve(g, n, R, tol=1e-6):
    """The Davidson solve of the headline problem (tps_ci_davidson, src/tpsci_outer.jl:364-454):
    R roots to a residual of tol, all-FP64 and mixed (float32 sigma builds, FP64 Gram-Schmidt,
    Rayleigh-Ritz, residuals and final FP64 refinement).  Reports the energy error of the mixed
    solve against the FP64 one per root."""
    from fermicg_gb300 import workloads
    guess = workloads.davidson_guess(n, R, seed=0, lowest=np.argsort(g.diagonal())[:R])
    res = {}
    for prec in ("fp64", "fp32"):
        g.davidson(guess, tol=tol, max_iter=200, precision=prec)  # warm-up (buffers)
        t1 = time.perf_counter()
        e, X, rn, it = g.davidson(guess, tol=tol, max_iter=200, precision=prec)
        res[prec] = (e, rn, it, time.perf_counter() - t1, g.stats()["davidson_sigma_calls"])
    e64, e32 = res["fp64"][0], res["fp32"][0]
    err = np.abs(e32 - e64)
    return {"workload": f"{WORKLOAD}: Davidson, {R} roots, tol {tol:g}",
            "energies_fp64": [float(x) for x in e64], "energies_mixed": [float(x) for x in e32],
            "energy_error_per_root": [float(x) for x in err], "max_energy_error": float(err.max()),
            "within_1uEh": bool(err.max() <= 1e-6),
            "fp64": {"seconds": res["fp64"][3], "iterations": res["fp64"][2],
                     "max_residual": float(np.max(res["fp64"][1]))},
            "mixed": {"seconds": res["fp32"][3], "iterations": res["fp32"][2],
                      "max_residual": float(np.max(res["fp32"][1]))},
            "mixed_over_fp64_solve": res["fp64"][3] / res["fp32"][3]}


def davidson_benchmark(reps=2, stored=True):
    """One solve per serving shape, alone on the GPU (tol 1e-6, mixed and FP64): the host time
    of each stage of a request (fcg_set_ops, fcg_set_terms, fcg_state_set, fcg_davidson), the
    iteration count and the time per iteration."""
    from fermicg_gb300 import pack, workloads
    from fermicg_gb300.gpu import GpuSigma
    g = GpuSigma(0)
    out = {}
    for name, build, n_cfg, R in DAVIDSON_SHAPES:
        prob = build(1001)
        st = workloads.energy_ordered_space(prob, n_cfg, R=R, seed=0)
        f, c, v, _ = pack.pack_state(st)
        guess = workloads.davidson_guess(f.shape[0], R, seed=0)
        po, pt = pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham)
        for prec in ("fp32", "fp64"):
            best = None
            for _ in range(reps):
                t = [time.perf_counter()]
                g.set_ops(po)
                t.append(time.perf_counter())
                g.set_terms(pt)
                t.append(time.perf_counter())
                g.state_set(f, c)
                t.append(time.perf_counter())
                e, X, res, it = g.davidson(guess, tol=1e-6, max_iter=200, precision=prec)
                t.append(time.perf_counter())
                d = np.diff(t) * 1e3
                if best is None or d[3] < best["davidson_ms"]:
                    best = {"set_ops_ms": d[0], "set_terms_ms": d[1], "state_set_ms": d[2], "davidson_ms": d[3],
                            "iterations": it, "ms_per_iteration": d[3] / max(it, 1)}
            out[f"{name}/{'mixed' if prec == 'fp32' else 'fp64'}"] = best
            if stored:  # the same solve after storing the Hamiltonian blocks (assembly timed)
                bs = None
                for _ in range(reps):
                    g.state_set(f, c)
                    t1 = time.perf_counter()
                    g.cache_hamiltonian()
                    t2 = time.perf_counter()
                    e2, X2, res2, it2 = g.davidson(guess, tol=1e-6, max_iter=200, precision=prec)
                    t3 = time.perf_counter()
                    if bs is None or (t3 - t1) < (bs["cache_ms"] + bs["davidson_ms"]) * 1e-3:
                        bs = {"cache_ms": (t2 - t1) * 1e3, "davidson_ms": (t3 - t2) * 1e3, "iterations": it2,
                              "ms_per_iteration": (t3 - t2) * 1e3 / max(it2, 1),
                              "max_energy_difference_vs_direct": float(np.abs(e2 - e).max())}
                g.cache_hamiltonian(0)
                out[f"{name}/{'mixed' if prec == 'fp32' else 'fp64'}/stored"] = bs
    g.close()
    return out


def serving_benchmark(n_req=600, rate=200.0, steady_rate=40.0, seed=7, slots=16, lanes=4):
    """Poisson streams of Davidson solves drawn 60/30/10 % from three problem shapes (12- and
    24-orbital TPSCI requests with stored Hamiltonian blocks, 32-orbital BST requests), tol
    1e-6, mixed and FP64: n_req requests at the stated arrival rate (above the GPU's capacity:
    the queue grows, and latency with it) and at a rate below capacity (steady state), served
    by the thread-per-slot server and the library's continuous-batching server.  Returns p50 /
    p99 latency and solves/s per run, and the largest energy difference of a request between
    runs."""
    from fermicg_gb300 import pack, workloads
    from fermicg_gb300.serving import NativeSolveServer, Request, SolveServer, latency_summary
    shapes = SERVING_SHAPES
    pools = []
    for k, (name, build, n_cfg, R, share) in enumerate(shapes):
        pool = []
        for j in range(4 if n_cfg is not None else 2):
            prob = build(1000 * (k + 1) + j)
            if n_cfg is None:
                pool.append(("bst",) + _bst_request_parts(prob, R, seed=j))
                continue
            st = workloads.energy_ordered_space(prob, n_cfg, R=R, seed=j)
            f, c, v, _ = pack.pack_state(st)
            guess = workloads.davidson_guess(f.shape[0], R, seed=j)
            pool.append(("tpsci", pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham), f, c, guess))
        pools.append(pool)
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0, n_req)
    kinds = rng.choice(len(shapes), size=n_req, p=[sh[4] for sh in shapes])
    picks = [int(rng.integers(len(pools[k]))) for k in kinds]

    def requests(prec, lam):
        arrivals = np.cumsum(gaps / lam)
        out = []
        for i in range(n_req):
            item = pools[kinds[i]][picks[i]]
            if item[0] == "bst":
                _, po, pt, pb, guess, hd = item
                out.append(Request(float(arrivals[i]), i, po, pt, None, None, guess, tol=1e-6, precision=prec,
                                   shape=shapes[kinds[i]][0], bst=pb, bst_hd=hd))
            else:
                _, po, pt, f, c, guess = item
                out.append(Request(float(arrivals[i]), i, po, pt, f, c, guess, tol=1e-6, precision=prec,
                                   shape=shapes[kinds[i]][0], cache=True))
        return out

    out = {"requests": n_req, "slots": slots, "mix": {sh[0]: sh[4] for sh in shapes},
           "arrival_rate_per_s": rate, "steady_rate_per_s": steady_rate,
           "servers": {"threads": "one context, stream and host thread per slot; solves overlap on the GPU",
                       "native": f"fcg_server: continuous batching in {lanes} lanes (a scheduler thread and a "
                                 "stream each); a lane's solves run in lockstep rounds, one grouped sigma launch "
                                 "per precision per round"},
           "note": "TPSCI requests store their Hamiltonian blocks after fcg_state_set (assembly inside the "
                   "request's latency); BST requests plan and cache their operators in fcg_bst_set"}
    energies = {}
    runs = [("native", rate), ("threads", rate), ("native", steady_rate), ("threads", steady_rate)]
    for server, lam in runs:
        for prec in ("fp32", "fp64"):
            srv = SolveServer(slots=slots) if server == "threads" else NativeSolveServer(slots=slots, lanes=lanes)
            res = srv.run(requests(prec, lam))
            srv.close()
            energies[(server, lam, prec)] = {r.rid: r.energies for r in res}
            summ = latency_summary(res)
            summ["by_shape_p50_s"] = {sh[0]: float(np.median([r.latency for r in res if r.shape == sh[0]] or [0]))
                                      for sh in shapes}
            summ["not_converged"] = int(sum(float(np.max(r.residuals)) >= 1e-6 for r in res))
            key = f"{server}_{'steady' if lam == steady_rate else 'stated_rate'}"
            out.setdefault(key, {})["mixed" if prec == "fp32" else "fp64"] = summ
    keys = list(energies)
    out["max_energy_difference_between_runs"] = max(
        float(np.abs(energies[k][i] - energies[keys[0]][i]).max()) for k in keys for i in range(n_req))
    out["max_energy_difference_mixed_vs_fp64"] = max(
        float(np.abs(energies[(s_, l_, "fp32")][i] - energies[(s_, l_, "fp64")][i]).max())
        for (s_, l_, p_) in keys if p_ == "fp32" for i in range(n_req))
    return out


def bst_benchmark(steps, warmup, cpu_seconds, peaks, n_sectors=5, max_q=4):
    """build_sigma! with the operator cache on the config-2 BST vector: 32 orbitals, 8
    clusters x 4, the reference Fock sector and its first single charge transfers, every
    TuckerConfig with at most `max_q` clusters in their excited range, Tucker ranks 4-12
    (cores up to 12^4), 2 roots.  FP64 and FP32 device timings (L2 flushed before each step;
    the FP32 build runs its GEMM-shaped groups on the tcgen05 tensor cores, also timed with
    them off), the HBM roofline of reading the operator cache, the tensor-pipe roofline of the
    tensor-core kernel, the host-buffer path, and a CPU sample of the oracle's build_sigma!."""
    import torch
    from fermicg_gb300 import pack, workloads
    from fermicg_gb300.bst import PackedBST, synthetic_bst
    from fermicg_gb300.gpu import GpuSigma
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    prob = workloads.config2_problem(0)
    secs = workloads.single_transfer_sectors(prob)
    if n_sectors > 0:
        secs = secs[:n_sectors]
    R = 2
    vec = synthetic_bst(prob, secs, max_q=max_q, rank_range=(4, 12), R=R, seed=0)
    pb = PackedBST(vec, len(prob.clusters), R)
    g = GpuSigma(torch.cuda.current_device())
    g.set_ops(pack.pack_ops(prob.ops, prob.bases))
    g.set_terms(pack.pack_terms(prob.ham))
    t0 = time.perf_counter()
    g.bst_set(pb)
    t_set = time.perf_counter() - t0
    st = g.stats()
    stream = torch.cuda.current_stream()
    g.set_stream(stream.cuda_stream)
    host = pb.cores_of(vec)
    x = torch.from_numpy(host).cuda()
    y = torch.empty_like(x)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(prec):
        for _ in range(warmup):
            g.bst_sigma_device(x.data_ptr(), y.data_ptr(), R, prec)
        torch.cuda.synchronize()
        ms, kern, tc = [], [], []
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.bst_sigma_device(x.data_ptr(), y.data_ptr(), R, prec)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            s_ = g.stats()
            kern.append(s_["last_kernel_ms"])
            tc.append(s_["bst_tc_ms"])
        return statistics.mean(ms), statistics.median(kern), statistics.median(tc)

    ms64, k64, _ = timed("fp64")
    y64 = y.clone()
    ms32, k32, tc32 = timed("fp32")
    rel32 = float((y - y64).abs().max() / y64.abs().max())
    s32 = g.stats()
    g.bst_tensor_cores(False)
    ms32c, k32c, _ = timed("fp32")
    relc = float((y - y64).abs().max() / y64.abs().max())
    g.bst_tensor_cores(True)
    walls = []
    for _ in range(max(3, steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        g.bst_sigma(host, "fp32")
        walls.append(time.perf_counter() - t1)
    e2e_ms = 1e3 * statistics.mean(walls)
    cache = st["bst_cache_elements"]
    core_bytes = 2 * pb.core_total * R

    def roof(kms, elem):
        alg = cache * elem + core_bytes * elem
        ach = alg / (kms * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                "bytes_per_sigma": alg, "note": "operator cache + cores read/written per sigma, of measured HBM copy peak"}

    # the sigma executes about 100 flops per byte of operator cache: its bound is arithmetic.
    # Executed flops (spectator mode products + group contractions, all roots) over the kernel
    # time, against the nominal CUDA-core peaks of GB300 (152 SMs at 2.07 GHz: 128 FP32 FMA or
    # the FP64 rate per cycle); no measured figure exists for these pipes
    flops_exec = st["bst_flops_executed"] * R
    nominal = {"fp32": 152 * 128 * 2 * 2.07e9 / 1e12, "fp64": 1.25}

    def flop_roof(kms, prec):
        ach = flops_exec / (kms * 1e-3) / 1e12
        return {"bound": f"{prec} cuda cores", "achieved": ach, "peak": nominal[prec], "unit": "TFLOP/s",
                "frac": ach / nominal[prec], "flops_per_sigma": flops_exec,
                "note": f"executed flops / kernel time, of the nominal {prec} CUDA-core peak (no measured peak)"}

    # tensor-core kernel: executed MMA flops (three TF32 products per tile, tiles padded to
    # 128 x 16k) over its CUDA-event time, against half the measured bf16 dense peak (TF32
    # runs at half the bf16 rate)
    tf32_peak = peaks.get("bf16_tflops", 1900.0) / 2
    tc_ach = s32["bst_tc_mma_flops"] / (tc32 * 1e-3) / 1e12 if tc32 > 0 else 0.0
    out = {
        "workload": f"bst_sigma_32o_8x4_M16_{len(secs)}sectors_q{max_q}_ranks4-12_R2",
        "max_core": int(pb.blocks[:, 1].max()), "blocks": len(pb.keys),
        "core_total": pb.core_total, "roots": R, "triples": st["bst_triples"], "groups": st["bst_groups"],
        "cache_elements": cache, "cache_seconds": st["bst_cache_seconds"], "plan_seconds": st["bst_plan_seconds"],
        "set_wall_s": t_set,
        "flops_reference_per_sigma": st["bst_flops_reference"] * R,
        "flops_executed_per_sigma": flops_exec,
        "fp64": {"value": 1e3 / ms64, "unit": "sigma_builds/s", "ms_per_step": ms64, "kernel_ms": k64,
                 "roofline": roof(k64, 8), "flop_roofline": flop_roof(k64, "fp64")},
        "fp32": {"value": 1e3 / ms32, "unit": "sigma_builds/s", "ms_per_step": ms32, "kernel_ms": k32,
                 "roofline": roof(k32, 4), "flop_roofline": flop_roof(k32, "fp32"), "rel_err_vs_fp64": rel32,
                 "tensor_cores": {"groups": s32["bst_tc_groups"], "of_groups": st["bst_groups"],
                                  "algorithmic_flops": s32["bst_tc_flops"], "mma_flops": s32["bst_tc_mma_flops"],
                                  "share_of_reference_flops": s32["bst_tc_flops"] / max(st["bst_flops_reference"] * R, 1),
                                  "kernel_ms": tc32,
                                  "roofline": {"bound": "tensor", "achieved": tc_ach, "peak": tf32_peak,
                                               "unit": "TFLOP/s", "frac": tc_ach / tf32_peak,
                                               "note": "bst_tc_gemm_kernel: executed 3xTF32 MMA flops / its time, "
                                                       "of half the measured bf16 dense peak"}},
                 "cuda_cores_only": {"ms_per_step": ms32c, "kernel_ms": k32c, "rel_err_vs_fp64": relc}},
        "e2e_fp32": {"value": 1e3 / e2e_ms, "unit": "sigma_builds/s", "h2d_bytes_per_step": host.nbytes,
                     "d2h_bytes_per_step": host.nbytes},
    }
    if cpu_seconds > 0:
        from oracle import bst as obst
        tri = g.bst_triples()
        keys = list(vec.keys())
        for stride in (400, 100, 25):
            sample = keys[::stride]
            idx = {pb.index[k] for k in sample}
            frac = float(np.isin(tri[:, 0], list(idx)).sum()) / max(len(tri), 1)
            t1 = time.perf_counter()
            obst.build_sigma({k: obst.zero_like({k: vec[k]}, R)[k] for k in sample}, vec, prob.ops, prob.ham,
                             len(prob.clusters), R)
            dt = time.perf_counter() - t1
            if dt > cpu_seconds / 4 or stride == 25:
                break
        out["cpu_baseline"] = {"value": frac / dt if frac > 0 else None, "unit": "sigma_builds/s", "cores": 1,
                               "kind": "port", "sample": f"{len(sample)} of {len(keys)} bra blocks "
                               f"({100 * frac:.2f} % of the triples) in {dt:.1f} s, oracle build_sigma!, numpy"}
    g.close()
    return out


def batched_benchmark(steps, warmup, n_inst=256, stored=True):
    """Batched uneven instances: n_inst independent problems (orbitals in {8,12,16,20},
    clusters of 2-5 orbitals, half filling, M=8-16, 1-3 roots, seeds 3000+i), each problem's
    closed sigma in one grouped launch (fcg_sigma_closed_grouped) against the same sigmas
    launched one context after another.  Returns problem-sigmas/s for both, mixed and FP64."""
    import torch
    from fermicg_gb300 import pack, workloads
    from fermicg_gb300.gpu import GpuSigma, sigma_closed_grouped
    t0 = time.perf_counter()
    items = []
    built = workloads.config3_batch(n_inst, max_cluster=5)  # local bases in worker processes
    t_inputs = time.perf_counter() - t0
    for po, pt, f, c, v in built:
        g = GpuSigma(torch.cuda.current_device())
        g.set_ops(po)
        g.set_terms(pt)
        g.state_set(f, c)
        dc = torch.from_numpy(np.asfortranarray(v).T.copy()).cuda()
        items.append((g, dc, torch.empty_like(dc), v.shape[1], f.shape[0]))
    t_build = time.perf_counter() - t0
    gs = [it[0] for it in items]
    cps, sps, rs = [it[1].data_ptr() for it in items], [it[2].data_ptr() for it in items], [it[3] for it in items]
    out = {"workload": f"{n_inst}_uneven_tpsci_problems_8-20o_clusters2-5_M8-16_R1-3",
           "instances": n_inst, "total_configs": int(sum(it[4] for it in items)),
           "instances_with_5_orbital_clusters": int(sum(int(5 in set(b[0].cluster_norb.tolist())) for b in built)),
           "total_triples": int(sum(it[0].stats()["n_triples"] for it in items)), "setup_s": t_build,
           "inputs_s": t_inputs}
    for prec in ("fp32", "fp64"):
        for _ in range(warmup):
            sigma_closed_grouped(gs, cps, sps, rs, prec)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            sigma_closed_grouped(gs, cps, sps, rs, prec)
        e1.record()
        torch.cuda.synchronize()
        grouped_ms = e0.elapsed_time(e1) / steps
        for g, dc, ds, R, _ in items[:4]:
            g.sigma_closed_device(dc.data_ptr(), ds.data_ptr(), R, prec)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(steps):
            for g, dc, ds, R, _ in items:
                g.sigma_closed_device(dc.data_ptr(), ds.data_ptr(), R, prec)
        e1.record()
        torch.cuda.synchronize()
        seq_ms = e0.elapsed_time(e1) / steps
        out["mixed" if prec == "fp32" else "fp64"] = {
            "grouped_ms": grouped_ms, "sequential_ms": seq_ms,
            "problem_sigmas_per_s_grouped": n_inst * 1e3 / grouped_ms,
            "problem_sigmas_per_s_sequential": n_inst * 1e3 / seq_ms, "grouped_over_sequential": seq_ms / grouped_ms}
    # whole Davidson solves of all instances (tol 1e-6): one after another, and in lockstep
    # with their sigma builds grouped per iteration (fcg_davidson_grouped); the guesses have a
    # seeded dense part, so every arm looks for the same (lowest) roots
    from fermicg_gb300.gpu import davidson_grouped
    guesses = [workloads.davidson_guess(n, R, seed=5000 + q, lowest=np.argsort(g.diagonal())[:R])
               for q, (g, dc, ds, R, n) in enumerate(items)]
    tol = 1e-6
    solved = {}
    for prec in ("fp32", "fp64"):
        davidson_grouped(gs[:8], guesses[:8], tol=tol, max_iter=200, precision=prec)  # warm-up
        t1 = time.perf_counter()
        res = davidson_grouped(gs, guesses, tol=tol, max_iter=200, precision=prec)
        grouped_s = time.perf_counter() - t1
        t1 = time.perf_counter()
        seq = [g.davidson(gu, tol=tol, max_iter=200, precision=prec) for g, gu in zip(gs, guesses)]
        seq_s = time.perf_counter() - t1
        # the same solves from 16 host threads, each problem on its own context's stream
        from concurrent.futures import ThreadPoolExecutor
        t1 = time.perf_counter()
        with ThreadPoolExecutor(16) as ex:
            list(ex.map(lambda a: a[0].davidson(a[1], tol=tol, max_iter=200, precision=prec), zip(gs, guesses)))
        conc_s = time.perf_counter() - t1
        st = gs[0].stats()
        solved[prec] = (res, seq)
        dmax = max(float(np.abs(r[0] - q[0]).max()) for r, q in zip(res, seq))
        out["solves_mixed" if prec == "fp32" else "solves_fp64"] = {
            "grouped_s": grouped_s, "sequential_s": seq_s, "concurrent_16_threads_s": conc_s,
            "solves_per_s_grouped": n_inst / grouped_s, "solves_per_s_sequential": n_inst / seq_s,
            "solves_per_s_concurrent": n_inst / conc_s, "grouped_over_sequential": seq_s / grouped_s,
            "grouped_over_concurrent": conc_s / grouped_s,
            "grouped_phases_s": {k[6:]: st[k] for k in ("group_setup_seconds", "group_step_seconds",
                                                         "group_issue_seconds", "group_wait_seconds")},
            "grouped_rounds": st["group_rounds"], "grouped_launches": st["group_launches"],
            "max_energy_difference": dmax, "iterations_total": int(sum(r[3] for r in res)),
            "not_converged_grouped": int(sum(r[2].max() >= tol for r in res)),
            "not_converged_sequential": int(sum(q[2].max() >= tol for q in seq))}
    out["solves_mixed"]["max_energy_difference_vs_fp64"] = max(
        float(np.abs(a[0] - b[0]).max()) for a, b in zip(solved["fp32"][0], solved["fp64"][1]))
    if stored:
        # the same grouped solves after storing every problem's Hamiltonian blocks (assembly timed)
        t1 = time.perf_counter()
        hc_bytes = sum(g.cache_hamiltonian() for g in gs)
        hc_s = time.perf_counter() - t1
        blk = {"assembly_s": hc_s, "bytes": hc_bytes}
        for prec in ("fp32", "fp64"):
            t1 = time.perf_counter()
            res = davidson_grouped(gs, guesses, tol=tol, max_iter=200, precision=prec)
            grouped_s = time.perf_counter() - t1
            st = gs[0].stats()
            from concurrent.futures import ThreadPoolExecutor
            t1 = time.perf_counter()
            with ThreadPoolExecutor(16) as ex:
                list(ex.map(lambda a: a[0].davidson(a[1], tol=tol, max_iter=200, precision=prec), zip(gs, guesses)))
            conc_s = time.perf_counter() - t1
            blk["solves_mixed" if prec == "fp32" else "solves_fp64"] = {
                "grouped_s": grouped_s, "solves_per_s_grouped": n_inst / grouped_s,
                "concurrent_16_threads_s": conc_s, "grouped_over_concurrent": conc_s / grouped_s,
                "solves_per_s_with_assembly": n_inst / (grouped_s + hc_s),
                "grouped_phases_s": {k[6:]: st[k] for k in ("group_step_seconds", "group_issue_seconds",
                                                             "group_wait_seconds")},
                "not_converged": int(sum(r[2].max() >= tol for r in res)),
                "max_energy_difference_vs_direct": max(float(np.abs(r[0] - q[0]).max())
                                                       for r, q in zip(res, solved[prec][0]))}
        out["stored_blocks"] = blk
    for g in gs:
        g.close()
    return out


def tpsci_benchmark(cpu_seconds):
    """tpsci_ci (src/tpsci.jl:39-363) on the 12-orbital / 4-cluster x 3 problem (full local FCI
    bases, 6a/6b, one root, thresh_cipsi 1e-3, thresh_foi 1e-5, FP64) from the reference
    configuration: the GPU driver to convergence with compute_pt2_energy on top, and the
    first three macro-iterations on the GPU and in the oracle's restatement on the host
    cores (equal work: the same spaces, the same energies)."""
    from fermicg_gb300 import workloads
    from fermicg_gb300.state import TPSCIstate
    from fermicg_gb300.tpsci import GpuTPSCI
    prob = workloads.config0_problem(0)
    N = len(prob.clusters)

    def start():
        st = TPSCIstate(N, 1)
        st[(tuple(map(tuple, prob.init_fspace)), (0,) * N)] = np.array([1.0])
        return st

    T = GpuTPSCI(prob.ops, prob.bases, prob.ham)
    T.tpsci_ci(start(), thresh_cipsi=1e-3, thresh_foi=1e-5, max_iter=2)  # warm-up
    t1 = time.perf_counter()
    e0, v0 = T.tpsci_ci(start(), thresh_cipsi=1e-3, thresh_foi=1e-5)
    t2 = time.perf_counter()
    e2 = T.pt2_energy(v0, thresh_foi=1e-5)
    t3 = time.perf_counter()
    e3, v3 = T.tpsci_ci(start(), thresh_cipsi=1e-3, thresh_foi=1e-5, max_iter=3)
    t4 = time.perf_counter()
    T.close()
    out = {"workload": "tpsci_ci 12o / 4 clusters x 3, full local FCI, 1 root, thresh_cipsi 1e-3, thresh_foi 1e-5",
           "gpu_tpsci_ci_s": t2 - t1, "gpu_pt2_s": t3 - t2, "e0": float(e0[0]), "e0_plus_e2": float(e0[0] + e2[0]),
           "configurations": len(v0), "first_3_iterations": {"gpu_s": t4 - t3, "configurations": len(v3),
                                                             "e0": float(e3[0])}}
    if cpu_seconds > 0:
        from oracle.tpsci import OracleTPSCI
        O = OracleTPSCI(prob.ops, prob.bases, prob.ham)
        t5 = time.perf_counter()
        eo, vo = O.tpsci_ci(start(), thresh_cipsi=1e-3, thresh_foi=1e-5, max_iter=3)
        t6 = time.perf_counter()
        f3 = out["first_3_iterations"]
        f3.update({"oracle_s": t6 - t5, "oracle_configurations": len(vo), "oracle_e0": float(eo[0]),
                   "gpu_over_oracle_speedup": (t6 - t5) / (t4 - t3), "cores": os.cpu_count(),
                   "energy_difference": float(abs(eo[0] - e3[0]))})
    return out


def fois_benchmark(steps, warmup, cpu_seconds, thresh=1e-3):
    """build_compressed_1st_order_state of the CMF state of the 32-orbital / 8-cluster x 4 problem
    (local bases of 16 states per sector) at thresh 1e-3: wall time of fcg_bst_fois (planning,
    SVD precontraction, expansion through the BST sigma, HOSVD compressions, nonorth_add, results
    fetched), one do_fois_pt2 on top of it, and the oracle's restatement of the same build on the
    host (one run, when the CPU budget allows)."""
    from fermicg_gb300 import bst_fois as G
    from fermicg_gb300 import workloads
    prob = workloads.config2_problem(0)
    g = G.GpuBSTFois(prob.ops, prob.bases, prob.ham)
    vec, P, Q = G.cmf_state(prob.bases, prob.init_fspace, R=1)
    for _ in range(warmup):
        fg = g.fois(vec, P, Q, thresh=thresh)
    walls = []
    for _ in range(steps):
        t1 = time.perf_counter()
        fg = g.fois(vec, P, Q, thresh=thresh)
        walls.append(time.perf_counter() - t1)
    st = g.H.stats()
    t1 = time.perf_counter()
    e, _ = g.do_fois_pt2(vec, P, Q, thresh_foi=thresh)
    pt2_s = time.perf_counter() - t1
    cg = g.cg_info[0]
    g.close()
    out = {"workload": "CMF state of the 32-orbital / 8-cluster x 4 problem, thresh 1e-3",
           "contributions": st["bst_fois_items"], "fois_blocks": len(fg),
           "fois_length": int(sum(G._len(t) for t in fg.values())), "fois_ms": 1e3 * float(np.median(walls)),
           "contributions_per_s": st["bst_fois_items"] / float(np.median(walls)),
           "fois_pt2_s": pt2_s, "e_pt2": float(e[0]),
           "hylleraas_cg": {"products": cg[0], "converged": cg[1], "residual": cg[2],
                            "note": "" if cg[1] else "the reference's CG (abstol 1e-6, at most 100 products) "
                                    "does not converge here: H0 - E0 is not positive definite on this synthetic "
                                    "problem, so E(PT2) is the last iterate's, as in the reference"}}
    if cpu_seconds > 0:
        from oracle import bst_fois as F
        t1 = time.perf_counter()
        fo = F.build_compressed_1st_order_state(vec, P, Q, prob.ops, prob.ham, len(prob.clusters), 1, thresh=thresh,
                                               norb=[len(c) for c in prob.clusters])
        cpu_s = time.perf_counter() - t1
        out["cpu_baseline"] = {"value": cpu_s, "unit": "s per build", "cores": 1, "kind": "port",
                               "sample": "the whole build (oracle restatement, numpy)", "blocks": len(fo)}
        out["gpu_over_cpu"] = cpu_s / (out["fois_ms"] * 1e-3)
    return out


def open_benchmark(steps, warmup, cpu_seconds, n_cfg=10000, R=4, thresh=1e-4):
    """open_matvec_thread (the FOIS sigma of TPSCI's selection step) on the bench problem:
    the n_cfg lowest configurations, R roots, contributions kept when |x| > thresh/max|c|.
    Device time of fcg_sigma_open (screen, expand, hash, compact) and the whole call with
    the outputs fetched to the host; the oracle's restatement on a sample of ket rows."""
    from fermicg_gb300 import pack, workloads
    from fermicg_gb300.gpu import GpuSigma
    prob = workloads.config1_problem(0)
    st = workloads.energy_ordered_space(prob, n_cfg, R=R, seed=0)
    f, c, v, _ = pack.pack_state(st)
    po, pt = pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham)
    g = GpuSigma(0)
    g.set_ops(po)
    g.set_terms(pt)
    g.state_set(f, c)
    for _ in range(warmup):
        of, oc, ov = g.sigma_open(v, thresh)
    walls, kms = [], []
    for _ in range(steps):
        t1 = time.perf_counter()
        of, oc, ov = g.sigma_open(v, thresh)
        walls.append(time.perf_counter() - t1)
        kms.append(g.stats()["last_kernel_ms"])
    st_ = g.stats()
    wall = statistics.median(walls)
    peaks = _peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    ach = st_["open_bytes"] / (st_["open_expand_ms"] * 1e-3) / 1e9
    out = {"workload": f"open_sigma_24o_6x4_M16_{n_cfg}cfg_R{R}_thresh{thresh:g}", "n_cfg": int(f.shape[0]),
           "roots": R, "thresh": thresh, "n_out": int(of.shape[0]), "jobs": st_["open_jobs"],
           "jobs_kept_by_screen": st_["open_jobs_kept"], "contractions": st_["open_contractions"],
           "value": 1.0 / wall, "unit": "open_sigma_builds/s", "wall_ms": 1e3 * wall,
           "device_ms": statistics.median(kms), "expand_kernel_ms": st_["open_expand_ms"],
           "contractions_per_s": st_["open_contractions"] / wall,
           "flops_reference": st_["open_flops_reference"],
           "gflops_reference_count": st_["open_flops_reference"] / (st_["open_expand_ms"] * 1e-3) / 1e9,
           "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                        "bytes": st_["open_bytes"],
                        "note": "compulsory bytes (TDM blocks touched, C, one key + row per output) over the "
                                "expand_jobs_kernel time, of measured HBM copy peak; the kernel is bound by the "
                                "exact FP64 evaluation of candidates, not HBM"}}
    if cpu_seconds > 0:
        import oracle
        O = oracle.Oracle(po, pt)
        threads = os.cpu_count() or 1
        n = f.shape[0]
        nblk = 8
        # ket rows of 8 evenly spaced blocks, regrouped so that the rows of a Fock sector are
        # contiguous; the open sigma is a sum over ket rows, so the GPU run on these rows alone
        # gives exactly their contributions
        for per in (3, 12):
            idx = np.concatenate([np.arange((b * n) // nblk, (b * n) // nblk + per) for b in range(nblk)])
            idx = idx[np.lexsort(f[idx].reshape(len(idx), -1).T[::-1])]
            t1 = time.perf_counter()
            ref = O.sigma_open(f[idx], c[idx], v[idx], thresh, n_threads=threads)
            dt = time.perf_counter() - t1
            if dt > cpu_seconds / 4:
                break
        done = len(idx)
        out["cpu_baseline"] = {"value": done / (dt * n), "unit": "open_sigma_builds/s", "cores": threads,
                               "kind": "port", "sample": f"{done} of {n} ket rows in {nblk} evenly spaced blocks, "
                               f"{dt:.1f} s, scaled to the full build (oracle open_matvec_thread restatement)"}
        g.state_set(f[idx], c[idx])
        mine = g.sigma_open(v[idx], thresh)
        ko, vo = _open_canon(*mine)
        kr, vr = _open_canon(*ref)
        same = ko.shape == kr.shape and bool(np.array_equal(ko, kr))
        out["parity"] = {"sample": f"the same {done} ket rows, GPU against the oracle",
                         "outputs": int(len(kr)), "key_sets_identical": same,
                         "values_rel": (float(np.abs(vo - vr).max() / np.abs(vr).max()) if same else None),
                         "tolerance": 1e-10}
    g.close()
    return out


def _open_canon(of, oc, ov):
    """Rows of an open sigma as (sorted (Fock key, state key) pairs, values in that order)."""
    fo = of.reshape(len(of), -1).astype(np.uint64)
    co = oc.astype(np.uint64)
    k1 = np.zeros(len(of), dtype=np.uint64)
    for j in range(fo.shape[1]):
        k1 = (k1 << np.uint64(4)) | fo[:, j]
    k2 = np.zeros(len(of), dtype=np.uint64)
    for j in range(co.shape[1]):
        k2 = (k2 << np.uint64(8)) | co[:, j]
    order = np.lexsort((k2, k1))
    return np.stack([k1[order], k2[order]], axis=1), ov[order]


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def clocks_sampler():
    out = []
    stop = threading.Event()

    def run():
        try:
            p = subprocess.Popen(["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                                  "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                                  "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                                  "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                                 stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            return
        while not stop.is_set():
            line = p.stdout.readline()
            if not line:
                break
            out.append(line.strip())
        p.terminate()

    th = threading.Thread(target=run, daemon=True)
    th.start()

    def finish():
        stop.set()
        th.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in out:
            parts = [x.strip() for x in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}

    return finish


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.impl == "reference":
        if rank != 0:
            return
        import oracle
        prob, st, po, pt, f, c, v = build_workload(a.n_cfg, a.roots)
        threads = os.cpu_count() or 1
        O = oracle.Oracle(po, pt)
        secs = []
        for i in range(a.warmup + a.steps):  # every step is one whole build over all bra rows
            _, dt = cpu_full_build(O, f, c, v, threads)
            if i >= a.warmup:
                secs.append(dt)
        ms = 1e3 * statistics.mean(secs)
        value = 1e3 / ms
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": "sigma_builds/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(f.shape[0], a.roots, world),
            "cpu_baseline": {"value": value, "unit": "sigma_builds/s", "cores": threads, "kind": "port",
                             "sample": f"the whole build (all {f.shape[0]} bra rows) every step; C++ restatement "
                                       "of tps_ci_matvec (the reference is Julia, which is not available)"},
            "e2e": {"value": value, "unit": "sigma_builds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    import torch
    from fermicg_gb300 import build as fbuild
    from fermicg_gb300.gpu import GpuSigma

    fbuild.build()
    torch.cuda.set_device(local)
    if a.open_only:
        if rank == 0:
            print(json.dumps({"open_sigma": open_benchmark(max(3, a.steps // 4), a.warmup, a.cpu_seconds,
                                                           n_cfg=a.open_cfg)}))
        return
    if a.serving_only:
        if rank == 0:
            print(json.dumps({"serving": serving_benchmark()}))
        return
    if a.davidson_only:
        if rank == 0:
            print(json.dumps({"davidson": davidson_benchmark(stored=a.stored)}))
        return
    if a.tpsci_only:
        if rank == 0:
            print(json.dumps({"tpsci": tpsci_benchmark(a.cpu_seconds)}))
        return
    if a.fois_only:
        if rank == 0:
            print(json.dumps({"bst_fois": fois_benchmark(max(3, a.steps // 4), a.warmup, a.cpu_seconds)}))
        return
    if a.batched_only:
        if rank == 0:
            print(json.dumps({"batched": batched_benchmark(max(3, a.steps // 2), a.warmup, a.instances, a.stored)}))
        return
    if a.bst_only:
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        if rank == 0:
            print(json.dumps({"bst": bst_benchmark(max(3, a.steps // 2), a.warmup, a.cpu_seconds, peaks,
                                                   a.bst_sectors, a.bst_maxq)}))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    prob, st, po, pt, f, c, v = build_workload(a.n_cfg, a.roots)
    n, R = v.shape
    g = GpuSigma(local)
    g.set_ops(po)
    g.set_terms(pt)
    # the state's rows, sectors and closed-sigma plan (device join); the first call also
    # uploads the term tables and grows the planner's buffers
    t_set = []
    for _ in range(3):
        t0 = time.perf_counter()
        g.state_set(f, c)
        t_set.append(time.perf_counter() - t0)
    stream = torch.cuda.current_stream()
    g.set_stream(stream.cuda_stream)
    stats = g.stats()

    d_c = torch.from_numpy(np.asfortranarray(v).T.copy()).cuda()  # (R, n) contiguous == column-major (n, R)
    d_s = torch.empty_like(d_c)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(prec, steps, warmup):
        for _ in range(warmup):
            g.sigma_closed_device(d_c.data_ptr(), d_s.data_ptr(), R, prec)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        tot = 0.0
        kern = []
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.sigma_closed_device(d_c.data_ptr(), d_s.data_ptr(), R, prec)
            e1.record(stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
            kern.append(g.stats()["last_kernel_ms"])
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return max_over_ranks(tot / steps, world), max_over_ranks(statistics.median(kern), world)

    finish = clocks_sampler()
    ms32, k32 = timed("fp32", a.steps, a.warmup)
    ms64, k64 = timed("fp64", max(3, a.steps // 4), a.warmup)
    clocks = finish()
    g.sigma_closed_device(d_c.data_ptr(), d_s.data_ptr(), R, "fp32")
    torch.cuda.synchronize()
    sig32 = d_s.clone()
    g.sigma_closed_device(d_c.data_ptr(), d_s.data_ptr(), R, "fp64")
    torch.cuda.synchronize()
    rel32 = float((sig32 - d_s).abs().max() / d_s.abs().max())
    sig64 = d_s.clone()

    # The same sigma from stored Hamiltonian blocks (fcg_cache_hamiltonian): the term-summed
    # matrix element of every (work item, bra, ket) pair computed once, then each build reads
    # one value per pair.  Reported beside the headline, which stays the direct build.
    stored = None
    if a.stored:
        t1 = time.perf_counter()
        hc_bytes = g.cache_hamiltonian()
        hc_s = time.perf_counter() - t1
        pairs = g.stats()["hcache_pairs"]
        hms32, hk32 = timed("fp32", a.steps, a.warmup)
        hms64, hk64 = timed("fp64", max(3, a.steps // 4), a.warmup)
        g.sigma_closed_device(d_c.data_ptr(), d_s.data_ptr(), R, "fp64")
        torch.cuda.synchronize()
        hrel64 = float((d_s - sig64).abs().max() / sig64.abs().max())
        g.sigma_closed_device(d_c.data_ptr(), d_s.data_ptr(), R, "fp32")
        torch.cuda.synchronize()
        hrel32 = float((d_s - sig64).abs().max() / sig64.abs().max())
        # algorithmic bytes of one float launch: the stored values, C and sigma, the work items
        hb32 = pairs * 4 + 2 * n * R * 4 + stats["n_work_items"] * 24
        stored = {"sigma_builds_per_s": 1e3 / hms32, "ms_per_step": hms32, "kernel_ms": hk32,
                  "fp64": {"sigma_builds_per_s": 1e3 / hms64, "ms_per_step": hms64, "kernel_ms": hk64},
                  "pairs": pairs, "bytes": hc_bytes, "assembly_s": hc_s,
                  "assembly_over_direct_fp64_sigma": hc_s / (ms64 * 1e-3),
                  "speedup_over_direct": {"fp32": ms32 / hms32, "fp64": ms64 / hms64},
                  "rel_err_vs_direct_fp64": {"fp64": hrel64, "fp32": hrel32},
                  "hbm_gbs_fp32": hb32 / (hk32 * 1e-3) / 1e9}
        g.cache_hamiltonian(0)  # the rest of this leg times the direct build

    # end to end through the C ABI with pinned host buffers
    h_c = torch.from_numpy(np.asfortranarray(v).T.copy()).pin_memory()
    h_s = torch.empty_like(h_c).pin_memory()
    import ctypes
    L = g.L
    for _ in range(a.warmup):
        L.fcg_sigma_closed(g.h, R, ctypes.c_void_p(h_c.data_ptr()), ctypes.c_void_p(h_s.data_ptr()), 1)
    # per-step wall time of the C-ABI call (H2D of C, sigma, D2H of sigma)
    walls = []
    for _ in range(a.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        L.fcg_sigma_closed(g.h, R, ctypes.c_void_p(h_c.data_ptr()), ctypes.c_void_p(h_s.data_ptr()), 1)
        walls.append(time.perf_counter() - t1)
    e2e_ms = max_over_ranks(1e3 * statistics.mean(walls), world)

    value = world * 1e3 / ms32
    # algorithmic (compulsory) bytes of one FP32 sigma launch
    N = prob.ham.n_clusters
    op_bytes = po.data.size * 4 + pt.ints.size * 4
    vec_bytes = 2 * n * R * 4
    idx_bytes = n * (2 * N + 4 * N)
    alg_bytes = op_bytes + vec_bytes + idx_bytes
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / (k32 * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": "sigma_builds/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (mixed; fp64 line in fp64)", "data": "synthetic",
        "config": bench_config(n, R, world),
        "workload_stats": {"n_terms": prob.ham.n_terms(), "triples_per_sigma": stats["n_triples"],
                           "work_items": stats["n_work_items"], "plan_seconds": stats["plan_seconds"],
                           "join_seconds": stats["join_seconds"], "join_on_device": bool(stats["join_on_device"]),
                           "state_set_ms": {"first": 1e3 * t_set[0], "warm": 1e3 * min(t_set[1:])},
                           "plan_over_fp64_sigma": 1e3 * stats["plan_seconds"] / k64},
        "fp64": {"value": world * 1e3 / ms64, "ms_per_step": ms64, "kernel_ms": k64,
                 "mixed_over_fp64": ms64 / ms32, "fp32_rel_err_vs_fp64": rel32},
        "flops_reference_per_sigma": stats["flops_reference"],
        "gflops_reference_count": {"fp32": stats["flops_reference"] / (k32 * 1e-3) / 1e9,
                                   "fp64": stats["flops_reference"] / (k64 * 1e-3) / 1e9},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak,
                     # dram__bytes_read.sum + dram__bytes_write.sum of one float launch on this
                     # exact workload, from the ncu capture summarised in
                     # profiles/closed_sigma_lane_kernel_24o6c.md
                     "traffic": (334.6e6 + 1.5e6) if (n == 100000 and R == 4) else None,
                     "note": "compulsory bytes per launch / closed_sigma_lane_kernel time (fp32), of measured HBM "
                             "copy peak; the float kernel is bound by the L1 data pipe (87 % of peak) and the "
                             "double kernel by the FP64 pipe, not by HBM"},
        "e2e": {"value": 1e3 / e2e_ms, "unit": "sigma_builds/s", "h2d_bytes_per_step": n * R * 8,
                "d2h_bytes_per_step": n * R * 8},
        "gpu_launches": int(g.stats()["kernel_launches"]) * a.steps,
        "tuning": dict(g.tuning(), note="closed-sigma kernel candidate chosen by the library's tuner on the "
                                        "first sigma of each precision (index into candidates)"),
        "clocks": clocks,
    }
    if stored is not None:
        # the stored-block kernel's own roofline: algorithmic bytes (stored float32 values, C,
        # sigma, work items) per launch over its CUDA-event time, of the measured HBM copy peak
        stored["roofline"] = {"bound": "hbm", "achieved": stored["hbm_gbs_fp32"], "peak": hbm_peak, "unit": "GB/s",
                              "frac": stored["hbm_gbs_fp32"] / hbm_peak,
                              "note": "cached_sigma_kernel<float>; bound by the L1 data pipe (ket and C-row "
                                      "gathers), not HBM"}
        out["stored_blocks"] = stored
    if rank == 0 and a.davidson:
        try:
            out["headline_solve"] = headline_solve(g, n, R)
        except Exception as ex:
            out["headline_solve"] = {"error": str(ex)}
    if rank == 0 and a.serving:
        try:
            out["serving"] = serving_benchmark()
        except Exception as ex:
            out["serving"] = {"error": str(ex)}
    if rank == 0 and a.open:
        try:
            out["open_sigma"] = open_benchmark(max(3, a.steps // 4), a.warmup, a.cpu_seconds, n_cfg=a.open_cfg)
        except Exception as ex:
            out["open_sigma"] = {"error": str(ex)}
    if rank == 0 and a.batched:
        try:
            out["batched"] = batched_benchmark(max(3, a.steps // 2), a.warmup, a.instances, a.stored)
        except Exception as ex:
            out["batched"] = {"error": str(ex)}
    if rank == 0 and a.bst:
        try:
            out["bst"] = bst_benchmark(max(3, a.steps // 2), a.warmup, a.cpu_seconds, peaks, a.bst_sectors, a.bst_maxq)
        except Exception as ex:
            out["bst"] = {"error": str(ex)}
    if rank == 0 and a.davidson:
        try:
            out["davidson"] = davidson_benchmark(stored=a.stored)
        except Exception as ex:
            out["davidson"] = {"error": str(ex)}
    if rank == 0 and a.fois:
        try:
            out["bst_fois"] = fois_benchmark(max(3, a.steps // 4), a.warmup, a.cpu_seconds)
        except Exception as ex:
            out["bst_fois"] = {"error": str(ex)}
    if rank == 0 and a.tpsci:
        try:
            out["tpsci"] = tpsci_benchmark(a.cpu_seconds)
        except Exception as ex:
            out["tpsci"] = {"error": str(ex)}
    if rank == 0 and a.cpu_seconds > 0:
        try:
            thr = os.cpu_count() or 1
            cv, sample, ref = cpu_reference(po, pt, f, c, v, a.cpu_seconds, thr)
            out["cpu_baseline"] = {"value": cv, "unit": "sigma_builds/s", "cores": thr, "kind": "port",
                                   "sample": sample}
            out["gpu_over_cpu"] = {"mixed": out["value"] / cv, "fp64": out["fp64"]["value"] / cv,
                                   "e2e_mixed": out["e2e"]["value"] / cv}
            if ref is not None:
                # the headline sigma against the oracle's full build of the same C (every row)
                s64 = sig64.double().cpu().numpy().T
                s32 = sig32.double().cpu().numpy().T
                scale = float(np.abs(ref).max())
                out["parity"] = {"oracle": "oracle tps_ci_matvec restatement, full build, all rows",
                                 "fp64_rel": float(np.abs(s64 - ref).max()) / scale,
                                 "fp32_rel": float(np.abs(s32 - ref).max()) / scale,
                                 "tolerance": {"fp64": 1e-10, "fp32": 2e-5}}
                out["parity"]["ok"] = bool(out["parity"]["fp64_rel"] <= 1e-10 and out["parity"]["fp32_rel"] <= 2e-5)
        except Exception as ex:  # the baseline must not kill the GPU line
            out["cpu_baseline"] = {"value": None, "error": str(ex)}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
