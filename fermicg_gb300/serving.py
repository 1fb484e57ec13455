"""A request loop serving Davidson solves on one GPU (continuous batching).

Requests (a problem = cluster operators + clustered Hamiltonian, a variational space,
a starting guess, a root count and a tolerance) arrive over time.  A request is admitted
as soon as a slot is free and its estimated HBM footprint fits the budget; admitted
requests run concurrently, each on its own device context and CUDA stream, so their
sigma builds and Davidson steps overlap on the GPU.  Operators, subspace vectors and the
sigma plan of a request stay resident on the device for the whole solve.  Each request's
latency runs from its arrival to its result.

The per-request work is exactly the standalone solve (fcg_set_ops, fcg_set_terms,
fcg_state_set, fcg_davidson), so a result does not depend on what else is in flight.
"""
from __future__ import annotations

import heapq
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from .gpu import PRECISION, FcgError, GpuSigma, _ptr


@dataclass(order=True)
class Request:
    arrival: float
    rid: int = field(compare=False)
    packed_ops: object = field(compare=False, default=None)
    packed_terms: object = field(compare=False, default=None)
    focks: np.ndarray = field(compare=False, default=None)
    cfgs: np.ndarray = field(compare=False, default=None)
    guess: np.ndarray = field(compare=False, default=None)
    tol: float = field(compare=False, default=1e-6)
    precision: str = field(compare=False, default="fp64")
    max_iter: int = field(compare=False, default=200)
    shape: str = field(compare=False, default="")
    cache: bool = field(compare=False, default=False)  # store the Hamiltonian blocks (fcg_cache_hamiltonian)
    # a BST solve (ci_solve, src/tucker_outer.jl:68-215) instead of a TPSCI one: the packed
    # Tucker blocks (focks / cfgs unused; guess (core_total, R)) and the preconditioner diagonal
    bst: object = field(compare=False, default=None)
    bst_hd: np.ndarray = field(compare=False, default=None)


@dataclass
class Result:
    rid: int
    shape: str
    energies: np.ndarray
    residuals: np.ndarray
    iters: int
    arrival: float
    start: float
    end: float

    @property
    def latency(self):
        return self.end - self.arrival


def footprint_bytes(req: Request) -> int:
    """HBM a solve holds while admitted: operators (float64 + float32 copies), dressed
    operators (estimated as 8x the TDM blob, both precisions), the state index, and the
    Davidson subspace (2 x 12R vectors) plus sigma working copies.  A BST solve holds its
    operator cache instead of the dressed operators and index, estimated from its cores
    (64 cached elements per core element, both precisions)."""
    n = req.guess.shape[0]
    R = req.guess.shape[1]
    ops = req.packed_ops.data.size * 12
    ints = req.packed_terms.ints.size * 12
    dav = n * 8 * (2 * (12 * R + R) + 6 * R)
    if req.bst is not None:
        return int(ops + ints + n * 64 * 12 + dav)
    dressed = req.packed_ops.data.size * 8 * 12
    index = n * (16 + 8 * 60)
    return int(ops + dressed + ints + index + dav)


class SolveServer:
    def __init__(self, slots: int = 4, hbm_budget: float = 64e9, device: int = 0):
        self.slots = slots
        self.budget = hbm_budget
        self.device = device
        self._lock = threading.Condition()
        self._in_use = 0
        self._active = 0
        self.results: list[Result] = []
        self._ctx_pool = [None] * slots

    def _run_one(self, slot: int, req: Request, fp: int):
        start = time.perf_counter()
        g = self._ctx_pool[slot]
        if g is None:
            g = GpuSigma(self.device)
            self._ctx_pool[slot] = g
        extra = 0
        try:
            g.set_ops(req.packed_ops)
            g.set_terms(req.packed_terms)
            if req.bst is not None:
                g.bst_set(req.bst)
                e, X, res, it = g.bst_davidson(req.guess, req.bst_hd, tol=req.tol, max_iter=req.max_iter,
                                               precision=req.precision)
                end = time.perf_counter()
                with self._lock:
                    self.results.append(Result(req.rid, req.shape, e, res, it, req.arrival, start, end))
                return
            g.state_set(req.focks, req.cfgs)
            if req.cache:  # within the memory the admitted solves leave free, else the direct build
                with self._lock:
                    room = self.budget - self._in_use
                try:
                    extra = g.cache_hamiltonian(max(room, 0))
                    with self._lock:
                        self._in_use += extra
                except FcgError:
                    extra = 0
            e, X, res, it = g.davidson(req.guess, tol=req.tol, max_iter=req.max_iter, precision=req.precision)
            end = time.perf_counter()
            with self._lock:
                self.results.append(Result(req.rid, req.shape, e, res, it, req.arrival, start, end))
        finally:
            # the pooled context keeps the stored blocks' buffers for its next request (the next
            # state invalidates them; freeing would wait for every stream of the device)
            with self._lock:
                self._in_use -= fp + extra
                self._active -= 1
                self._free_slots.append(slot)
                self._lock.notify_all()

    def run(self, requests: list[Request], t0: float | None = None):
        """Serve `requests` (arrival times relative to t0 = now); returns the results."""
        pending = sorted(requests)
        t0 = time.perf_counter() if t0 is None else t0
        for r in pending:
            r.arrival = t0 + r.arrival
        self._free_slots = list(range(self.slots))
        threads = []
        queue: list = []
        i = 0
        while i < len(pending) or queue:
            now = time.perf_counter()
            while i < len(pending) and pending[i].arrival <= now:
                heapq.heappush(queue, pending[i])
                i += 1
            admitted = False
            with self._lock:
                if queue and self._free_slots:
                    fp = footprint_bytes(queue[0])
                    if self._in_use + fp <= self.budget or self._active == 0:
                        req = heapq.heappop(queue)
                        slot = self._free_slots.pop()
                        self._in_use += fp
                        self._active += 1
                        th = threading.Thread(target=self._run_one, args=(slot, req, fp), daemon=True)
                        th.start()
                        threads.append(th)
                        admitted = True
                if not admitted:
                    wait = 0.01
                    if i < len(pending):
                        wait = max(0.0, min(wait, pending[i].arrival - time.perf_counter()))
                    self._lock.wait(timeout=wait if wait > 0 else 0.0005)
        for th in threads:
            th.join()
        return sorted(self.results, key=lambda r: r.rid)

    def close(self):
        for g in self._ctx_pool:
            if g is not None:
                g.close()


def latency_summary(results: list[Result]):
    lat = np.array([r.latency for r in results])
    span = max(r.end for r in results) - min(r.arrival for r in results)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "solves_per_s": len(results) / span, "n": len(results)}


class NativeSolveServer:
    """The library's continuous-batching server (fcg_server_create / fcg_submit / fcg_wait).

    Each request is set up in a host thread of its own (a pooled context: fcg_set_ops,
    fcg_set_terms, fcg_state_set; at most 2 x slots requests hold a context at one time, the
    others wait in arrival order) and submitted when ready; the library's `lanes` scheduler
    threads (a stream each) admit requests while fewer than `slots` run and the memory budget
    allows, and each advances its admitted solves together: one wait for its stream, or one
    grouped sigma launch per precision, per round for all of them, with finished solves
    leaving and new ones joining between rounds.  Latency runs from a request's arrival to its
    result, set-up included."""

    def __init__(self, slots: int = 16, hbm_budget: float = 64e9, device: int = 0, lanes: int = 4,
                 cache_budget: float = 8e9):
        import ctypes
        from .gpu import load_library
        self._ct = ctypes
        self.L = load_library()
        h = ctypes.c_void_p()
        rc = self.L.fcg_server_create(device, int(slots), int(lanes), float(hbm_budget), ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"fcg_server_create failed ({rc})")
        self.h = h
        self.device = device
        self.cache_budget = cache_budget  # largest stored Hamiltonian of one request (bytes)
        self._free = []
        self._lock = threading.Lock()
        self.results: list[Result] = []
        # requests prepared or in the library at one time: each holds a context with its problem
        # on the device, so the rest wait on the host (in arrival order) until one ends
        self._prepared = threading.Semaphore(2 * int(slots))

    def _context(self):
        with self._lock:
            if self._free:
                return self._free.pop()
        return GpuSigma(self.device)

    def _serve(self, req: Request, t0: float):
        ct = self._ct
        wait = req.arrival - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        self._prepared.acquire()
        start = time.perf_counter()
        g = self._context()
        try:
            g.set_ops(req.packed_ops)
            g.set_terms(req.packed_terms)
            v = np.asfortranarray(req.guess, dtype=np.float64)
            n, R = v.shape
            ticket = ct.c_int64(0)
            if req.bst is not None:
                g.bst_set(req.bst)
                hd = None if req.bst_hd is None else np.ascontiguousarray(req.bst_hd, dtype=np.float64)
                g._check(self.L.fcg_submit_bst(self.h, g.h, R, _ptr(v), _ptr(hd) if hd is not None else None,
                                               int(req.max_iter), 12, float(req.tol), 1e-12, PRECISION[req.precision],
                                               ct.byref(ticket)), "fcg_submit_bst")
            else:
                g.state_set(req.focks, req.cfgs)
                if req.cache:
                    try:
                        g.cache_hamiltonian(self.cache_budget)
                    except FcgError:  # larger than a request may store: the direct build
                        pass
                g._check(self.L.fcg_submit(self.h, g.h, R, _ptr(v), int(req.max_iter), 12, float(req.tol), 1e-12,
                                           PRECISION[req.precision], 1, ct.byref(ticket)), "fcg_submit")
            e, res = np.zeros(R), np.zeros(R)
            X = np.zeros((n, R), order="F")
            it = ct.c_int(0)
            while True:
                rc = self.L.fcg_wait(self.h, ticket.value, 1000, _ptr(e), _ptr(X), _ptr(res), ct.byref(it))
                if rc != -5:  # FCG_ETIMEDOUT: keep waiting
                    break
            g._check(rc, "fcg_wait")
            end = time.perf_counter()
            with self._lock:
                self.results.append(Result(req.rid, req.shape, e, res, it.value, req.arrival, start, end))
        finally:
            with self._lock:  # the pooled context keeps its buffers for the next request
                self._free.append(g)
            self._prepared.release()

    def run(self, requests: list[Request], t0: float | None = None):
        """Serve `requests` (arrival times relative to t0 = now); returns the results by id."""
        t0 = time.perf_counter() if t0 is None else t0
        reqs = sorted(requests)
        for r in reqs:
            r.arrival = t0 + r.arrival
        errors = []

        def work(r):
            try:
                self._serve(r, t0)
            except Exception as ex:  # reported after all threads end
                errors.append(ex)

        threads = [threading.Thread(target=work, args=(r,), daemon=True) for r in reqs]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
        return sorted(self.results, key=lambda r: r.rid)

    def close(self):
        if getattr(self, "h", None):
            self.L.fcg_server_destroy(self.h)
            self.h = None
        for g in self._free:
            g.close()
        self._free = []
