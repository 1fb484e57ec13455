"""Serving loop: concurrent Davidson solves give the same result alone and in the mix."""
import numpy as np
import pytest

from fermicg_gb300 import pack, workloads
from fermicg_gb300.serving import Request, SolveServer, latency_summary

pytestmark = pytest.mark.gpu


def _request(rid, prob, n_cfg, R, seed, arrival, precision="fp64"):
    st = workloads.energy_ordered_space(prob, n_cfg, R=R, seed=seed)
    f, c, v, _ = pack.pack_state(st)
    guess = workloads.davidson_guess(f.shape[0], R, seed=seed)  # lowest configurations first
    return Request(arrival, rid, pack.pack_ops(prob.ops, prob.bases), pack.pack_terms(prob.ham), f, c, guess,
                   tol=1e-7, precision=precision, shape=f"{prob.meta['norb']}o")


def test_results_alone_equal_results_in_the_mix():
    p0 = workloads.build_problem(12, [3, 3, 3, 3], [(2, 1), (1, 2), (2, 1), (1, 2)], 36, 3, max_roots=1000)
    p1 = workloads.build_problem(16, [4, 4, 4, 4], [(2, 2)] * 4, 24, 4, max_roots=12, delta_elec=2)
    reqs = [_request(i, p0 if i % 2 == 0 else p1, 1500 if i % 2 == 0 else 3000, 1 + (i % 3), i, 0.002 * i)
            for i in range(8)]
    alone = []
    for r in reqs:
        srv = SolveServer(slots=1)
        alone.append(srv.run([Request(0.0, r.rid, r.packed_ops, r.packed_terms, r.focks, r.cfgs, r.guess, r.tol,
                                      r.precision, r.max_iter, r.shape)])[0])
        srv.close()
    srv = SolveServer(slots=4)
    mixed = srv.run(reqs)
    srv.close()
    assert len(mixed) == len(reqs)
    for a, m in zip(alone, mixed):
        assert a.rid == m.rid
        np.testing.assert_allclose(m.energies, a.energies, rtol=0, atol=1e-9)
        assert m.residuals.max() < 1e-7
    s = latency_summary(mixed)
    assert s["p99_s"] >= s["p50_s"] > 0


@pytest.mark.parametrize("slots,lanes", [(3, 1), (4, 2)])
def test_native_server_results_equal_results_alone(slots, lanes):
    """fcg_server (continuous batching, grouped sigma builds; one lane, and two lanes of two
    solves each): each request's energies equal its solve alone."""
    from fermicg_gb300.serving import NativeSolveServer
    p0 = workloads.build_problem(12, [3, 3, 3, 3], [(2, 1), (1, 2), (2, 1), (1, 2)], 36, 3, max_roots=1000)
    p1 = workloads.build_problem(16, [4, 4, 4, 4], [(2, 2)] * 4, 24, 4, max_roots=12, delta_elec=2)
    reqs = [_request(i, p0 if i % 2 == 0 else p1, 1500 if i % 2 == 0 else 3000, 1 + (i % 3), i, 0.002 * i,
                     precision="fp64" if i % 4 < 2 else "fp32")
            for i in range(8)]
    alone = []
    for r in reqs:
        srv = SolveServer(slots=1)
        alone.append(srv.run([Request(0.0, r.rid, r.packed_ops, r.packed_terms, r.focks, r.cfgs, r.guess, r.tol,
                                      r.precision, r.max_iter, r.shape)])[0])
        srv.close()
    srv = NativeSolveServer(slots=slots, lanes=lanes)
    mixed = srv.run(reqs)
    srv.close()
    assert [m.rid for m in mixed] == [r.rid for r in reqs]
    for a, m in zip(alone, mixed):
        np.testing.assert_allclose(m.energies, a.energies, rtol=0, atol=1e-9)
        assert m.residuals.max() < 1e-7


def test_native_server_wait_times_out_and_a_failed_request_leaves_the_others():
    import ctypes
    from fermicg_gb300.gpu import GpuSigma, load_library, _ptr
    L = load_library()
    p0 = workloads.build_problem(12, [3, 3, 3, 3], [(2, 1), (1, 2), (2, 1), (1, 2)], 36, 3, max_roots=1000)
    h = ctypes.c_void_p()
    assert L.fcg_server_create(0, 1, 1, 1e10, ctypes.byref(h)) == 0
    gs, tickets, guesses = [], [], []
    for i in range(3):
        r = _request(i, p0, 1500, 1, 0, 0.0)  # requests 0 and 2 are the same solve
        g = GpuSigma(0)
        g.set_ops(r.packed_ops)
        g.set_terms(r.packed_terms)
        g.state_set(r.focks, r.cfgs)
        guess = np.asfortranarray(r.guess.copy())
        if i == 1:
            guess[:] = np.nan  # fails inside the solve: no usable initial direction
        t = ctypes.c_int64(0)
        assert L.fcg_submit(h, g.h, 1, _ptr(guess), 200, 12, 1e-7, 1e-12, 0, 1, ctypes.byref(t)) == 0
        gs.append(g)
        tickets.append(t.value)
        guesses.append(guess)
    # one slot: the last request is still queued behind the first
    e = np.zeros(1)
    assert L.fcg_wait(h, tickets[2], 0, _ptr(e), None, None, None) == -5  # FCG_ETIMEDOUT
    st = ctypes.c_int(-1)
    assert L.fcg_poll(h, tickets[2], ctypes.byref(st)) == 0 and st.value in (0, 1)
    it = ctypes.c_int(0)
    assert L.fcg_wait(h, tickets[0], 60000, _ptr(e), None, None, ctypes.byref(it)) == 0 and it.value > 0
    e_ok = e.copy()
    assert L.fcg_wait(h, tickets[1], 60000, _ptr(e), None, None, None) != 0
    assert b"linearly dependent" in L.fcg_last_error(gs[1].h)
    assert L.fcg_wait(h, tickets[2], 60000, _ptr(e), None, None, None) == 0
    np.testing.assert_allclose(e, e_ok, atol=1e-9)  # same problem, same guess
    assert L.fcg_server_destroy(h) == 0
    for g in gs:
        g.close()


@pytest.mark.parametrize("native", [False, True])
def test_stored_blocks_in_the_mix_give_the_same_energies(native):
    """Requests that store their Hamiltonian blocks (fcg_cache_hamiltonian) before the solve
    end with the energies of the same requests without them."""
    from fermicg_gb300.serving import NativeSolveServer
    p0 = workloads.build_problem(12, [3, 3, 3, 3], [(2, 1), (1, 2), (2, 1), (1, 2)], 36, 3, max_roots=1000)
    p1 = workloads.build_problem(16, [4, 4, 4, 4], [(2, 2)] * 4, 24, 4, max_roots=12, delta_elec=2)
    base = [_request(i, p0 if i % 2 == 0 else p1, 1500 if i % 2 == 0 else 3000, 1 + (i % 3), i, 0.002 * i,
                     precision="fp64" if i % 4 < 2 else "fp32")
            for i in range(6)]
    out = {}
    for cache in (False, True):
        reqs = [Request(r.arrival, r.rid, r.packed_ops, r.packed_terms, r.focks, r.cfgs, r.guess, r.tol,
                        r.precision, r.max_iter, r.shape, cache=cache) for r in base]
        srv = NativeSolveServer(slots=3, lanes=1) if native else SolveServer(slots=3)
        out[cache] = srv.run(reqs)
        srv.close()
    for a, b in zip(out[False], out[True]):
        assert a.rid == b.rid
        np.testing.assert_allclose(b.energies, a.energies, rtol=0, atol=1e-9)
        assert b.residuals.max() < 1e-7
