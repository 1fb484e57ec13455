"""FlatTPSCI (the array form the GPU TPSCI driver uses for first-order spaces) against
TPSCIstate: the same configurations, coefficients and row order after every operation."""
import numpy as np

from fermicg_gb300.state import (FlatTPSCI, SectorRegistry, TPSCIstate, add_state, clip, copy_state, minus_state,
                                 overlap, project_out, times_matrix, zero_state)

N, R = 3, 2
SECTORS = [((1, 1), (0, 1), (1, 0)), ((0, 1), (1, 1), (1, 0)), ((1, 0), (1, 1), (0, 1)), ((2, 0), (0, 1), (0, 1))]


def _random_state(rng, n, scale=1.0):
    s = TPSCIstate(N, R)
    for _ in range(n):
        f = SECTORS[int(rng.integers(len(SECTORS)))]
        c = tuple(int(x) for x in rng.integers(0, 5, size=N))
        s[(f, c)] = scale * rng.standard_normal(R)
    return s


def _same(flat: FlatTPSCI, st: TPSCIstate):
    f1, c1, v1 = flat.rows()
    f2, c2, v2, _ = st.flat()
    assert np.array_equal(f1, f2) and np.array_equal(c1, c2)
    np.testing.assert_allclose(v1, v2, atol=1e-13, rtol=0)


def test_flat_operations_match_tpscistate():
    rng = np.random.default_rng(0)
    reg = SectorRegistry(N, [5, 5, 5])
    for trial in range(20):
        A, B = _random_state(rng, 60), _random_state(rng, 40)
        fa, fb = FlatTPSCI.from_state(reg, A), FlatTPSCI.from_state(reg, B)
        _same(fa, A)
        np.testing.assert_allclose(fa.overlap(fb), overlap(A, B), atol=1e-12)
        C = np.array([[0.3, -1.2], [0.7, 0.4]])
        _same(fa.times_matrix(C), times_matrix(A, C))
        _same(fa.minus(fb), minus_state(A, B))
        a2, A2 = fa.copy(), copy_state(A)
        a2.add(fb)
        add_state(A2, B)
        _same(a2, A2)
        # a sector emptied by clip goes to the end when it comes back
        a3, A3 = a2.copy(), copy_state(A2)
        a3.clip(0.8)
        clip(A3, 0.8)
        _same(a3, A3)
        a3.project_out(fb)
        project_out(A3, B)
        _same(a3, A3)
        a3.add(fa)
        add_state(A3, A)
        _same(a3, A3)
        a3.zero()
        zero_state(A3)
        _same(a3, A3)
        v = rng.standard_normal((len(a3), R))
        a3.set_vector(v)
        A3.set_vector(v)
        _same(a3, A3)
        assert a3.to_state().as_dict().keys() == A3.as_dict().keys()


def test_rows_of_new_sectors_keep_their_first_appearance_order():
    reg = SectorRegistry(N, [5, 5, 5])
    s = FlatTPSCI(reg, 1)
    rows = [(SECTORS[2], (1, 0, 0)), (SECTORS[0], (0, 0, 1)), (SECTORS[2], (0, 2, 0))]
    f = np.array([r[0] for r in rows], dtype=np.int16)
    c = np.array([r[1] for r in rows], dtype=np.int16)
    t = FlatTPSCI.from_rows(reg, 1, f, c, np.ones((3, 1)))
    s.add(t)
    st = TPSCIstate(N, 1)
    for r in rows:
        st[r] = np.ones(1)
    _same(s, st)


def test_empty_states_and_round_trip():
    reg = SectorRegistry(N, [5, 5, 5])
    empty = FlatTPSCI(reg, R)
    other = FlatTPSCI.from_state(reg, _random_state(np.random.default_rng(3), 30))
    assert len(empty) == 0 and empty.get_vector().shape == (0, R)
    np.testing.assert_array_equal(empty.overlap(other), np.zeros((R, R)))
    np.testing.assert_array_equal(other.overlap(empty), np.zeros((R, R)))
    e2 = empty.copy()
    e2.project_out(other)
    e2.clip(1.0)
    assert len(e2) == 0 and len(empty.times_matrix(np.eye(R))) == 0
    # adding into an empty state keeps the added state's row order
    e2.add(other)
    st = other.to_state()
    _same(e2, st)
    # TPSCIstate -> FlatTPSCI -> TPSCIstate keeps configurations, values and order
    back = FlatTPSCI.from_state(reg, st).to_state()
    f1, c1, v1, _ = back.flat()
    f2, c2, v2, _ = st.flat()
    assert np.array_equal(f1, f2) and np.array_equal(c1, c2) and np.array_equal(v1, v2)


def test_keys_refuse_to_overflow():
    import pytest
    reg = SectorRegistry(2, [1 << 30, 1 << 30])  # 2^60 configurations per sector: 4 sectors fit in 2^62
    focks = np.array([[[a, 0], [0, 0]] for a in range(6)], dtype=np.int16)
    with pytest.raises(OverflowError):
        reg.sector_ids(focks)
