"""ohg_find_indset_graph on random graphs against the set the reference's
rules settle on (src/Omega_h_indset_inline.hpp:14-76): a candidate is in the
set exactly when no neighbour of higher rank, by (quality, index), is in it,
the greedy set by decreasing rank.  Qualities drawn from a few values make
most comparisons ties, so the index order decides them; the graphs are
large enough for many thread blocks and, in the largest, several vertices
per thread of the one cooperative launch, whose in-place state updates must
not change the set.  A path whose ranks decrease along it makes every
decision wait for the previous one: the longest chain of dependencies a
graph of its size can have."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from omega_h_gb300 import build
    build.build()
    from omega_h_gb300.mesh import Context
    c = Context(0)
    yield c
    c.close()


def _graph(n, deg, seed):
    """symmetric random graph with about deg neighbours per vertex, mostly
    between nearby indices (as in a Hilbert-ordered mesh), as CSR"""
    rng = np.random.default_rng(seed)
    m = n * deg // 2
    a = rng.integers(0, n, m)
    b = np.clip(a + rng.integers(-40, 41, m), 0, n - 1)
    keep = a != b
    a, b = a[keep], b[keep]
    src = np.concatenate([a, b])
    dst = np.concatenate([b, a])
    pairs = np.unique(np.stack([src, dst], 1), axis=0)
    xadj = np.zeros(n + 1, np.int32)
    np.add.at(xadj, pairs[:, 0] + 1, 1)
    xadj = np.cumsum(xadj).astype(np.int32)
    return xadj, pairs[:, 1].astype(np.int32)


def _greedy(xadj, adj, q, cands):
    n = len(q)
    order = np.lexsort((np.arange(n), q))[::-1]  # decreasing (quality, index)
    state = np.zeros(n, np.int8)
    for v in order:
        if not cands[v]:
            continue
        nb = adj[xadj[v]:xadj[v + 1]]
        if not np.any(state[nb] == 1):
            state[v] = 1
    return state


@pytest.mark.parametrize("n,deg,levels,seed", [(1000, 6, 3, 1), (60_000, 12, 4, 2),
                                               (200_000, 14, 1000, 3), (200_000, 8, 2, 4)])
def test_indset_is_the_greedy_set_by_rank(ctx, n, deg, levels, seed):
    import torch
    from omega_h_gb300 import _lib
    xadj, adj = _graph(n, deg, seed)
    rng = np.random.default_rng(seed + 100)
    q = rng.integers(0, levels, n).astype(np.float64) / levels
    cands = (rng.random(n) < 0.7).astype(np.int8)
    want = _greedy(xadj, adj, q, cands)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dx, da, dq, dc = dev(xadj), dev(adj), dev(q), dev(cands)
    out = torch.full((n,), -1, dtype=torch.int8, device="cuda")
    rounds = ctypes.c_int(-1)
    for _ in range(3):  # the schedule varies between calls; the set may not
        _lib.call("ohg_find_indset_graph", ctx.handle, n, ctypes.c_void_p(dx.data_ptr()),
                  ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(dq.data_ptr()),
                  ctypes.c_void_p(dc.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                  ctypes.byref(rounds))
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), want)
        assert rounds.value >= 1


def _run(ctx, xadj, adj, q, cands):
    import torch
    from omega_h_gb300 import _lib
    n = len(q)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dx, da, dq, dc = dev(xadj), dev(adj if len(adj) else np.zeros(1, np.int32)), dev(q), dev(cands)
    out = torch.full((n,), -1, dtype=torch.int8, device="cuda")
    rounds = ctypes.c_int(-1)
    _lib.call("ohg_find_indset_graph", ctx.handle, n, ctypes.c_void_p(dx.data_ptr()),
              ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(dq.data_ptr()),
              ctypes.c_void_p(dc.data_ptr()), ctypes.c_void_p(out.data_ptr()),
              ctypes.byref(rounds))
    torch.cuda.synchronize()
    return out.cpu().numpy(), rounds.value


def test_indset_more_vertices_than_threads(ctx):
    n = 900_000
    xadj, adj = _graph(n, 6, 7)
    rng = np.random.default_rng(107)
    q = rng.integers(0, 50, n).astype(np.float64) / 50
    cands = (rng.random(n) < 0.8).astype(np.int8)
    got, rounds = _run(ctx, xadj, adj, q, cands)
    assert np.array_equal(got, _greedy(xadj, adj, q, cands))
    assert rounds >= 1


@pytest.mark.parametrize("n", [2, 3, 30_000])
def test_indset_path_with_decreasing_ranks(ctx, n):
    """every vertex waits for its predecessor: IN, NOT_IN, IN, ..."""
    src = np.concatenate([np.arange(n - 1), np.arange(1, n)])
    dst = np.concatenate([np.arange(1, n), np.arange(n - 1)])
    order = np.lexsort((dst, src))
    xadj = np.zeros(n + 1, np.int32)
    np.add.at(xadj, src + 1, 1)
    xadj = np.cumsum(xadj).astype(np.int32)
    adj = dst[order].astype(np.int32)
    q = np.linspace(1.0, 0.0, n)
    got, _ = _run(ctx, xadj, adj, q, np.ones(n, np.int8))
    want = (np.arange(n) % 2 == 0).astype(np.int8)
    assert np.array_equal(got, want)


def test_indset_without_candidates_and_single_vertex(ctx):
    n = 5000
    xadj, adj = _graph(n, 6, 9)
    q = np.random.default_rng(9).random(n)
    got, _ = _run(ctx, xadj, adj, q, np.zeros(n, np.int8))
    assert not got.any()
    got, _ = _run(ctx, np.array([0, 0], np.int32), np.zeros(0, np.int32), np.array([0.5]),
                  np.ones(1, np.int8))
    assert got.tolist() == [1]
