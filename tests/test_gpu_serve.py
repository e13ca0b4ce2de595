"""Serving with continuous batching: every request's result is bit for bit
its result alone, whatever it was batched with, and the admission budget
holds requests back without losing any."""
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


# (dim, n, metric kind, seed, passes, arrival s)
STREAM = [(3, 6, 1, 11, 2, 0.0), (2, 30, 3, 12, 1, 0.0), (3, 9, 2, 13, 3, 0.001),
          (2, 50, 1, 14, 2, 0.002), (3, 5, 3, 15, 1, 0.003), (2, 20, 2, 16, 3, 0.004),
          (3, 11, 3, 17, 2, 0.02), (2, 64, 3, 18, 1, 0.03)]


@pytest.fixture(scope="module")
def ctx2(ctx):
    from omega_h_gb300.mesh import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def more(ctx):
    from omega_h_gb300.mesh import Context
    cs = [Context(0), Context(0)]
    yield cs
    for c in cs:
        c.close()


def _mesh(ctx, dim, n, kind, seed):
    from omega_h_gb300.mesh import Mesh
    m = Mesh.build_box(ctx, dim, n)
    m.apply_workload(n, seed, kind)
    return m


def _arrays(m):
    names = ["coords", "metric", "ev2v_1", "ev2v_2", "down_1", "down_2", "downcodes_2",
             "length", "quality"]
    if m.dim == 3:
        names += ["ev2v_3", "down_3", "downcodes_3"]
    names += [f"class_id_{d}" for d in range(m.dim + 1)]
    return {k: m.get(k).cpu().numpy() for k in names}


@pytest.mark.parametrize("slots", [1, 2, 4], ids=["one_ctx", "two_ctx", "four_ctx"])
@pytest.mark.parametrize("budget", [150e9, 3e7], ids=["roomy", "tight"])
def test_served_results_equal_results_alone(ctx, ctx2, more, budget, slots):
    """Requests arrive as box specifications; each slot builds its meshes
    when they are routed to it, runs its own step loop, and the result of
    every request equals its result alone, bit for bit."""
    from omega_h_gb300.serve import Request, serve, summary
    alone = []
    for dim, n, kind, seed, passes, _ in STREAM:
        m = _mesh(ctx, dim, n, kind, seed)
        for _ in range(passes):
            m.adapt_pass()
        alone.append(_arrays(m))
        m.close()
    # slots per dimension: one context for both, one each, or two each
    per_dim = {1: {2: [ctx], 3: [ctx]}, 2: {2: [ctx2], 3: [ctx]},
               4: {2: [ctx2, more[0]], 3: [ctx, more[1]]}}[slots]
    reqs = [Request(rid=i, arrival=a, passes=p, dim=d, n=n, kind=k, seed=s)
            for i, (d, n, k, s, p, a) in enumerate(STREAM)]
    out = serve(per_dim, reqs, budget_bytes=budget)
    assert all(r.done >= r.built >= r.admitted >= r.arrival - 1e-9 and r.passes_done == r.passes
               for r in out)
    for r in out:
        got = _arrays(r.mesh)
        want = alone[r.rid]
        for k in want:
            assert np.array_equal(want[k].view(np.uint8), got[k].view(np.uint8)), \
                f"request {r.rid}: {k} differs from its result alone"
        r.mesh.close()
    s = summary(out)
    assert s["requests"] == len(STREAM) and s["p99_ms"] >= s["p50_ms"] > 0


def test_served_resident_meshes_stay_on_their_context(ctx, ctx2):
    """Requests may also bring a mesh already on the device; it is served by
    the slot of its own context and released when asked."""
    from omega_h_gb300.serve import Request, serve
    spec = STREAM[:4]
    alone = []
    for dim, n, kind, seed, passes, _ in spec:
        m = _mesh(ctx, dim, n, kind, seed)
        for _ in range(passes):
            m.adapt_pass()
        alone.append(_arrays(m))
        m.close()
    slots = {2: [ctx2], 3: [ctx]}
    reqs = [Request(rid=i, arrival=a, passes=p, mesh=_mesh(slots[d][0], d, n, k, s))
            for i, (d, n, k, s, p, a) in enumerate(spec)]
    out = serve(slots, reqs)
    for r in out:
        got = _arrays(r.mesh)
        for k, v in alone[r.rid].items():
            assert np.array_equal(v.view(np.uint8), got[k].view(np.uint8))
        r.mesh.close()
    reqs = [Request(rid=i, arrival=a, passes=p, dim=d, n=n, kind=k, seed=s)
            for i, (d, n, k, s, p, a) in enumerate(spec)]
    out = serve(slots, reqs, release=True)
    assert all(r.mesh is None and r.passes_done == r.passes for r in out)


def test_admission_counts_device_bytes(ctx, ctx2):
    """calibrate() measures bytes per element on the device; with a budget
    of about two meshes' footprint the loop never holds more than that in
    reservations, and every request still completes."""
    from omega_h_gb300.serve import Request, calibrate, serve
    bpe, peak = calibrate({2: ctx2, 3: ctx})
    assert all(100 < bpe[d] < 20000 and 1.0 <= peak[d] < 20 for d in (2, 3))
    reqs = [Request(rid=i, arrival=0.0, passes=1, dim=3, n=12, kind=1, seed=i) for i in range(6)]
    budget = 2.2 * bpe[3] * 6 * 12 ** 3
    trace = []
    out = serve({3: [ctx]}, reqs, budget_bytes=budget, bytes_per_element=bpe, pass_peak=peak,
                release=True, trace=trace)
    assert all(r.passes_done == 1 for r in out) and len(trace) == len(reqs)
    # every admission kept the reservations within the budget
    assert all(reserved <= budget for _, reserved, _ in trace)
    # and held requests back: never were all six in flight at once
    spans = sorted((r.admitted, r.done) for r in out)
    assert max(sum(1 for b, e in spans if b <= a < e) for a, _ in spans) < len(reqs)
