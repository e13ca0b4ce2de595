"""Metric tools on the GPU against the reference's own outputs
(tests/golden/metric, written by the reference through oracle/ref_driver):
intersection (Barral's degenerate cases included), clamping, Hessian
metrics, implied metrics, gradation limiting, the expected element count and
generate_metrics.  Every one of these goes through the closed-form
eigensolve, whose cube root the library takes correctly rounded while
glibc's is not (the reference's results depend on that last ulp near
repeated eigenvalues); the tensors are held to the suite's interpolation
tolerance relative to each tensor's largest entry, and the expected element
count to the one for reals derived from interpolated metrics (the measured
errors are printed: about 1e-12 on these cases)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "metric")
DEGENERATE = "degenerate_intersections"
CASES = sorted(f[:-4] for f in os.listdir(GOLD) if f.endswith(".npz") and f[:-4] != DEGENERATE)
from conftest import INTERP_RTOL, INTERP_TENSOR_RTOL  # noqa: E402

TOL = INTERP_TENSOR_RTOL


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


def _gold(case):
    g = dict(np.load(os.path.join(GOLD, case + ".npz")))
    meta = json.loads(bytes(g.pop("meta_json")).decode())
    return g, meta


def _close(want, got, what, nc):
    want = np.asarray(want).reshape(-1, nc)
    got = got.detach().cpu().numpy().reshape(-1, nc)
    scale = np.maximum(np.abs(want).max(axis=1, keepdims=True), 1e-300)
    err = (np.abs(want - got) / scale).max()
    nbit = int(np.sum(np.any(want.view(np.uint64) != got.view(np.uint64), axis=1)))
    print(f"{what}: max error {err:.2e}, {nbit}/{want.shape[0]} tensors not bitwise equal")
    assert err <= TOL, f"{what}: max error {err:.3e}"


# Metric kinds with two equal principal sizes (the shock's two tangential
# sizes, the boundary layer's x and z sizes): every intersection of such
# metrics solves a cubic with an exact double root through Cardano's branch,
# whose result depends on the cube root's last ulp (glibc's is not correctly
# rounded on half of all arguments), so the two sides differ by about 1e-7
# per intersection.  Gradation limiting repeats dozens of intersections per
# vertex per sweep until nothing changes by 1e-3, and on these metrics the
# reference's own iteration does not settle quickly (188 sweeps for
# box4_shock): the fixed point it stops at depends on the rounding.  These
# cases are checked on the properties the result must have instead.
REPEATED_SIZES = {"box4_shock", "sq8_blayer"}


def _full(x, nc):
    x = x.detach().cpu().numpy().reshape(-1, nc)
    if nc == 6:
        t = np.zeros((x.shape[0], 3, 3))
        t[:, 0, 0], t[:, 1, 1], t[:, 2, 2] = x[:, 0], x[:, 1], x[:, 2]
        t[:, 1, 0] = t[:, 0, 1] = x[:, 3]
        t[:, 2, 1] = t[:, 1, 2] = x[:, 4]
        t[:, 2, 0] = t[:, 0, 2] = x[:, 5]
    else:
        t = np.zeros((x.shape[0], 2, 2))
        t[:, 0, 0], t[:, 1, 1] = x[:, 0], x[:, 1]
        t[:, 1, 0] = t[:, 0, 1] = x[:, 2]
    return t


def _gradation_properties(m, grad, rate, tol, nc):
    """The result is (to tol) a fixed point of one more sweep and meets the
    gradation bound along every edge, v^T M_a v >= v^T M_b v / (1 + rate
    |e|_Mb)^2 in random directions v (the reference's outputs on these cases
    meet it with a margin of 1.5 or more)."""
    again, sweeps = m.limit_metric_gradation(grad, rate, tol)
    g, a = grad.cpu().numpy(), again.cpu().numpy()
    rel = np.abs(a - g).reshape(-1, nc).max(1) / np.abs(g).reshape(-1, nc).max(1)
    print(f"gradation fixed point: {sweeps} sweep(s), max change {rel.max():.2e}")
    assert sweeps <= 2 and rel.max() <= 10 * tol
    # (the reference's own output is not always at least as fine as its
    # input: merging near-double roots loses up to a few percent in some
    # directions, 4 % on box4_shock; so that is not a property to check)
    G = _full(grad, nc)
    rng = np.random.default_rng(0)
    ev = m.get("ev2v_1").cpu().numpy().reshape(-1, 2)
    X = m.get("coords").cpu().numpy().reshape(G.shape[0], -1)
    for a_, b_ in ((0, 1), (1, 0)):
        va, vb = ev[:, a_], ev[:, b_]
        e = X[vb] - X[va]
        mb = G[vb]
        dist = np.sqrt(np.einsum("ni,nij,nj->n", e, mb, e))
        lim = mb / ((1 + rate * dist) ** 2)[:, None, None]
        dd = rng.normal(size=(len(va), G.shape[1], 1))
        qa = (np.transpose(dd, (0, 2, 1)) @ G[va] @ dd).ravel()
        ql = (np.transpose(dd, (0, 2, 1)) @ lim @ dd).ravel()
        assert (qa >= ql * (1 - 2 * tol)).all()


def _mesh(ctx, meta):
    from omega_h_gb300.mesh import Mesh
    m = Mesh.build_box(ctx, meta["dim"], meta["n"])
    m.apply_workload(meta["n"], meta["seed"], meta["metric"])
    return m


@pytest.mark.parametrize("case", CASES)
def test_metric_tools_match_the_reference(ctx, case):
    import torch
    from omega_h_gb300.mesh import clamp_metrics, hessian_metrics, intersect_metrics
    g, meta = _gold(case)
    dim = meta["dim"]
    nc = 6 if dim == 3 else 3
    m = _mesh(ctx, meta)
    try:
        given = m.get("metric")
        assert np.array_equal(given.cpu().numpy(), g["mt_given"])
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
        _close(g["mt_implied"], m.implied_metrics(), "implied", nc)
        _close(g["mt_intersect"], intersect_metrics(ctx, dim, dev(g["mt_given"]),
                                                    dev(g["mt_implied"])), "intersect", nc)
        _close(g["mt_clamp"], clamp_metrics(ctx, dim, given, 0.02, 0.2), "clamp", nc)
        _close(g["mt_hessian_metrics"], hessian_metrics(ctx, dim, dev(g["mt_hessians"]), 0.01),
               "hessian", nc)
        grad, sweeps = m.limit_metric_gradation(given, 1.0, 1e-3)
        print(f"gradation: {sweeps} sweeps")
        ne = m.expected_nelems(given)
        want = float(g["mt_expected_nelems"][0])
        print(f"expected elements: relative error {abs(ne - want) / abs(want):.2e}")
        assert abs(ne - want) <= INTERP_RTOL * abs(want), (ne, want)
        out, niters = m.generate_metrics(
            [{"type": "given", "knob": 1.0, "metrics": given, "scales": True},
             {"type": "implied", "knob": 2.0, "isotropy": "iso_size", "scales": False},
             {"type": "constant", "knob": 0.3, "scales": False}],
            should_limit_lengths=1, min_length=0.05, max_length=0.5,
            should_limit_gradation=1, max_gradation_rate=1.0, nsmoothing_steps=1,
            should_limit_element_count=1, max_element_count=4.0 * m.nelems(),
            min_element_count=1.0 * m.nelems())
        print(f"generate_metrics: {niters} element-count iterations")
        if case in REPEATED_SIZES:
            _gradation_properties(m, grad, 1.0, 1e-3, nc)
        else:
            _close(g["mt_gradation"], grad, "gradation", nc)
            _close(g["mt_generated"], out, "generate_metrics", nc)
    finally:
        m.close()


def test_intersection_properties(ctx):
    """At a size the fixtures do not reach (24^3, the isotropic sine metric
    against the anisotropic implied metric): intersecting a metric with
    itself gives it back, and the intersection is at least as fine as each
    operand in every direction.  (On metrics with repeated sizes neither
    holds beyond the cubic solver's O(eps^(1/3)) resolution of a triple
    root, in the reference as here.)"""
    import torch
    from omega_h_gb300.mesh import Mesh, intersect_metrics
    m = Mesh.build_box(ctx, 3, 24)
    m.apply_workload(24, 11, 3)
    a = m.get("metric")
    b = m.implied_metrics()
    m.close()
    aa = intersect_metrics(ctx, 3, a, a)
    rel = ((aa - a).abs().view(-1, 6).amax(1) / a.abs().view(-1, 6).amax(1)).max().item()
    print(f"intersect(a, a) vs a: {rel:.2e}")
    assert rel < 1e-12, rel
    c = intersect_metrics(ctx, 3, a, b)
    G, A, B = (_full(t, 6) for t in (c, a, b))
    rng = np.random.default_rng(1)
    d = rng.normal(size=(G.shape[0], 3, 1))
    q = lambda T: (np.transpose(d, (0, 2, 1)) @ T @ d).ravel()  # noqa: E731
    ra, rb = (q(G) / q(A)).min(), (q(G) / q(B)).min()
    print(f"intersection vs operands: smallest ratios {ra:.12f} {rb:.12f}")
    assert ra >= 1 - 1e-9 and rb >= 1 - 1e-9


@pytest.mark.parametrize("dim", [2, 3])
def test_degenerate_intersections_match_reference(ctx, dim):
    """Barral's degenerate cases (src/Omega_h_metric_intersect.hpp:25-212) on
    seeded pairs of rank-1 and rank-2 metrics, in random orientations and in
    shared eigenbases, plus the reference's unit-test pairs, against the
    reference's own intersect_metrics.  Where the reference's 2D case 5.b
    meets parallel null directions (its test is v1 . v2 < 1e-10, so equal
    directions go to 5.b) it inverts a singular matrix: the result is
    infinite, not a number or huge depending on the last bit of the
    eigenvectors, and so must ours blow up on exactly those pairs."""
    import torch
    from omega_h_gb300 import _lib
    import ctypes
    g = dict(np.load(os.path.join(GOLD, DEGENERATE + ".npz")))
    nc = 6 if dim == 3 else 3
    a = torch.tensor(g[f"di{dim}_a"]).cuda()
    b = torch.tensor(g[f"di{dim}_b"]).cuda()
    want = g[f"di{dim}_out"].reshape(-1, nc)
    n = want.shape[0]
    out = torch.empty(n * nc, dtype=torch.float64, device="cuda")
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    _lib.call("ohg_intersect_metrics", ctx.handle, dim, n, P(a), P(b), P(out))
    got = out.cpu().numpy().reshape(-1, nc)

    def blown_up(x):
        with np.errstate(invalid="ignore"):
            return ~np.isfinite(x).all(axis=1) | (np.nan_to_num(np.abs(x), nan=0.0).max(axis=1) > 1e8)

    assert np.array_equal(blown_up(want), blown_up(got))
    rows = ~blown_up(want)
    w, o = want[rows], got[rows]
    scale = np.maximum(np.abs(w).max(axis=1, keepdims=True), 1e-300)
    err = float((np.abs(w - o) / scale).max())
    nbit = int(np.sum(np.any(w.view(np.uint64) != o.view(np.uint64), axis=1)))
    print(f"{dim}D degenerate intersections: {rows.sum()} finite of {n}, max error {err:.2e}, "
          f"{nbit} not bitwise equal")
    assert err <= TOL
