"""Known answers of the reference's unit tests, through the C ABI on the GPU:
sort_by_keys, offset_scan, invert_adj (src/unit_array_algs.cpp:36-57,
75-84, 138-148), reflect_down, find_unique, downward adjacencies of
single simplices, stars, the dual graph, element qualities and refine
qualities (src/unit_mesh.cpp:130-169, 197-206, 245-315, 317-359,
382-391)."""
import ctypes
import math

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


def _dev(a, dtype):
    import torch
    return torch.tensor(np.asarray(a), dtype=dtype).cuda()


def _P(t):
    return ctypes.c_void_p(t.data_ptr() if t is not None and t.numel() else 0)


def code(flip, rot, wd):
    return (wd << 3) | (rot << 1) | int(flip)


@pytest.mark.parametrize("keys,width,perm", [([0, 1], 1, [0, 1]), ([0, 2, 0, 1], 2, [1, 0]),
                                            ([0, 2, 1, 1], 2, [0, 1]),
                                            ([1, 2, 3, 1, 2, 2, 3, 0, 0], 3, [1, 0, 2])])
def test_sort_by_keys(ctx, keys, width, perm):
    import torch
    from omega_h_gb300 import _lib
    k = _dev(keys, torch.int32)
    n = len(keys) // width
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    _lib.call("ohg_sort_by_keys", ctx.handle, _P(k), n, width, 4, _P(out))
    assert out.cpu().tolist() == perm


def test_offset_scan(ctx):
    import torch
    from omega_h_gb300 import _lib
    c = _dev([1, 1, 1], torch.int32)
    out = torch.empty(4, dtype=torch.int32, device="cuda")
    _lib.call("ohg_offset_scan", ctx.handle, _P(c), 3, _P(out))
    assert out.cpu().tolist() == [0, 1, 2, 3]


def _invert(ctx, hl2l, k, nlows, codes=None):
    import torch
    from omega_h_gb300 import _lib
    h = _dev(hl2l, torch.int32)
    c = _dev(codes, torch.int8) if codes is not None else None
    nh = len(hl2l) // k
    a2ab = torch.empty(nlows + 1, dtype=torch.int32, device="cuda")
    ab2b = torch.empty(max(len(hl2l), 1), dtype=torch.int32, device="cuda")
    cod = torch.empty(max(len(hl2l), 1), dtype=torch.int8, device="cuda")
    _lib.call("ohg_invert_adj", ctx.handle, _P(h), _P(c), nh, k, nlows, _P(a2ab), _P(ab2b),
              _P(cod))
    n = len(hl2l)
    return a2ab, ab2b[:n], cod[:n]


def test_invert_adj(ctx):
    a2ab, ab2b, cod = _invert(ctx, [0, 1, 2, 2, 3, 0], 3, 4)
    assert a2ab.cpu().tolist() == [0, 2, 3, 5, 6]
    assert ab2b.cpu().tolist() == [0, 1, 0, 0, 1, 1]
    assert cod.cpu().tolist() == [code(0, 0, 0), code(0, 0, 2), code(0, 0, 1), code(0, 0, 2),
                                  code(0, 0, 0), code(0, 0, 1)]


@pytest.mark.parametrize("hv2v,lv2v,nlows,hd,ld,want,want_codes", [
    ([0, 1, 2], [0, 1, 1, 2, 2, 0], 3, 2, 1, [0, 1, 2], [0, 0, 0]),
    ([0, 1, 2, 3], [0, 1, 1, 2, 2, 0, 0, 3, 1, 3, 2, 3], 6, 3, 1, [0, 1, 2, 3, 4, 5], [0] * 6),
    ([0, 1, 2, 3], [0, 2, 1, 0, 1, 3, 1, 2, 3, 2, 0, 3], 4, 3, 2, [0, 1, 2, 3], [0] * 4),
    ([0, 1, 2, 3], [0, 1, 2, 0, 3, 1, 1, 3, 2, 2, 3, 0], 4, 3, 2, [0, 1, 2, 3],
     [code(True, 0, 0)] * 4),
    ([0, 1, 2, 2, 3, 0], [0, 1, 1, 2, 2, 3, 3, 0, 0, 2], 5, 2, 1, [0, 1, 4, 2, 3, 4], None),
])
def test_reflect_down(ctx, hv2v, lv2v, nlows, hd, ld, want, want_codes):
    import torch
    from omega_h_gb300 import _lib
    nverts = max(hv2v) + 1
    a2ab, ab2b, cod = _invert(ctx, lv2v, ld + 1, nverts)
    h = _dev(hv2v, torch.int32)
    lv = _dev(lv2v, torch.int32)
    nh = len(hv2v) // (hd + 1)
    nuse = nh * math.comb(hd + 1, ld + 1)
    out = torch.empty(nuse, dtype=torch.int32, device="cuda")
    oc = torch.empty(nuse, dtype=torch.int8, device="cuda")
    _lib.call("ohg_reflect_down", ctx.handle, _P(h), nh, hd, ld, _P(lv), nlows, _P(a2ab),
              _P(ab2b), _P(cod), nverts, _P(out), _P(oc))
    assert out.cpu().tolist() == want
    if want_codes is not None:
        assert oc.cpu().tolist() == want_codes


def _mesh(ctx, dim, ev2v, nverts, coords=None, metric=None):
    import torch
    from omega_h_gb300.mesh import Mesh
    mc = 6 if dim == 3 else 3
    if coords is None:
        coords = np.arange(nverts * dim, dtype=np.float64)
    if metric is None:
        metric = np.tile(np.array([1.0] * dim + [0.0] * (mc - dim)), nverts)
    return Mesh.from_elems(ctx, dim, _dev(ev2v, torch.int32),
                           _dev(np.asarray(coords, dtype=np.float64).ravel(), torch.float64),
                           _dev(np.asarray(metric, dtype=np.float64).ravel(), torch.float64))


def test_find_unique_and_single_simplex_adjacency(ctx):
    m = _mesh(ctx, 2, [0, 1, 2, 2, 3, 0], 4)
    assert m.get("ev2v_1").cpu().tolist() == [0, 1, 0, 2, 3, 0, 1, 2, 2, 3]
    m.close()
    m = _mesh(ctx, 2, [0, 1, 2], 3)
    assert m.get("ev2v_2").cpu().tolist() == [0, 1, 2]
    assert m.get("down_2").cpu().tolist() == [0, 2, 1]
    assert m.get("ev2v_1").cpu().tolist() == [0, 1, 2, 0, 1, 2]
    m.close()
    m = _mesh(ctx, 3, [0, 1, 2, 3], 4)
    assert m.get("ev2v_3").cpu().tolist() == [0, 1, 2, 3]
    m.close()


def test_stars(ctx):
    m = _mesh(ctx, 2, [0, 1, 2], 3)
    assert m.get("star_a2ab_0").cpu().tolist() == [0, 2, 4, 6]
    assert m.get("star_ab2b_0").cpu().tolist() == [1, 2, 0, 2, 0, 1]
    assert m.get("star_a2ab_1").cpu().tolist() == [0, 2, 4, 6]
    assert m.get("star_ab2b_1").cpu().tolist() == [2, 1, 0, 2, 1, 0]
    m.close()
    m = _mesh(ctx, 3, [0, 1, 2, 3], 4)
    assert m.get("star_a2ab_0").cpu().tolist() == [0, 3, 6, 9, 12]
    assert m.get("star_ab2b_0").cpu().tolist() == [1, 2, 3, 0, 2, 3, 0, 1, 3, 0, 1, 2]
    assert m.get("star_a2ab_1").cpu().tolist() == list(range(0, 31, 5))
    assert m.get("star_ab2b_1").cpu().tolist() == [1, 3, 4, 2, 5, 3, 0, 2, 5, 4, 0, 4, 5, 1, 3,
                                                   0, 1, 5, 4, 2, 2, 0, 3, 5, 1, 1, 2, 4, 3, 0]
    m.close()


def test_dual(ctx):
    m = _mesh(ctx, 2, [0, 1, 2, 2, 3, 0], 4)
    assert m.get("dual_a2ab").cpu().tolist() == [0, 1, 2]
    assert m.get("dual_ab2b").cpu().tolist() == [1, 0]
    m.close()


S3 = math.sqrt(3.0)
R2 = 1.0 / math.sqrt(2.0)
TRI_OK = [[1, 0], [0, S3], [-1, 0]]
TET_OK = [[1, 0, -R2], [-1, 0, -R2], [0, -1, R2], [0, 1, R2]]


@pytest.mark.parametrize("dim,coords,metric,want", [
    (2, TRI_OK, None, 1.0),
    (3, TET_OK, None, 1.0),
    (2, [[1, 0], [0, 0], [-1, 0]], None, 0.0),
    (3, [[1, 0, 0], [-1, 0, 0], [0, -1, 0], [0, 1, 0]], None, 0.0),
    (2, [[1, 0], [-1, 0], [0, S3]], None, "negative"),
    (3, [[1, 0, -R2], [-1, 0, -R2], [0, 1, R2], [0, -1, R2]], None, "negative"),
    # a metric of lengths (1, 0.5) on the element squeezed by 0.5 in y
    (2, [[x, y / 2] for x, y in TRI_OK], [1.0, 4.0, 0.0], 1.0),
    (3, [[x, y, z / 2] for x, y, z in TET_OK], [1.0, 1.0, 4.0, 0.0, 0.0, 0.0], 1.0),
])
def test_element_quality(ctx, dim, coords, metric, want):
    nv = dim + 1
    met = None if metric is None else np.tile(np.array(metric), nv)
    m = _mesh(ctx, dim, list(range(nv)), nv, coords=coords, metric=met)
    q = float(m.get("quality").cpu()[0])
    m.close()
    if want == "negative":
        assert q < 0.0
    else:
        assert abs(q - want) <= 1e-10


def test_refine_qualities_unit_square(ctx):
    from omega_h_gb300.mesh import Mesh
    import torch
    m = Mesh.build_box(ctx, 2, 1)
    m.apply_workload(1, 1, 0)  # no interior vertex to jitter; allocates the metric
    m.set("metric", torch.tensor([1.0, 1.0, 0.0] * m.nents(0), dtype=torch.float64).cuda())
    c2e = torch.arange(m.nents(1), dtype=torch.int32, device="cuda")
    q = sorted(m.refine_qualities(c2e).cpu().tolist())
    want = sorted([0.494872, 0.494872, 0.866025, 0.494872, 0.494872])
    assert np.allclose(q, want, atol=1e-4)
    m.close()


# ---------------------------------------------------------------- Hilbert
def test_hilbert_skilling_7865(ctx):
    """Skilling's own example (src/unit_mesh.cpp:211-236): the point
    (5, 10, 20) of a 32^3 grid has Hilbert index 001111010111001 = 7865."""
    import torch
    from omega_h_gb300 import _lib
    axes = _dev([5, 10, 20], torch.int64)
    keys = torch.empty(3, dtype=torch.int64, device="cuda")
    _lib.call("ohg_hilbert_transpose", ctx.handle, _P(axes), 1, 3, 5, _P(keys))
    words = keys.cpu().tolist()
    bits = "".join(format(w, "05b") for w in words)
    assert bits == "001111010111001"
    assert int(bits, 2) == 7865


def test_hilbert_rejects_coordinates_wider_than_bits(ctx):
    import torch
    from omega_h_gb300 import _lib
    axes = _dev([32, 0, 0], torch.int64)
    keys = torch.empty(3, dtype=torch.int64, device="cuda")
    with pytest.raises(_lib.OhgError) as e:
        _lib.call("ohg_hilbert_transpose", ctx.handle, _P(axes), 1, 3, 5, _P(keys))
    assert e.value.code == 2  # OHG_ERR_BOUNDS


# ---------------------------------------------------------------- swap3d loop
# build_box_internal(1, 1, 1, 1, 1, 1) of the reference: make_3d_box's one hex
# (0, 1, 3, 2, 4, 5, 7, 6) split by tets_from_hexes (its minimum vertex is
# first and all three diagonals leave vertex 0, the six-tet case)
CUBE_TETS = [0, 3, 2, 7, 0, 2, 6, 7, 0, 6, 4, 7, 0, 5, 7, 4, 1, 5, 7, 0, 1, 7, 3, 0]
CUBE_COORDS = [[i % 2, (i // 2) % 2, i // 4] for i in range(8)]


def test_swap3d_loop(ctx):
    """swap3d::find_loop on edge 6 of the one-cube box (src/unit_mesh.cpp:424-447):
    edge vertices (7, 0), six tets, loop vertices 2, 3, 1, 5, 4, 6."""
    import torch
    from omega_h_gb300 import _lib
    m = _mesh(ctx, 3, CUBE_TETS, 8, coords=CUBE_COORDS)
    edges = _dev([6], torch.int32)
    sizes = torch.empty(1, dtype=torch.int32, device="cuda")
    eev = torch.empty(2, dtype=torch.int32, device="cuda")
    lv = torch.empty(7, dtype=torch.int32, device="cuda")
    _lib.call("ohg_swap3d_find_loops", m.handle, _P(edges), 1, _P(sizes), _P(eev), _P(lv))
    assert eev.cpu().tolist() == [7, 0]
    assert int(sizes.cpu()[0]) == 6
    assert lv.cpu().tolist()[:6] == [2, 3, 1, 5, 4, 6]
    m.close()


# ---------------------------------------------------------------- cubic, eigen
def _close(a, b, tol=1e-10, floor=1e-10):
    """are_close of the reference (src/Omega_h_scalar.hpp:266-277), elementwise."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    am, bm = np.abs(a), np.abs(b)
    d = np.where((am <= floor) & (bm <= floor), 0.0,
                 np.abs(b - a) / np.maximum(np.maximum(am, bm), 1e-300))
    return bool(np.all(d <= tol))


@pytest.mark.parametrize("coeffs,nroots,roots,mults", [
    ([0, 0, 0], 1, [0], [3]),
    ([1.0, -3.0 / 2.0, -3.0 / 2.0], 3, [2, -1, 0.5], [1, 1, 1]),
    ([2.0, -3.0, 0], 2, [-2, 1], [1, 2]),
    ([-8, -6, 3], 3, [2, -4, -1], [1, 1, 1]),
])
def test_cubic_roots(ctx, coeffs, nroots, roots, mults):
    """find_polynomial_roots known answers (src/unit_math.cpp:37-53), default eps 1e-6."""
    import torch
    from omega_h_gb300 import _lib
    c = _dev(coeffs, torch.float64)
    nr = torch.empty(1, dtype=torch.int32, device="cuda")
    rv = torch.empty(3, dtype=torch.float64, device="cuda")
    mu = torch.empty(3, dtype=torch.int32, device="cuda")
    _lib.call("ohg_cubic_roots", ctx.handle, 1, _P(c), 1e-6, _P(nr), _P(rv), _P(mu))
    assert int(nr.cpu()[0]) == nroots
    assert mu.cpu().tolist()[:nroots] == mults
    assert _close(rv.cpu().numpy()[:nroots], roots)


def _eigen(ctx, mats):
    """decompose_eigen through the C ABI; mats: (n, d, d) row-major arrays."""
    import torch
    from omega_h_gb300 import _lib
    mats = np.asarray(mats, dtype=np.float64)
    n, d = mats.shape[0], mats.shape[1]
    cols = np.ascontiguousarray(np.transpose(mats, (0, 2, 1)))  # column storage
    m = _dev(cols.ravel(), torch.float64)
    q = torch.empty(n * d * d, dtype=torch.float64, device="cuda")
    l = torch.empty(n * d, dtype=torch.float64, device="cuda")
    _lib.call("ohg_decompose_eigen", ctx.handle, d, n, _P(m), _P(q), _P(l))
    qs = np.transpose(q.cpu().numpy().reshape(n, d, d), (0, 2, 1))  # back to rows
    return qs, l.cpu().numpy().reshape(n, d)


def test_eigen_quadratic(ctx):
    """src/unit_math.cpp:107-115: identity, zero, and a non-symmetric 2x2 with
    its eigenvectors and eigenvalues."""
    q, l = _eigen(ctx, [np.eye(2), np.zeros((2, 2)),
                        [[8.67958, -14.0234], [-1.04985, 2.25873]]])
    assert _close(q[0], np.eye(2)) and _close(l[0], [1, 1])
    assert _close(q[1], np.eye(2)) and _close(l[1], [0, 0])
    want_q = [[9.9192948778227130e-01, 8.6289280817702185e-01],
              [-1.2679073810022995e-01, 5.0538698202107812e-01]]
    assert _close(q[2], want_q)
    assert _close(l[2], [1.0472083659357935e+01, 4.6622634064206342e-01])


def _rot3(angle, axis):
    """rotate(angle, axis) of the reference (src/Omega_h_matrix.hpp:531-535)."""
    a = np.asarray(axis, dtype=np.float64)
    cx = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return math.cos(angle) * np.eye(3) + math.sin(angle) * cx + \
        (1 - math.cos(angle)) * np.outer(a, a)


Q45 = _rot3(math.pi / 4, [0, 0, 1]) @ _rot3(math.pi / 4, [0, 1, 0])


def test_eigen_cubic(ctx):
    """src/unit_math.cpp:117-137: identity, zero, a non-symmetric matrix with
    eigenvalues (1, 2, 2), and metrics of lengths h rotated by Q45, including
    h with entries 1e3, 1e-3 and 1e-6 (eigenvalues 1/h^2 from 1e-6 to 1e12)."""
    hs = [[1e3, 1, 1], [1, 1e3, 1e3], [1e-3, 1, 1], [1, 1e-3, 1e-3], [1e-6, 1e-3, 1e-3]]
    metrics = [Q45 @ np.diag(1.0 / np.square(h)) @ Q45.T for h in hs]
    ns = np.array([[-1, 3, -1], [-3, 5, -1], [-3, 3, 1]], dtype=np.float64)
    q, l = _eigen(ctx, [np.eye(3), np.zeros((3, 3)), ns] + metrics)
    assert _close(q[0], np.eye(3)) and _close(l[0], [1, 1, 1])
    assert _close(q[1], np.eye(3)) and _close(l[1], [0, 0, 0])
    assert _close(l[2], [1, 2, 2], 1e-8, 1e-8)
    assert _close(ns, q[2] @ np.diag(l[2]) @ np.linalg.inv(q[2]))
    for k, h in enumerate(hs):
        qq, ll, a = q[3 + k], l[3 + k], metrics[k]
        assert _close(qq.T @ qq, np.eye(3), 1e-8, 1e-8)
        assert _close(ll, 1.0 / np.square(h), 1e-8, 1e-8)
        assert _close(a, qq @ np.diag(ll) @ qq.T, 1e-8, 1e-8)


# ---------------------------------------------------------------- intersection
def _pack(m):
    m = np.asarray(m, dtype=np.float64)
    if m.shape == (3, 3):
        return [m[0, 0], m[1, 1], m[2, 2], m[1, 0], m[2, 1], m[2, 0]]
    return [m[0, 0], m[1, 1], m[1, 0]]


def _unpack(v):
    if len(v) == 6:
        return np.array([[v[0], v[3], v[5]], [v[3], v[1], v[4]], [v[5], v[4], v[2]]])
    return np.array([[v[0], v[2]], [v[2], v[1]]])


def _intersect(ctx, pairs):
    import torch
    from omega_h_gb300 import _lib
    dim = np.asarray(pairs[0][0]).shape[0]
    a = _dev(np.concatenate([_pack(p[0]) for p in pairs]), torch.float64)
    b = _dev(np.concatenate([_pack(p[1]) for p in pairs]), torch.float64)
    mc = 6 if dim == 3 else 3
    out = torch.empty(len(pairs) * mc, dtype=torch.float64, device="cuda")
    _lib.call("ohg_intersect_metrics", ctx.handle, dim, len(pairs), _P(a), _P(b), _P(out))
    o = out.cpu().numpy().reshape(len(pairs), mc)
    return [_unpack(v) for v in o]


def _metric(q, h):
    return q @ np.diag(1.0 / np.square(np.asarray(h, dtype=np.float64))) @ q.T


def test_intersect_ortho_metrics(ctx):
    """src/unit_math.cpp:195-207, 254-262: metrics sharing the eigenvectors
    Q45; the intersection's lengths along them are the smaller ones (1e-3)."""
    cases = [([0.5, 1, 1], [1, 0.5, 1], [0.5, 0.5, 1]),
             ([1e-2, 1, 1], [1, 1, 1e-2], [1e-2, 1, 1e-2]),
             ([1e-2, 1e-2, 1], [1, 1, 1e-2], [1e-2, 1e-2, 1e-2]),
             ([1e-5, 1e-3, 1e-3], [1e-3, 1e-3, 1e-5], [1e-5, 1e-3, 1e-5])]
    got = _intersect(ctx, [(_metric(Q45, h1), _metric(Q45, h2)) for h1, h2, _ in cases])
    for mi, (_, _, want) in zip(got, cases):
        for i in range(3):
            d = Q45[:, i]
            assert _close(1.0 / math.sqrt(d @ mi @ d), want[i], 1e-3)


def test_intersect_subset_metrics(ctx):
    """src/unit_math.cpp:209-219: a 2D metric contained in the other is the
    intersection, in either order."""
    c, s = math.cos(math.pi / 4), math.sin(math.pi / 4)
    m1 = _metric(np.eye(2), [1, 2])
    m2 = _metric(np.array([[c, -s], [s, c]]), [2, 3])
    got = _intersect(ctx, [(m2, m1), (m1, m2)])
    assert _close(got[0], m1) and _close(got[1], m1)


def test_intersect_degenerate_metrics(ctx):
    """Barral's degenerate cases (src/unit_math.cpp:221-252): with the null
    metric, and cases 2.a, 2.b, 3.a, 3.b, 4.a and 4.b on diagonal metrics."""
    d = np.diag
    m1 = _metric(Q45, [1, 1, 1e-3])
    z = np.zeros((3, 3))
    pairs = [(m1, z), (z, m1),
             (d([1, 0, 0]), d([0, 0, 1])), (d([1, 0, 0]), d([2, 0, 0])),
             (d([1, 0, 0]), d([2, 1, 0])), (d([1, 0, 0]), d([0, 1, 2])),
             (d([1, 0, 2]), d([2, 0, 1])), (d([1, 0, 2]), d([2, 1, 0]))]
    want = [m1, m1, d([1, 0, 1]), d([2, 0, 0]), d([2, 1, 0]), d([1, 1, 2]), d([2, 0, 2]),
            d([2, 1, 2])]
    got = _intersect(ctx, pairs)
    for k, (g, w) in enumerate(zip(got, want)):
        assert _close(g, w), (k, g, w)

