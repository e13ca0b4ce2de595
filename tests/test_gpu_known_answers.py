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
