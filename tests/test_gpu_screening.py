"""Precision mode: the FP32 enclosures contain the FP64 values, and an adapt
pass with screening gives bit for bit the arrays of the FP64-throughout pass
(decisions, connectivity and every real)."""
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


def _mesh(ctx, n, kind, seed, dim=3):
    from omega_h_gb300.mesh import Mesh
    m = Mesh.build_box(ctx, dim, n)
    m.apply_workload(n, seed, kind)
    return m


def _screen(m, name, verts, k):
    import torch
    from omega_h_gb300 import _lib
    n = verts.numel() // k
    lo = torch.empty(n, dtype=torch.float32, device=verts.device)
    hi = torch.empty_like(lo)
    ex = torch.empty(n, dtype=torch.float64, device=verts.device)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    _lib.call(name, m.handle, P(verts), n, P(lo), P(hi), P(ex))
    torch.cuda.synchronize()
    return lo.cpu().numpy().astype(np.float64), hi.cpu().numpy().astype(np.float64), \
        ex.cpu().numpy()


def _check_enclosure(lo, hi, ex, what):
    bad = ~((lo <= ex) & (ex <= hi))
    assert not bad.any(), f"{what}: {int(bad.sum())} FP64 values outside their enclosure, " \
                          f"first {np.nonzero(bad)[0][:5]}"
    fin = np.isfinite(lo) & np.isfinite(hi) & (np.abs(ex) > 0)
    w = (hi[fin] - lo[fin]) / np.abs(ex[fin])
    print(f"{what}: {ex.size} values, {int((~fin).sum())} unbounded, relative width "
          f"median {np.median(w):.2e} max {w.max():.2e}")


# kinds 10 and 13: isotropic metrics stored as one scalar per vertex
@pytest.mark.parametrize("n,kind,seed", [(12, 0, 1), (16, 1, 7), (16, 2, 3), (24, 1, 2024),
                                         (16, 10, 3), (16, 13, 4)])
def test_enclosures_contain_the_fp64_values(ctx, n, kind, seed):
    import torch
    m = _mesh(ctx, n, kind, seed)
    tv = m.get("ev2v_3").view(-1, 4)
    nt = tv.shape[0]
    # the mesh's own tets, mirrored ones (negative size), and tets with one
    # vertex taken from the next tet in Hilbert order (arbitrary shapes,
    # slivers and inversions included)
    mirrored = tv[:, [1, 0, 2, 3]]
    mixed = tv.clone()
    g = torch.Generator().manual_seed(seed)
    col = torch.randint(0, 4, (nt,), generator=g).cuda()
    rows = torch.arange(nt, device=tv.device)
    mixed[rows, col] = tv[(rows + 1) % nt, col]
    tets = torch.cat([tv, mirrored, mixed]).contiguous()
    lo, hi, ex = _screen(m, "ohg_screen_tet_qualities", tets, 4)
    q = m.get("quality").cpu().numpy()
    assert np.array_equal(ex[:nt], q), "exact tet quality differs from measure_qualities"
    _check_enclosure(lo, hi, ex, "tet qualities")
    assert (ex[nt:2 * nt] < 0).all()

    ev = m.get("ev2v_1").view(-1, 2)
    ne = ev.shape[0]
    nv = m.nents(0)
    far = torch.stack([ev[:, 0], (ev[:, 1] + 17) % nv], 1)
    edges = torch.cat([ev, far]).contiguous()
    lo, hi, ex = _screen(m, "ohg_screen_edge_lengths", edges, 2)
    ln = m.get("length").cpu().numpy()
    assert np.array_equal(ex[:ne], ln), "exact length differs from measure_edges_metric"
    _check_enclosure(lo, hi, ex, "edge lengths")
    m.close()


@pytest.mark.parametrize("n,kind,seed", [(12, 0, 1), (16, 1, 7), (16, 2, 3), (16, 13, 4)])
def test_face_route_enclosures_contain_the_fp64_values(ctx, n, kind, seed):
    """The collapse screen's route: invariants of the face opposite one slot,
    then the vertex at that slot, for every slot, on the mesh's tets, their
    mirror images and tets with one vertex moved to a far vertex (arbitrary
    shapes, slivers, inversions).  The intervals must hold the FP64 value as
    the reference evaluates it, in its slot order."""
    import torch
    from omega_h_gb300 import _lib
    m = _mesh(ctx, n, kind, seed)
    tv = m.get("ev2v_3").view(-1, 4)
    nt = tv.shape[0]
    nv = m.nents(0)
    g = torch.Generator().manual_seed(seed)
    col = torch.randint(0, 4, (nt,), generator=g).cuda()
    rows = torch.arange(nt, device=tv.device)
    mixed = tv.clone()
    far = torch.randint(0, nv - 1, (nt,), generator=g).cuda()
    mixed[rows, col] = ((tv[rows, col].long() + 1 + far) % nv).to(tv.dtype)
    tets = torch.cat([tv, tv[:, [1, 0, 2, 3]], mixed]).contiguous()
    lo0, hi0, ex0 = _screen(m, "ohg_screen_tet_qualities", tets, 4)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    nn = tets.shape[0]
    def face(slot, cubed):
        lo = torch.empty(nn, dtype=torch.float32, device="cuda")
        hi = torch.empty_like(lo)
        ex = torch.empty(nn, dtype=torch.float64, device="cuda")
        _lib.call("ohg_screen_tet_qualities_face", m.handle, P(tets), nn, slot, int(cubed),
                  P(lo), P(hi), P(ex))
        torch.cuda.synchronize()
        return (lo.cpu().numpy().astype(np.float64), hi.cpu().numpy().astype(np.float64),
                ex.cpu().numpy())

    for slot in range(4):
        lo, hi, ex = face(slot, False)
        assert np.array_equal(ex, ex0)
        _check_enclosure(lo, hi, ex, f"tet qualities, face route, slot {slot}")
        # no wider than a few times the direct route's interval
        fin = np.isfinite(lo) & np.isfinite(hi) & np.isfinite(lo0) & np.isfinite(hi0) & (ex > 0)
        r = (hi[fin] - lo[fin]) / np.maximum(hi0[fin] - lo0[fin], 1e-300)
        assert np.median(r) < 2.0
        # the cube of the quality, as the 3D collapse screen takes it: the
        # double cube of ex is within 2.1 u_double of the exact one
        lo3, hi3, _ = face(slot, True)
        c = ex ** 3
        bad = ~((lo3 <= c * (1 + 4.7e-16 * np.sign(c))) & (c * (1 - 4.7e-16 * np.sign(c)) <= hi3))
        assert not bad.any(), f"slot {slot}: {int(bad.sum())} cubes outside their interval"
        # a settled negative size gives [-inf, 0], an unsettled sign or an
        # unbounded case [-inf, inf]; a positive quality's cube is >= 0
        neg, pos = ex < 0, ex > 0
        assert ((hi3[neg] <= 0) | ~np.isfinite(hi3[neg])).all()
        assert ((lo3[pos] >= 0) | ~np.isfinite(lo3[pos])).all()
    m.close()


@pytest.mark.parametrize("n,kind,seed", [(32, 0, 1), (48, 1, 7), (40, 2, 3), (64, 3, 5),
                                         (48, 13, 6)])
def test_2d_enclosures_contain_the_fp64_values(ctx, n, kind, seed):
    import torch
    m = _mesh(ctx, n, kind, seed, dim=2)
    tv = m.get("ev2v_2").view(-1, 3)
    nt = tv.shape[0]
    mirrored = tv[:, [1, 0, 2]]
    mixed = tv.clone()
    g = torch.Generator().manual_seed(seed)
    col = torch.randint(0, 3, (nt,), generator=g).cuda()
    rows = torch.arange(nt, device=tv.device)
    mixed[rows, col] = tv[(rows + 1) % nt, col]
    tris = torch.cat([tv, mirrored, mixed]).contiguous()
    lo, hi, ex = _screen(m, "ohg_screen_tet_qualities", tris, 3)
    assert np.array_equal(ex[:nt], m.get("quality").cpu().numpy())
    _check_enclosure(lo, hi, ex, "2D triangle qualities")
    ev = m.get("ev2v_1").view(-1, 2)
    nv = m.nents(0)
    far = torch.stack([ev[:, 0], (ev[:, 1] + 17) % nv], 1)
    edges = torch.cat([ev, far]).contiguous()
    lo, hi, ex = _screen(m, "ohg_screen_edge_lengths", edges, 2)
    assert np.array_equal(ex[:ev.shape[0]], m.get("length").cpu().numpy())
    _check_enclosure(lo, hi, ex, "2D edge lengths")
    m.close()


PASS_ARRAYS = ["coords", "metric", "length", "quality"] + \
    [f"ev2v_{d}" for d in (1, 2, 3)] + [f"down_{d}" for d in (1, 2, 3)] + \
    [f"downcodes_{d}" for d in (2, 3)] + [f"class_dim_{d}" for d in range(4)] + \
    [f"class_id_{d}" for d in range(4)]


def _pass_arrays(ctx, n, kind, seed, mqa, screening, dim=3):
    from omega_h_gb300.mesh import adapt_opts
    ctx.set_screening(screening)
    try:
        m = _mesh(ctx, n, kind, seed, dim=dim)
        st = m.adapt_pass(adapt_opts(dim, min_quality_allowed=mqa))
        names = PASS_ARRAYS if dim == 3 else [k for k in PASS_ARRAYS if not k.endswith("_3")]
        out = {k: m.get(k).cpu().numpy() for k in names}
        m.close()
    finally:
        ctx.set_screening(True)
    return st, out


@pytest.mark.parametrize("dim,n,kind,seed,mqa", [(3, 8, 0, 12345, 0.3), (3, 12, 1, 7, 0.2),
                                                 (3, 12, 2, 3, 0.2), (3, 20, 1, 11, 0.2),
                                                 (3, 16, 0, 5, 0.3), (3, 32, 1, 2024, 0.2),
                                                 (3, 10, 3, 5, 0.2), (2, 64, 1, 3, 0.3),
                                                 (2, 96, 2, 4, 0.3), (2, 80, 3, 5, 0.3),
                                                 (3, 16, 13, 8, 0.2), (3, 12, 10, 2, 0.3),
                                                 (2, 80, 13, 9, 0.3)])
def test_screened_pass_equals_fp64_pass_bit_for_bit(ctx, dim, n, kind, seed, mqa):
    ctx.screen_counts(reset=True)
    st1, a1 = _pass_arrays(ctx, n, kind, seed, mqa, True, dim)
    counts = ctx.screen_counts(reset=True)
    st0, a0 = _pass_arrays(ctx, n, kind, seed, mqa, False, dim)
    # (indset_rounds is left out: the independent-set rounds update their
    # states in place, so their count depends on the launch schedule)
    for k in ("did_refine", "did_coarsen", "did_swap", "nelems_out", "refine_keys",
              "coarsen_keys", "swap_keys"):
        assert st1[k] == st0[k], k
    for k in a0:
        assert a1[k].shape == a0[k].shape, k
        assert np.array_equal(a1[k].view(np.uint8), a0[k].view(np.uint8)), f"{k} differs"
    tets, tets_fp64, lens, lens_fp64 = counts
    print(f"box{n} kind {kind}: tets screened {tets}, recomputed {tets_fp64} "
          f"({tets_fp64 / max(tets, 1):.3%}); lengths screened {lens}, recomputed "
          f"{lens_fp64} ({lens_fp64 / max(lens, 1):.3%})")
