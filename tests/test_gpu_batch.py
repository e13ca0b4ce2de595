"""Batched passes: one adapt pass over the disjoint union of many meshes
gives, mesh by mesh, bit for bit the arrays of separate passes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ARRAYS = {3: ["coords", "metric", "length", "quality", "ev2v_1", "ev2v_2", "ev2v_3", "down_1",
              "down_2", "down_3", "downcodes_2", "downcodes_3"],
          2: ["coords", "metric", "length", "quality", "ev2v_1", "ev2v_2", "down_1", "down_2",
              "downcodes_2"]}


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


def _make(ctx, dim, n, kind, seed):
    from omega_h_gb300.mesh import Mesh
    m = Mesh.build_box(ctx, dim, n)
    m.apply_workload(n, seed, kind)
    return m


def _arrays(m):
    d = m.dim
    names = ARRAYS[d] + [f"class_dim_{i}" for i in range(d + 1)] + \
        [f"class_id_{i}" for i in range(d + 1)]
    return {k: m.get(k).cpu().numpy() for k in names}


def _same(a, b, what):
    for k in a:
        assert a[k].shape == b[k].shape, f"{what}: {k} shape"
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), f"{what}: {k} differs"


SPECS3 = [(3, 4, 0, 1), (3, 9, 1, 2), (3, 6, 3, 3), (3, 12, 2, 4), (3, 5, 3, 5), (3, 8, 1, 6)]
SPECS2 = [(2, 16, 1, 1), (2, 40, 3, 2), (2, 24, 2, 3), (2, 9, 0, 4)]


@pytest.mark.parametrize("specs", [SPECS3, SPECS2], ids=["3d", "2d"])
def test_batch_pass_equals_separate_passes(ctx, specs):
    from omega_h_gb300.mesh import adapt_opts, adapt_pass_batch
    dim = specs[0][0]
    o = adapt_opts(dim)
    solo = []
    for s in specs:
        m = _make(ctx, *s)
        m.adapt_pass(o)
        m.adapt_pass(o)
        solo.append(_arrays(m))
        m.close()
    ms = [_make(ctx, *s) for s in specs]
    adapt_pass_batch(ctx, ms, o)
    adapt_pass_batch(ctx, ms, o)
    for s, m, want in zip(specs, ms, solo):
        _same(want, _arrays(m), f"mesh {s}")
        m.close()


def test_concat_then_split_round_trips(ctx):
    from omega_h_gb300.mesh import concat, split
    ms = [_make(ctx, *s) for s in SPECS3[:4]]
    before = [_arrays(m) for m in ms]
    u = concat(ctx, ms)
    parts = split(u, len(ms))
    u.close()
    for b, p in zip(before, parts):
        _same(b, _arrays(p), "round trip")
        p.close()
    for m in ms:
        m.close()


def test_concat_rejects_mixed_dimensions(ctx):
    from omega_h_gb300 import _lib
    from omega_h_gb300.mesh import concat
    a, b = _make(ctx, 3, 4, 0, 1), _make(ctx, 2, 8, 0, 1)
    with pytest.raises(_lib.OhgError):
        concat(ctx, [a, b])
    a.close()
    b.close()
