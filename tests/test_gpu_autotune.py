"""The launch-shape autotuner: every variant of every tuned launch site gives
bit for bit the same adapt pass, and exploration settles on choices that
frozen mode then keeps (no counterpart in the reference)."""
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


def _pass(ctx, n=24, kind=1, seed=5):
    import gpu_dump
    from omega_h_gb300.mesh import Mesh, adapt_opts
    m = Mesh.build_box(ctx, 3, n)
    m.apply_workload(n, seed, kind)
    st = m.adapt_pass(adapt_opts(3, min_quality_allowed=0.2))
    out = {}
    gpu_dump.dump_mesh(m, "out_", out, with_length=True, with_quality=True)
    m.close()
    return st, out


def _counts(st):
    """the pass statistics that do not depend on timing or on the launch
    schedule (the independent-set rounds update their states in place, so
    their count may vary; the set does not)"""
    return {k: v for k, v in st.items() if not k.startswith("ms_") and k != "indset_rounds"}


def _same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        assert x.shape == y.shape and np.array_equal(x.view(np.uint8), y.view(np.uint8)), k


def test_every_variant_gives_the_same_pass(ctx):
    ctx.autotune("off")
    try:
        st0, ref = _pass(ctx)
        assert st0["did_coarsen"]
        for v in range(4):
            ctx.force_variant(v)
            st, out = _pass(ctx)
            assert _counts(st) == _counts(st0)
            _same(ref, out)
    finally:
        ctx.force_variant(None)
        ctx.autotune("frozen")


def test_exploration_then_frozen(ctx):
    ctx.autotune("off")
    _, ref = _pass(ctx)
    ctx.autotune("explore")
    for _ in range(5):
        _pass(ctx)
    ctx.autotune("frozen")
    seen, chosen, moved = ctx.tuning()
    print(f"tuned sites: {seen} seen, {chosen} chosen, {moved} not the default")
    assert seen > 10 and chosen > 0 and chosen <= seen and moved <= chosen
    _, out = _pass(ctx)
    _same(ref, out)
