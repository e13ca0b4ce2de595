"""ohg_offset_scan_noalloc (fixed device scratch, no allocation) against the
allocating ohg_offset_scan, both called through the C ABI.

Collected last on purpose: the fixed scratch is shared per device, so this
file also shows that calls made after every other test still agree."""
import ctypes

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


def _limit():
    from omega_h_gb300 import _lib
    v = ctypes.c_int()
    _lib.call("ohg_offset_scan_noalloc_limit", ctypes.byref(v))
    return v.value


def _scan(ctx, name, counts):
    import torch
    from omega_h_gb300 import _lib
    out = torch.full((counts.numel() + 1,), -7, dtype=torch.int32, device=counts.device)
    _lib.call(name, ctx.handle, ctypes.c_void_p(counts.data_ptr()), counts.numel(),
              ctypes.c_void_p(out.data_ptr()))
    torch.cuda.synchronize()
    return out


def _counts(n, seed, hi=5):
    import torch
    g = torch.Generator().manual_seed(seed)
    return torch.randint(0, hi, (n,), generator=g, dtype=torch.int32).cuda()


@pytest.mark.parametrize("n", [0, 1, 4095, 4096, 4097, 1_000_003, "limit"])
def test_noalloc_scan_matches_allocating_scan_twice_in_a_row(ctx, n):
    import torch
    if n == "limit":
        n = _limit()
    # two calls in a row on different inputs: nothing left in the shared
    # scratch by the first call may change the second
    for seed in (n, n + 1):
        counts = _counts(n, seed)
        want = _scan(ctx, "ohg_offset_scan", counts)
        got = _scan(ctx, "ohg_offset_scan_noalloc", counts)
        assert torch.equal(got, want)
        c64 = counts.to(torch.int64)
        assert int(got[-1]) == int(c64.sum())
        if n:
            assert torch.equal(got[1:].to(torch.int64), torch.cumsum(c64, 0))


def test_noalloc_scan_allocates_nothing(ctx):
    """The property the entry point exists for: after its first call on the
    device (which looks up the scratch address), further calls make no
    device allocation through the library, while the allocating scan does."""
    counts = _counts(1_000_003, 11)
    _scan(ctx, "ohg_offset_scan_noalloc", counts)
    before = ctx.allocations()
    for _ in range(3):
        _scan(ctx, "ohg_offset_scan_noalloc", counts)
    assert ctx.allocations() == before
    _scan(ctx, "ohg_offset_scan", counts)
    assert ctx.allocations() > before


def test_noalloc_scan_rejects_sizes_beyond_its_scratch(ctx):
    from omega_h_gb300 import _lib
    lim = _limit()
    assert lim == 4096 * 1024
    counts = _counts(lim + 1, 3)
    with pytest.raises(_lib.OhgError) as e:
        _scan(ctx, "ohg_offset_scan_noalloc", counts)
    assert e.value.args and "exceed the fixed scratch limit" in str(e.value)
    # the context stays usable after the rejection
    small = _counts(10, 4)
    import torch
    assert torch.equal(_scan(ctx, "ohg_offset_scan_noalloc", small),
                       _scan(ctx, "ohg_offset_scan", small))
