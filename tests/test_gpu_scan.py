"""The single-pass offset scan and the marked-index compaction, through the
C ABI, against torch's cumsum and nonzero: sizes from one tile to thousands
of tiles (the look-back then crosses many 32-tile windows), aligned and
unaligned pointers (the scalar load and store path), and mark densities
from none to all.  offset_scan follows src/Omega_h_int_scan.cpp:10-20 and
collect_marked src/Omega_h_map.cpp:174-185."""
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


def _P(t):
    return ctypes.c_void_p(t.data_ptr())


def _scan(ctx, counts, out):
    import torch
    from omega_h_gb300 import _lib
    _lib.call("ohg_offset_scan", ctx.handle, _P(counts), counts.numel(), _P(out))
    torch.cuda.synchronize()


@pytest.mark.parametrize("n", [4097, 65_536, 1_000_001, 8_392_705, 20_000_003])
@pytest.mark.parametrize("offset", [0, 1])
def test_offset_scan_matches_cumsum(ctx, n, offset):
    """offset 1 starts both the counts and the output one int past a
    16-byte boundary; 8,392,705 counts are 2,050 tiles of 4,096."""
    import torch
    g = torch.Generator().manual_seed(n + offset)
    buf = torch.randint(0, 9, (n + offset,), generator=g, dtype=torch.int32).cuda()
    counts = buf[offset:]
    obuf = torch.full((n + 1 + offset,), -7, dtype=torch.int32, device="cuda")
    out = obuf[offset:]
    _scan(ctx, counts, out)
    want = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    want[1:] = torch.cumsum(counts.to(torch.int64), 0)
    assert torch.equal(out.to(torch.int64), want)
    if offset:
        assert int(obuf[0]) == -7


def _collect(ctx, marks):
    import torch
    from omega_h_gb300 import _lib
    n = marks.numel()
    out = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    cnt = ctypes.c_int(-1)
    _lib.call("ohg_collect_marked", ctx.handle, _P(marks) if n else None, n, _P(out),
              ctypes.byref(cnt))
    torch.cuda.synchronize()
    return out[:cnt.value], cnt.value


@pytest.mark.parametrize("n", [0, 1, 4095, 4096, 4097, 3_000_017, 12_000_000])
@pytest.mark.parametrize("density", [0.0, 0.001, 0.5, 1.0])
def test_collect_marked_matches_nonzero(ctx, n, density):
    import torch
    g = torch.Generator().manual_seed(n * 7 + int(density * 1000))
    marks = (torch.rand(n, generator=g) < density).to(torch.int8)
    # marks of other nonzero values count as marked
    marks[::5] *= 3
    marks = marks.cuda()
    got, cnt = _collect(ctx, marks)
    want = torch.nonzero(marks, as_tuple=False).flatten().to(torch.int32)
    assert cnt == want.numel()
    assert torch.equal(got, want)


def test_collect_marked_from_an_unaligned_start(ctx):
    import torch
    g = torch.Generator().manual_seed(11)
    buf = (torch.rand(1_000_003, generator=g) < 0.3).to(torch.int8).cuda()
    for off in (1, 3, 8):
        marks = buf[off:]
        got, cnt = _collect(ctx, marks)
        want = torch.nonzero(marks, as_tuple=False).flatten().to(torch.int32)
        assert cnt == want.numel() and torch.equal(got, want)


def test_scan_wait_limit_reports_a_timeout_and_the_context_stays_usable(ctx):
    """The look-back's waits are bounded: with the first tile withheld (a
    status word nothing will set) the other tiles give up after their poll
    limit, the call returns OHG_ERR_TIMEOUT, and the next scan is correct."""
    import torch
    from omega_h_gb300 import _lib
    n = 3 * 4096
    counts = torch.ones(n, dtype=torch.int32, device="cuda")
    out = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    with pytest.raises(_lib.OhgError) as e:
        _lib.call("ohg_selftest_scan_wait_limit", ctx.handle, _P(counts), n, _P(out))
    assert e.value.code == 5  # OHG_ERR_TIMEOUT
    _scan(ctx, counts, out)
    assert torch.equal(out.cpu(), torch.arange(n + 1, dtype=torch.int32))
