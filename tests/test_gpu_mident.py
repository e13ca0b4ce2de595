"""Midpoint metrics of edges (get_mident_metrics, src/Omega_h_metric.cpp:
56-104) by the two routes of the library: for many edges each vertex's log
metric is made once and every edge does one eigendecomposition; for few
edges every edge does all three.  The log metric is a function of the
vertex's metric alone, so both routes must give the same doubles."""
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


@pytest.mark.parametrize("n,kind,seed", [(10, 0, 1), (12, 1, 7), (12, 2, 3), (10, 3, 5)])
def test_mident_routes_agree_bit_for_bit(ctx, n, kind, seed):
    import torch
    from omega_h_gb300.mesh import Mesh
    m = Mesh.build_box(ctx, 3, n)
    m.apply_workload(n, seed, kind)
    ne, nv = m.nents(1), m.nents(0)
    every = torch.arange(ne, dtype=torch.int32, device="cuda")
    full = m.mident_metrics(every).view(ne, -1).cpu().numpy()
    rng = np.random.default_rng(seed)
    few = np.sort(rng.choice(ne, size=max(1, nv // 4), replace=False)).astype(np.int32)
    part = m.mident_metrics(torch.from_numpy(few).cuda()).view(len(few), -1).cpu().numpy()
    assert 2 * ne >= nv and 2 * len(few) < nv
    assert np.array_equal(part.view(np.uint64), full[few].view(np.uint64))
    m.close()
