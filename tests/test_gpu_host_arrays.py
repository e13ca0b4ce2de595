"""The C ABI's host-memory paths: ohg_mesh_from_arrays reading pinned and
pageable host arrays gives the mesh that device arrays give (the same pass
result, bit for bit), and ohg_mesh_get_arrays returns what one
ohg_mesh_get_array call per array returns, checking every name and
capacity before it copies anything."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = ["down_1", "down_2", "downcodes_2", "down_3", "downcodes_3", "coords", "metric"] + \
        [f"class_dim_{d}" for d in range(4)] + [f"class_id_{d}" for d in range(4)]


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


def _from_arrays(ctx, arrs, nents):
    from omega_h_gb300 import _lib
    from omega_h_gb300.mesh import Mesh
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    n4 = (ctypes.c_int * 4)(*nents)
    down = (ctypes.c_void_p * 4)(None, P(arrs["down_1"]), P(arrs["down_2"]), P(arrs["down_3"]))
    codes = (ctypes.c_void_p * 4)(None, None, P(arrs["downcodes_2"]), P(arrs["downcodes_3"]))
    cdim = (ctypes.c_void_p * 4)(*[P(arrs[f"class_dim_{d}"]) for d in range(4)])
    cid = (ctypes.c_void_p * 4)(*[P(arrs[f"class_id_{d}"]) for d in range(4)])
    h = ctypes.c_void_p()
    _lib.call("ohg_mesh_from_arrays", ctx.handle, 3, n4, down, codes, cdim, cid,
              P(arrs["coords"]), P(arrs["metric"]), ctypes.byref(h))
    return Mesh(ctx, h)


def _get_all(m):
    import torch
    from omega_h_gb300 import _lib
    bufs, caps, dsts = [], (ctypes.c_longlong * len(NAMES))(), (ctypes.c_void_p * len(NAMES))()
    for i, k in enumerate(NAMES):
        nb = ctypes.c_longlong()
        _lib.call("ohg_mesh_array_bytes", m.handle, k.encode(), ctypes.byref(nb))
        b = torch.full((nb.value,), 0xAB, dtype=torch.uint8).pin_memory()
        bufs.append(b)
        caps[i] = nb.value
        dsts[i] = b.data_ptr()
    names = (ctypes.c_char_p * len(NAMES))(*[k.encode() for k in NAMES])
    _lib.call("ohg_mesh_get_arrays", m.handle, len(NAMES), names, dsts, caps)
    return {k: b.numpy().copy() for k, b in zip(NAMES, bufs)}


def test_mesh_from_host_arrays_equals_mesh_from_device_arrays(ctx):
    from omega_h_gb300.mesh import Mesh, adapt_opts
    base = Mesh.build_box(ctx, 3, 10)
    base.apply_workload(10, 7, 1)
    nents = [base.nents(d) for d in range(4)]
    dev = {k: base.get(k) for k in NAMES}
    results = []
    for kind in ("device", "pinned", "pageable"):
        if kind == "device":
            arrs = dev
        elif kind == "pinned":
            arrs = {k: v.cpu().pin_memory() for k, v in dev.items()}
        else:
            arrs = {k: v.cpu() for k, v in dev.items()}
        m = _from_arrays(ctx, arrs, nents)
        st = m.adapt_pass(adapt_opts(3, min_quality_allowed=0.2))
        results.append((st, _get_all(m)))
        m.close()
    base.close()
    (s0, a0) = results[0]
    # timings and the schedule-dependent independent-set round count aside
    counts = lambda st: {k: v for k, v in st.items()  # noqa: E731
                         if not k.startswith("ms_") and k != "indset_rounds"}
    for st, a in results[1:]:
        assert counts(st) == counts(s0)
        for k in NAMES:
            assert np.array_equal(a[k], a0[k]), k


def test_get_arrays_equals_get_array_and_checks_first(ctx):
    import torch
    from omega_h_gb300 import _lib
    from omega_h_gb300.mesh import Mesh
    m = Mesh.build_box(ctx, 3, 6)
    m.apply_workload(6, 3, 3)
    got = _get_all(m)
    for k in NAMES:
        one = m.get(k).cpu()
        assert np.array_equal(got[k], one.view(torch.uint8).numpy()), k
    # an unknown name or a short destination fails before any copy
    b = torch.full((16,), 7, dtype=torch.uint8).pin_memory()
    names = (ctypes.c_char_p * 2)(b"coords", b"no_such_array")
    big = torch.zeros(m.nents(0) * 3 * 8, dtype=torch.uint8).pin_memory()
    dsts = (ctypes.c_void_p * 2)(big.data_ptr(), b.data_ptr())
    caps = (ctypes.c_longlong * 2)(big.numel(), 16)
    with pytest.raises(_lib.OhgError):
        _lib.call("ohg_mesh_get_arrays", m.handle, 2, names, dsts, caps)
    assert int(big.sum()) == 0
    names = (ctypes.c_char_p * 2)(b"coords", b"metric")
    caps = (ctypes.c_longlong * 2)(big.numel(), 16)
    with pytest.raises(_lib.OhgError):
        _lib.call("ohg_mesh_get_arrays", m.handle, 2, names, dsts, caps)
    assert int(big.sum()) == 0 and int(b.sum()) == 16 * 7
    m.close()
