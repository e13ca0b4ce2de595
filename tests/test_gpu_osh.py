"""The device-resident .osh reader and writer against files the reference
itself wrote (tests/golden/osh, made by tests/golden/make_golden.py):
read-then-write gives the same bytes, the box built here and written gives
the reference's file byte for byte, and after one adapt pass (from the box
or from the reference's file) the written mesh equals the reference's:
metadata, connectivity, tag names, order and integers exactly, reals within
1e-12 (the reference's own parity bound)."""
import filecmp
import json
import os

import numpy as np
import pytest

import osh_format as osh

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
OSH = os.path.join(HERE, "golden", "osh")
CASES = sorted(os.listdir(OSH))


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


def _case(case):
    with open(os.path.join(OSH, case, "case.json")) as f:
        return json.load(f)


def _same_files(a, b):
    for f in ("0.osh", "nparts", "version"):
        assert filecmp.cmp(os.path.join(a, f), os.path.join(b, f), shallow=False), f


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("part", ["in.osh", "out.osh"])
def test_read_then_write_is_byte_identical(ctx, tmp_path, case, part):
    from omega_h_gb300.mesh import Mesh
    m = Mesh.read_osh(ctx, os.path.join(OSH, case, part))
    m.write_osh(tmp_path / "w.osh")
    m.close()
    _same_files(os.path.join(OSH, case, part), str(tmp_path / "w.osh"))


@pytest.mark.parametrize("case", CASES)
def test_built_box_is_the_reference_file(ctx, tmp_path, case):
    from omega_h_gb300.mesh import Mesh
    c = _case(case)
    m = Mesh.build_box(ctx, c["dim"], c["n"])
    m.apply_workload(c["n"], c["seed"], c["metric"])
    m.write_osh(tmp_path / "in.osh")
    m.close()
    _same_files(os.path.join(OSH, case, "in.osh"), str(tmp_path / "in.osh"))


@pytest.mark.parametrize("start", ["box", "file"])
@pytest.mark.parametrize("case", CASES)
def test_pass_then_write_matches_the_reference(ctx, tmp_path, case, start):
    from omega_h_gb300.mesh import Mesh, adapt_opts
    c = _case(case)
    if start == "box":
        m = Mesh.build_box(ctx, c["dim"], c["n"])
        m.apply_workload(c["n"], c["seed"], c["metric"])
    else:
        m = Mesh.read_osh(ctx, os.path.join(OSH, case, "in.osh"))
    m.adapt_pass(adapt_opts(c["dim"], min_quality_allowed=c["min_quality_allowed"]))
    m.write_osh(tmp_path / "out.osh")
    m.close()
    got = osh.read(str(tmp_path / "out.osh"))
    want = osh.read(os.path.join(OSH, case, "out.osh"))
    bad = osh.compare(want, got)
    assert not bad, bad


def test_compressed_write_reads_back(ctx, tmp_path):
    from omega_h_gb300 import _lib
    import ctypes
    z = ctypes.c_int()
    _lib.call("ohg_osh_zlib", ctypes.byref(z))
    if not z.value:
        pytest.skip("no zlib on this system")
    from omega_h_gb300.mesh import Mesh
    src = os.path.join(OSH, CASES[0], "out.osh")
    m = Mesh.read_osh(ctx, src)
    m.write_osh(tmp_path / "z.osh", compress=True)
    m.close()
    zm = osh.read(str(tmp_path / "z.osh"))
    assert zm["compressed"] == 1
    assert not osh.compare(osh.read(src), zm, rtol=0.0)
    # and the library reads its compressed file back to the same bytes
    m2 = Mesh.read_osh(ctx, tmp_path / "z.osh")
    m2.write_osh(tmp_path / "u.osh")
    m2.close()
    _same_files(src, str(tmp_path / "u.osh"))


def test_tags_it_does_not_model_survive(ctx, tmp_path):
    from omega_h_gb300.mesh import Mesh
    m0 = osh.read(os.path.join(OSH, CASES[0], "out.osh"))
    dim = m0["dim"]
    ne = m0["tags"][dim][0][3].size
    nv = m0["nverts"]
    rng = np.random.default_rng(3)
    m0["tags"][dim].insert(1, ("density", 1, 5, rng.uniform(size=ne)))
    m0["tags"][0].append(("flag", 2, 0, rng.integers(-5, 5, 2 * nv).astype(np.int8)))
    gi = [t[0] for t in m0["tags"][0]].index("global")
    m0["tags"][0][gi] = ("global", 1, 3, np.arange(nv, dtype=np.int64)[::-1].copy())
    osh.write(str(tmp_path / "x.osh"), m0)
    m = Mesh.read_osh(ctx, tmp_path / "x.osh")
    m.write_osh(tmp_path / "y.osh")
    m.close()
    _same_files(str(tmp_path / "x.osh"), str(tmp_path / "y.osh"))


def test_scalar_metric_round_trip(ctx, tmp_path):
    """A mesh with an isotropic metric (one component per vertex) is written
    with a one-component metric tag, as the reference writes it, and reads
    back to the same bytes."""
    from omega_h_gb300.mesh import Mesh, adapt_opts
    m = Mesh.build_box(ctx, 3, 6)
    m.apply_workload(6, 4, 13)
    m.adapt_pass(adapt_opts(3, min_quality_allowed=0.2))
    m.write_osh(tmp_path / "a.osh")
    m.close()
    f = osh.read(str(tmp_path / "a.osh"))
    name, ncomps, ty, arr = [t for t in f["tags"][0] if t[0] == "metric"][0]
    assert ncomps == 1 and ty == 5 and arr.size == f["nverts"]
    r = Mesh.read_osh(ctx, tmp_path / "a.osh")
    assert r.metric_components() == 1
    r.write_osh(tmp_path / "b.osh")
    r.close()
    _same_files(str(tmp_path / "a.osh"), str(tmp_path / "b.osh"))
