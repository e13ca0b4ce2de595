"""A compiled C++ program that uses only include/ohg.h (tests/capi_caller.cpp)
runs the full upload -> adapt pass -> read-back sequence from plain host
arrays: the reference's input mesh of box12_shock (refine, coarsen and swap
on a 12^3 shock-metric box) in, the reference's mesh after the pass out."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, SMALL_CASES, compare_arrays, load_dump_dir, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def caller(tmp_path_factory):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from omega_h_gb300 import build
    build.build()
    libdir = os.path.join(ROOT, "omega_h_gb300")
    out = str(tmp_path_factory.mktemp("caller") / "capi_caller")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "capi_caller.cpp"), "-L" + libdir, "-lohg",
                    "-Wl,-rpath," + libdir, "-o", out], check=True)
    return out


def test_compiled_caller_matches_reference_pass(caller, tmp_path):
    case = "box12_shock"
    g = load_golden(case)
    dim, mqa = SMALL_CASES[case][0], SMALL_CASES[case][4]
    ind, outd = tmp_path / "in", tmp_path / "out"
    ind.mkdir()
    outd.mkdir()
    nents = [g["in_coords"].size // dim] + [g[f"in_down_{d}"].size // (d + 1)
                                             for d in range(1, dim + 1)]
    nents += [0] * (4 - len(nents))
    (ind / "meta.txt").write_text(" ".join(str(x) for x in [dim, *nents, mqa]))
    for d in range(dim + 1):
        if d > 0:
            g[f"in_down_{d}"].astype(np.int32).tofile(ind / f"down_{d}.bin")
        if d > 1:
            g[f"in_downcodes_{d}"].astype(np.int8).tofile(ind / f"downcodes_{d}.bin")
        g[f"in_class_dim_{d}"].astype(np.int8).tofile(ind / f"class_dim_{d}.bin")
        g[f"in_class_id_{d}"].astype(np.int32).tofile(ind / f"class_id_{d}.bin")
    g["in_coords"].astype(np.float64).tofile(ind / "coords.bin")
    g["in_metric"].astype(np.float64).tofile(ind / "metric.bin")
    r = subprocess.run([caller, str(ind), str(outd)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    print(r.stdout.strip())
    got = load_dump_dir(str(outd))
    assert list(got["pass_flags"]) == list(g["pass_flags"])
    keys = [k for k in g if k.startswith("out_") and k in got]
    assert len(keys) >= 15
    fails, maxerr, ndiff = compare_arrays(g, got, keys=keys)
    print(f"{case} through the compiled caller: max real rel err {maxerr:.2e}")
    assert not fails, fails[:10]
