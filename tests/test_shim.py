"""The C++ drop-in for Omega_h::Mesh callers (omega_h_gb300/shim) compiled
against the reference's own headers and linked with the reference's library
(built from its sources by oracle/ref.mk) and libohg.so; and the plain C++
caller of include/ohg.h (tests/capi_caller.cpp) compiled and linked.  CPU
only: the shim's refusals are checked before any GPU work; the GPU run of
the whole upload -> pass -> read-back sequence is test_gpu_capi_caller.py."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)


def _reference_src():
    import __graft_entry__
    return __graft_entry__.REFERENCE


@pytest.fixture(scope="module")
def shim_check(tmp_path_factory):
    ref = _reference_src()
    lib_ref = os.path.join(ROOT, "oracle", "_ref", "libomega_h_ref.a")
    if not os.path.isdir(os.path.join(ref, "src")):
        pytest.skip("the reference's sources are not here")
    if not os.path.exists(lib_ref):
        subprocess.run(["make", "-f", "oracle/ref.mk", f"REF={ref}", "-j8"], cwd=ROOT,
                       check=True, stdout=subprocess.DEVNULL)
    from omega_h_gb300 import build
    build.build()
    out = str(tmp_path_factory.mktemp("shim") / "shim_check")
    inc = ["-I" + os.path.join(ROOT, "oracle", "_ref", "include"), "-I" + os.path.join(ref, "src"),
           "-I" + os.path.join(ref, "tpl"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "omega_h_gb300", "shim")]
    libdir = os.path.join(ROOT, "omega_h_gb300")
    subprocess.run(["g++", "-std=c++17", "-O1", *inc,
                    os.path.join(ROOT, "tests", "shim_check.cpp"),
                    os.path.join(ROOT, "omega_h_gb300", "shim", "omega_h_adapt_gb300.cpp"),
                    lib_ref, "-L" + libdir, "-lohg", "-Wl,-rpath," + libdir, "-o", out],
                   check=True)
    return out


@pytest.mark.parametrize("case,message", [
    ("no_metric", 'the mesh has no "metric" tag'),
    ("user_field", 'tag "user_field" on dimension 0 would not be transferred'),
    ("null_context", "ohg_mesh_from_arrays failed (8): null context"),
])
def test_shim_refuses_what_it_cannot_carry(shim_check, case, message):
    """The reference's fail() prints and aborts in this build: each case runs in
    its own process and must end there, with the message."""
    r = subprocess.run([shim_check, case], capture_output=True, text=True)
    assert r.returncode != 0 and "not refused" not in r.stdout
    assert message in r.stderr, r.stderr


def test_capi_caller_builds(tmp_path):
    from omega_h_gb300 import build
    build.build()
    libdir = os.path.join(ROOT, "omega_h_gb300")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "capi_caller.cpp"), "-L" + libdir, "-lohg",
                    "-Wl,-rpath," + libdir, "-o", str(tmp_path / "capi_caller")], check=True)
