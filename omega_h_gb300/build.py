"""Builds the CUDA library omega_h_gb300/libohg.so for sm_103a in place.

Translation units compile in parallel with nvcc; -fmad=false keeps every
a*b+c as two rounded operations (the reference's host arithmetic), the
default IEEE division and square root are kept.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libohg.so")
# bounds-checked variant: every device array subscript is checked and each
# launch is followed by a synchronising check that names its source line
LIB_CHECKED = os.path.join(HERE, "libohg_checked.so")
SOURCES = ["ohg_prims.cu", "ohg_mesh.cu", "ohg_adapt.cu", "ohg_batch.cu", "ohg_osh.cu",
           "ohg_metric.cu", "ohg_capi.cu"]
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "--extended-lambda", "-fmad=false", "-lineinfo",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]


def _newest_dep_mtime():
    t = 0.0
    for d in (CSRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _compile(src, checked=False):
    bdir = BUILD + ("_checked" if checked else "")
    obj = os.path.join(bdir, src.replace(".cu", ".o"))
    extra = ["-DOHG_CHECKED"] if checked else []
    cmd = [NVCC, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def build(force=False, verbose=False, checked=False):
    """Compile and link libohg.so (or the checked variant) unless it is newer
    than every source."""
    lib = LIB_CHECKED if checked else LIB
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= _newest_dep_mtime():
        return lib
    os.makedirs(BUILD + ("_checked" if checked else ""), exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, checked), SOURCES))
    tmp = lib + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv)
