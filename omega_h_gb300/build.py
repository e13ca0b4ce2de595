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
SOURCES = ["ohg_prims.cu", "ohg_mesh.cu", "ohg_adapt.cu", "ohg_capi.cu"]
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


def _compile(src):
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [NVCC, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def build(force=False, verbose=False):
    """Compile and link libohg.so unless it is newer than every source."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_dep_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
