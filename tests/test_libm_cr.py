"""The correctly rounded cbrt, log, exp, cos and acos of ohg_libm.cuh (the
functions the GPU path and the oracle's ORC_CR_LIBM variants call), compiled
for the host: every result checked against mpmath at 300 bits on the
arguments where they differ from glibc's and on a random sample; the quick
evaluations checked against the accurate ones (OHG_LIBM_QUICK=0) on millions
of arguments.  Also measures how often glibc's results are not correctly
rounded.  CPU only."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

mpmath = pytest.importorskip("mpmath")


def _lib(tmp_path_factory, quick):
    out = str(tmp_path_factory.mktemp("libm") / f"libm_host_{quick}.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                    f"-DOHG_LIBM_QUICK={quick}", os.path.join(ROOT, "tests", "libm_host.cpp"),
                    "-o", out], check=True)
    return ctypes.CDLL(out)


@pytest.fixture(scope="module")
def libs(tmp_path_factory):
    return _lib(tmp_path_factory, 1), _lib(tmp_path_factory, 0)


def _call(lib, fn, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    getattr(lib, fn)(x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p),
                     ctypes.c_long(x.size))
    return y


def _args(name, rng, n):
    if name in ("cbrt", "log"):
        x = rng.uniform(1, 2, n) * np.exp2(rng.integers(-1074, 1023, n).astype(float))
        extra = [1 + rng.uniform(-1e-3, 1e-3, n // 4), np.exp(rng.uniform(-30, 30, n // 4))]
        if name == "cbrt":
            extra.append(-x[: n // 4])
        return np.concatenate([x] + extra + [np.array([1.0, 8.0, 0.5, 5e-324, 1e-310])])
    if name == "exp":
        return np.concatenate([rng.uniform(-745, 709.7, n), rng.uniform(-30, 30, n // 2),
                               rng.uniform(-1e-6, 1e-6, n // 4), np.array([0.0, 1.0, -1.0])])
    if name == "cos":
        return np.concatenate([rng.uniform(-np.pi, np.pi, n), rng.uniform(-1000, 1000, n // 4),
                               rng.uniform(-1e-3, 1e-3, n // 8),
                               np.array([0.0, np.pi / 2, np.pi, 0.7853981633974483])])
    return np.concatenate([rng.uniform(-1, 1, n), 1 - rng.uniform(0, 1e-6, n // 4),
                           -1 + rng.uniform(0, 1e-6, n // 4),
                           1 - np.exp2(-rng.integers(1, 53, n // 8).astype(float)),
                           np.array([1.0, -1.0, 0.0, 0.5, -0.5])])


EXACT = {"cbrt": mpmath.cbrt, "log": mpmath.log, "exp": mpmath.exp, "cos": mpmath.cos,
         "acos": mpmath.acos}


def _exact(name, v):
    if name == "cbrt" and v < 0:
        return -float(mpmath.cbrt(mpmath.mpf(-v)))
    return float(EXACT[name](mpmath.mpf(v)))


@pytest.mark.parametrize("name", ["cbrt", "log", "exp", "cos", "acos"])
def test_correctly_rounded(libs, name):
    mpmath.mp.prec = 300
    rng = np.random.default_rng(7)
    x = _args(name, rng, 1_000_000)
    quick, accurate = libs
    cr = _call(quick, name + "_cr_n", x)
    assert np.array_equal(cr.view(np.uint64), _call(accurate, name + "_cr_n", x).view(np.uint64))
    gl = _call(quick, name + "_glibc_n", x)
    differ = np.nonzero(cr != gl)[0]
    check = np.concatenate([differ[:2000], rng.choice(x.size, 3000, replace=False)])
    wrong = [i for i in check if _exact(name, x[i]) != cr[i]]
    sample = rng.choice(x.size, 2000, replace=False)
    glibc_wrong = sum(_exact(name, x[i]) != gl[i] for i in sample)
    print(f"{name}: {x.size} arguments, differ from glibc on {differ.size}; "
          f"glibc not correctly rounded on {glibc_wrong} of {sample.size} sampled")
    assert not wrong, [(x[i], cr[i]) for i in wrong[:5]]
