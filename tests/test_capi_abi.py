"""The C-ABI library builds, loads and exports every entry point that
include/ohg.h declares; host-only entry points behave without a GPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ohg.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ohg_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from omega_h_gb300 import build
    build.build()
    from omega_h_gb300 import _lib
    return _lib.load()


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("ohg_adapt_pass", "ohg_measure_edges_metric", "ohg_measure_qualities",
                     "ohg_refine_qualities", "ohg_coarsen_qualities", "ohg_swap3d_qualities",
                     "ohg_find_indset", "ohg_invert_adj", "ohg_reflect_down",
                     "ohg_hilbert_sort", "ohg_sort_by_keys", "ohg_prevent_coarsen_overshoot",
                     "ohg_choose_rails"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    from omega_h_gb300 import _lib
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_adapt_opts_defaults_match_reference(lib):
    # AdaptOpts::AdaptOpts(Int dim) (src/Omega_h_adapt.cpp:52-85)
    from omega_h_gb300 import _lib
    for dim, (qa, qd) in {3: (0.2, 0.3), 2: (0.3, 0.4)}.items():
        o = _lib.AdaptOpts()
        _lib.call("ohg_adapt_opts_default", dim, ctypes.byref(o))
        assert o.min_length_desired == 1.0 / 2 ** 0.5
        assert o.max_length_desired == 2 ** 0.5
        assert o.max_length_allowed == 2 ** 0.5 * 2.0
        assert (o.min_quality_allowed, o.min_quality_desired) == (qa, qd)
        assert o.nsliver_layers == 4


def test_invalid_arguments_fail_loudly_without_a_gpu(lib):
    from omega_h_gb300 import _lib
    h = ctypes.c_void_p()
    with pytest.raises(_lib.OhgError) as e:
        _lib.call("ohg_build_box", None, 4, 8, ctypes.byref(h))
    assert e.value.code == 8
    with pytest.raises(_lib.OhgError):
        _lib.call("ohg_adapt_opts_default", 5, ctypes.byref(_lib.AdaptOpts()))
    with pytest.raises(_lib.OhgError):
        _lib.call("ohg_mesh_nents", None, 0, ctypes.byref(ctypes.c_int()))
