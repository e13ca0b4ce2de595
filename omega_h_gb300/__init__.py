"""omega_h_gb300: the per-pass core of Omega_h::adapt() on a GB300 GPU.

The computation lives in libohg.so (hand-written CUDA for sm_103a, C ABI in
include/ohg.h); this package is its host-side interface.
"""
from ._lib import AdaptOpts, OhgError, PassStats, load  # noqa: F401

__all__ = ["AdaptOpts", "OhgError", "PassStats", "load", "Context", "Mesh", "adapt_opts"]


def __getattr__(name):
    # torch-backed classes are imported lazily so the ABI can be probed
    # without initialising CUDA
    if name in ("Context", "Mesh", "adapt_opts"):
        from . import mesh
        return getattr(mesh, name)
    raise AttributeError(name)
