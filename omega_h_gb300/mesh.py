"""Host-side mirror of the Omega_h Mesh / Read<T> / AdaptOpts interface on
the adapt path, over the C ABI.  Device arrays are torch CUDA tensors; the
computation is the CUDA library's (no CPU path exists).
"""
import ctypes

import torch

from . import _lib

# dtype of every named mesh array (see ohg_mesh_get_array in include/ohg.h)
_F64 = ("coords", "metric", "length", "quality")


def array_dtype(name):
    if name in _F64:
        return torch.float64
    if name.startswith(("class_dim_", "downcodes", "up_codes_")):
        return torch.int8
    if name.startswith("global_"):
        return torch.int64
    return torch.int32


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class Context:
    """One device, one stream (ohg_context)."""

    def __init__(self, device=0):
        self.device = device
        h = ctypes.c_void_p()
        _lib.call("ohg_context_create", device, ctypes.byref(h))
        self.handle = h

    def launches(self):
        v = ctypes.c_ulonglong()
        _lib.call("ohg_context_launches", self.handle, ctypes.byref(v))
        return v.value

    def syncs(self):
        v = ctypes.c_ulonglong()
        _lib.call("ohg_context_syncs", self.handle, ctypes.byref(v))
        return v.value

    def pool_bytes(self, reset_high=False):
        """(bytes in use, bytes reserved, high-water mark of bytes in use) of
        the device's memory pool, which all contexts of the device share."""
        u, r, h = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        _lib.call("ohg_context_pool_bytes", self.handle, 1 if reset_high else 0,
                  ctypes.byref(u), ctypes.byref(r), ctypes.byref(h))
        return u.value, r.value, h.value

    def allocations(self):
        """Device allocations the library has made on this context."""
        v = ctypes.c_ulonglong()
        _lib.call("ohg_context_allocations", self.handle, ctypes.byref(v))
        return v.value

    def autotune(self, mode):
        """Launch-shape autotuner: "off", "explore" or "frozen" (default)."""
        _lib.call("ohg_context_autotune", self.handle, {"off": 0, "explore": 1, "frozen": 2}[mode])

    def force_variant(self, v):
        """Run every tuned launch site with variant v (None: the tuner's)."""
        _lib.call("ohg_context_force_variant", self.handle, -1 if v is None else int(v))

    def tuning(self):
        """(sites seen, sites with a choice, choices other than the default)."""
        v = (ctypes.c_int * 3)()
        _lib.call("ohg_context_tuning", self.handle, v)
        return tuple(int(x) for x in v)

    def set_screening(self, on):
        """FP32 screening with exact FP64 recheck (True, default) or FP64
        throughout (False)."""
        _lib.call("ohg_context_set_screening", self.handle, 1 if on else 0)

    def screen_counts(self, reset=False):
        """(tets screened, tets recomputed in FP64, lengths screened, lengths
        recomputed in FP64) since the last reset."""
        v = (ctypes.c_ulonglong * 4)()
        _lib.call("ohg_context_screen_counts", self.handle, v, 1 if reset else 0)
        return tuple(int(x) for x in v)

    def time_kernels(self, on):
        _lib.call("ohg_context_time_kernels", self.handle, 1 if on else 0)

    def kernel_time(self, name, reset=False):
        """(total ms, total algorithmic bytes, launches) of a named kernel."""
        ms, by, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        _lib.call("ohg_context_kernel_time", self.handle, name.encode(), ctypes.byref(ms),
                  ctypes.byref(by), ctypes.byref(n), 1 if reset else 0)
        return ms.value, by.value, n.value

    def close(self):
        if self.handle:
            _lib.call("ohg_context_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def adapt_opts(dim, **overrides):
    """AdaptOpts(dim) defaults (src/Omega_h_adapt.cpp:52-85) with overrides."""
    o = _lib.AdaptOpts()
    _lib.call("ohg_adapt_opts_default", dim, ctypes.byref(o))
    for k, v in overrides.items():
        setattr(o, k, v)
    return o


class Mesh:
    """A device-resident simplex mesh (ohg_mesh)."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.handle = handle

    @classmethod
    def build_box(cls, ctx, dim, n):
        """build_box on the unit square/cube, Hilbert-ordered and classified."""
        h = ctypes.c_void_p()
        _lib.call("ohg_build_box", ctx.handle, dim, n, ctypes.byref(h))
        return cls(ctx, h)

    @classmethod
    def from_elems(cls, ctx, dim, ev2v, coords, metric):
        h = ctypes.c_void_p()
        nverts = coords.numel() // dim
        _lib.call("ohg_mesh_from_elems", ctx.handle, dim, nverts, ev2v.numel() // (dim + 1),
                  _ptr(ev2v), _ptr(coords), _ptr(metric), ctypes.byref(h))
        return cls(ctx, h)

    @classmethod
    def read_osh(cls, ctx, path):
        """A mesh from an .osh directory (the reference's binary format)."""
        h = ctypes.c_void_p()
        _lib.call("ohg_mesh_read_osh", ctx.handle, str(path).encode(), ctypes.byref(h))
        return cls(ctx, h)

    def write_osh(self, path, compress=False):
        """Write the mesh as an .osh directory, as the reference would."""
        _lib.call("ohg_mesh_write_osh", self.handle, str(path).encode(), 1 if compress else 0)

    def apply_workload(self, n, seed, metric_kind):
        _lib.call("ohg_mesh_apply_workload", self.handle, n, seed, metric_kind)

    @property
    def dim(self):
        v = ctypes.c_int()
        _lib.call("ohg_mesh_dim", self.handle, ctypes.byref(v))
        return v.value

    def nents(self, d):
        v = ctypes.c_int()
        _lib.call("ohg_mesh_nents", self.handle, d, ctypes.byref(v))
        return v.value

    def nelems(self):
        return self.nents(self.dim)

    def device_bytes(self):
        """Device memory held by the mesh (arrays, adjacencies, caches)."""
        v = ctypes.c_longlong()
        _lib.call("ohg_mesh_device_bytes", self.handle, ctypes.byref(v))
        return v.value

    def get(self, name):
        """A copy of a named mesh array as a CUDA tensor."""
        nb = ctypes.c_longlong()
        _lib.call("ohg_mesh_array_bytes", self.handle, name.encode(), ctypes.byref(nb))
        dt = array_dtype(name)
        t = torch.empty(nb.value // torch.tensor([], dtype=dt).element_size(), dtype=dt,
                        device=f"cuda:{self.ctx.device}")
        _lib.call("ohg_mesh_get_array", self.handle, name.encode(), _ptr(t), nb.value)
        return t

    def set(self, name, t):
        t = t.contiguous()
        _lib.call("ohg_mesh_set_array", self.handle, name.encode(), _ptr(t),
                  t.numel() * t.element_size())

    def adapt_pass(self, opts=None):
        o = opts or adapt_opts(self.dim)
        s = _lib.PassStats()
        _lib.call("ohg_adapt_pass", self.handle, ctypes.byref(o), ctypes.byref(s))
        return s.as_dict()

    def adapt(self, opts=None):
        """Omega_h::adapt: passes until lengths settle, then swaps and sliver
        collapses until the quality goal is met or nothing helps."""
        o = opts or adapt_opts(self.dim)
        r = _lib.AdaptResult()
        _lib.call("ohg_adapt", self.handle, ctypes.byref(o), ctypes.byref(r))
        return r.as_dict()

    def coarsen_slivers(self, opts=None):
        return self._op("ohg_coarsen_slivers", opts)

    def _op(self, fname, opts):
        o = opts or adapt_opts(self.dim)
        did = ctypes.c_int()
        _lib.call(fname, self.handle, ctypes.byref(o), ctypes.byref(did))
        return bool(did.value)

    def refine_by_size(self, opts=None):
        return self._op("ohg_refine_by_size", opts)

    def coarsen_by_size(self, opts=None):
        return self._op("ohg_coarsen_by_size", opts)

    def swap_edges(self, opts=None):
        return self._op("ohg_swap_edges", opts)

    # ---- stage kernels --------------------------------------------------
    def _dev(self):
        return f"cuda:{self.ctx.device}"

    def measure_edges_metric(self, a2e=None):
        n = a2e.numel() if a2e is not None else self.nents(1)
        out = torch.empty(n, dtype=torch.float64, device=self._dev())
        _lib.call("ohg_measure_edges_metric", self.handle, _ptr(a2e), n, _ptr(out))
        return out

    def measure_qualities(self, a2e=None):
        n = a2e.numel() if a2e is not None else self.nelems()
        out = torch.empty(n, dtype=torch.float64, device=self._dev())
        _lib.call("ohg_measure_qualities", self.handle, _ptr(a2e), n, _ptr(out))
        return out

    def metric_components(self):
        """6 (3D) or 3 (2D) for a packed tensor metric, 1 for an isotropic one."""
        nb = ctypes.c_longlong()
        _lib.call("ohg_mesh_array_bytes", self.handle, b"metric", ctypes.byref(nb))
        return nb.value // 8 // max(1, self.nents(0))

    def mident_metrics(self, edges):
        mc = self.metric_components()
        out = torch.empty(edges.numel() * mc, dtype=torch.float64, device=self._dev())
        _lib.call("ohg_get_mident_metrics", self.handle, _ptr(edges), edges.numel(), _ptr(out))
        return out

    def refine_qualities(self, c2e):
        out = torch.empty(c2e.numel(), dtype=torch.float64, device=self._dev())
        _lib.call("ohg_refine_qualities", self.handle, _ptr(c2e), c2e.numel(), _ptr(out))
        return out

    def check_collapse_class(self, c2e, codes):
        out = torch.empty_like(codes)
        _lib.call("ohg_check_collapse_class", self.handle, _ptr(c2e), c2e.numel(), _ptr(codes), _ptr(out))
        return out

    def check_collapse_exposure(self, c2e, codes):
        out = torch.empty_like(codes)
        _lib.call("ohg_check_collapse_exposure", self.handle, _ptr(c2e), c2e.numel(), _ptr(codes),
                  _ptr(out))
        return out

    def prevent_coarsen_overshoot(self, max_length, c2e, codes):
        out = torch.empty_like(codes)
        _lib.call("ohg_prevent_coarsen_overshoot", self.handle, max_length, _ptr(c2e), c2e.numel(),
                  _ptr(codes), _ptr(out))
        return out

    def coarsen_qualities(self, c2e, codes):
        out = torch.empty(c2e.numel() * 2, dtype=torch.float64, device=self._dev())
        _lib.call("ohg_coarsen_qualities", self.handle, _ptr(c2e), c2e.numel(), _ptr(codes), _ptr(out))
        return out

    def choose_rails(self, c2e, codes, quals2):
        nv = self.nents(0)
        vc = torch.empty(nv, dtype=torch.int8, device=self._dev())
        vq = torch.empty(nv, dtype=torch.float64, device=self._dev())
        vr = torch.empty(nv, dtype=torch.int64, device=self._dev())
        _lib.call("ohg_choose_rails", self.handle, _ptr(c2e), c2e.numel(), _ptr(codes), _ptr(quals2),
                  _ptr(vc), _ptr(vq), _ptr(vr))
        return vc, vq, vr

    def mark_sliver_layers(self, qual_ceil, nlayers):
        out = torch.empty(self.nelems(), dtype=torch.int8, device=self._dev())
        _lib.call("ohg_mark_sliver_layers", self.handle, qual_ceil, nlayers, _ptr(out))
        return out

    def swap2d_qualities(self, max_length_allowed, c2e):
        q = torch.empty(c2e.numel(), dtype=torch.float64, device=self._dev())
        _lib.call("ohg_swap2d_qualities", self.handle, max_length_allowed, _ptr(c2e), c2e.numel(),
                  _ptr(q))
        return q

    def swap3d_qualities(self, max_length_allowed, c2e):
        q = torch.empty(c2e.numel(), dtype=torch.float64, device=self._dev())
        cf = torch.empty(c2e.numel(), dtype=torch.int8, device=self._dev())
        _lib.call("ohg_swap3d_qualities", self.handle, max_length_allowed, _ptr(c2e), c2e.numel(),
                  _ptr(q), _ptr(cf))
        return q, cf

    def find_indset(self, ent_dim, quality, candidates):
        out = torch.empty_like(candidates)
        r = ctypes.c_int()
        _lib.call("ohg_find_indset", self.handle, ent_dim, _ptr(quality), _ptr(candidates), _ptr(out),
                  ctypes.byref(r))
        return out, r.value

    # ---- metric tools ---------------------------------------------------
    def _metric_out(self):
        return torch.empty(self.nents(0) * (6 if self.dim == 3 else 3), dtype=torch.float64,
                           device=self._dev())

    def implied_metrics(self):
        """get_implied_metrics: the metric the current elements imply."""
        out = self._metric_out()
        _lib.call("ohg_mesh_implied_metrics", self.handle, _ptr(out))
        return out

    def limit_metric_gradation(self, metrics, max_rate=1.0, tol=1e-3):
        """limit_metric_gradation; returns (metrics, sweeps)."""
        out = self._metric_out()
        steps = ctypes.c_int()
        _lib.call("ohg_mesh_limit_metric_gradation", self.handle, _ptr(metrics.contiguous()),
                  max_rate, tol, _ptr(out), ctypes.byref(steps))
        return out, steps.value

    def expected_nelems(self, metrics):
        v = ctypes.c_double()
        _lib.call("ohg_mesh_expected_nelems", self.handle, _ptr(metrics.contiguous()),
                  ctypes.byref(v))
        return v.value

    def generate_metrics(self, sources, **opts):
        """generate_metrics.  sources: dicts with type ("constant", "given",
        "implied"), knob, isotropy ("anisotropic", "iso_size"), scales
        (bool) and, for "given", metrics (a device tensor).  opts: the
        MetricInput fields.  Returns (metrics, element-count iterations)."""
        types = {"constant": 0, "given": 3, "implied": 4}
        isos = {"anisotropic": 0, "iso_length": 1, "iso_size": 2}
        mi = _lib.MetricInput()
        _lib.call("ohg_metric_input_default", ctypes.byref(mi))
        keep = []
        for i, s in enumerate(sources):
            src = mi.sources[i]
            src.type = types[s["type"]]
            src.knob = s.get("knob", 1.0)
            src.isotropy = isos[s.get("isotropy", "anisotropic")]
            src.scales = 1 if s.get("scales", True) else 0
            if "metrics" in s:
                t = s["metrics"].contiguous()
                keep.append(t)
                src.given = t.data_ptr()
        mi.nsources = len(sources)
        for k, v in opts.items():
            setattr(mi, k, v)
        out = self._metric_out()
        nit = ctypes.c_int()
        _lib.call("ohg_mesh_generate_metrics", self.handle, ctypes.byref(mi), _ptr(out),
                  ctypes.byref(nit))
        return out, nit.value

    def close(self):
        if self.handle:
            _lib.call("ohg_mesh_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _handles(meshes):
    return (ctypes.c_void_p * len(meshes))(*[m.handle.value for m in meshes])


def concat(ctx, meshes):
    """The disjoint union of meshes of one dimension (ohg_mesh_concat)."""
    h = ctypes.c_void_p()
    _lib.call("ohg_mesh_concat", ctx.handle, _handles(meshes), len(meshes), ctypes.byref(h))
    return Mesh(ctx, h)


def split(union, n):
    """The n parts of a union (ohg_mesh_split); the union's arrays are
    rewritten, so close it afterwards."""
    outs = (ctypes.c_void_p * n)()
    _lib.call("ohg_mesh_split", union.handle, n, outs)
    return [Mesh(union.ctx, ctypes.c_void_p(outs[i])) for i in range(n)]


def intersect_metrics(ctx, dim, a, b):
    """intersect_metrics over packed metric tensors (device tensors)."""
    out = torch.empty_like(a)
    _lib.call("ohg_intersect_metrics", ctx.handle, dim, a.numel() // (6 if dim == 3 else 3),
              _ptr(a.contiguous()), _ptr(b.contiguous()), _ptr(out))
    return out


def clamp_metrics(ctx, dim, m, h_min, h_max):
    out = torch.empty_like(m)
    _lib.call("ohg_clamp_metrics", ctx.handle, dim, m.numel() // (6 if dim == 3 else 3),
              _ptr(m.contiguous()), h_min, h_max, _ptr(out))
    return out


def hessian_metrics(ctx, dim, hessians, eps):
    out = torch.empty_like(hessians)
    _lib.call("ohg_hessian_metrics", ctx.handle, dim, hessians.numel() // (6 if dim == 3 else 3),
              _ptr(hessians.contiguous()), eps, _ptr(out))
    return out


def adapt_pass_batch(ctx, meshes, opts=None):
    """One adapt pass over the union of meshes (ohg_adapt_pass_batch); each
    mesh is replaced by its result.  Returns the union's pass stats."""
    o = opts or adapt_opts(meshes[0].dim)
    s = _lib.PassStats()
    _lib.call("ohg_adapt_pass_batch", ctx.handle, _handles(meshes), len(meshes), ctypes.byref(o),
              ctypes.byref(s))
    return s.as_dict()
