"""ctypes binding of the C ABI in include/ohg.h (libohg.so, built in place)."""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# OHG_CHECKED=1 selects the bounds-checked build of the same library
LIB_PATH = os.path.join(_HERE, "libohg_checked.so" if os.environ.get("OHG_CHECKED") == "1"
                        else "libohg.so")

c_int, c_double, c_void_p, c_char_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p
c_ll, c_ull = ctypes.c_longlong, ctypes.c_ulonglong
P = ctypes.POINTER

STATUS = {0: "OK", 1: "CUDA", 2: "BOUNDS", 3: "LOOP_TOO_BIG", 4: "NO_MATCH", 5: "TIMEOUT",
          6: "OOM", 7: "ADMISSION", 8: "INVALID", 9: "NUMERIC", 10: "TOPOLOGY"}


class OhgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"ohg error {code} ({STATUS.get(code, '?')}): {msg}")
        self.code = code


class AdaptOpts(ctypes.Structure):
    """Mirror of ohg_adapt_opts / the AdaptOpts fields one pass uses."""
    _fields_ = [("min_length_desired", c_double), ("max_length_desired", c_double),
                ("max_length_allowed", c_double), ("min_quality_allowed", c_double),
                ("min_quality_desired", c_double), ("nsliver_layers", c_int)]


class AdaptResult(ctypes.Structure):
    _fields_ = [("did", c_int), ("quality_satisfied", c_int), ("refines", c_int),
                ("coarsens", c_int), ("swaps", c_int), ("sliver_coarsens", c_int),
                ("length_rounds", c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MetricSource(ctypes.Structure):
    """ohg_metric_source (MetricSource, src/Omega_h_metric_input.cpp:13-20)."""
    _fields_ = [("type", c_int), ("knob", c_double), ("isotropy", c_int), ("scales", c_int),
                ("given", c_void_p)]


class MetricInput(ctypes.Structure):
    """ohg_metric_input (MetricInput, src/Omega_h_metric_input.cpp:23-35)."""
    _fields_ = [("nsources", c_int), ("sources", MetricSource * 8),
                ("should_limit_lengths", c_int), ("min_length", c_double),
                ("max_length", c_double), ("should_limit_gradation", c_int),
                ("max_gradation_rate", c_double), ("gradation_convergence_tolerance", c_double),
                ("should_limit_element_count", c_int), ("max_element_count", c_double),
                ("min_element_count", c_double), ("element_count_over_relaxation", c_double),
                ("nsmoothing_steps", c_int)]


class PassStats(ctypes.Structure):
    _fields_ = [("did_refine", c_int), ("did_coarsen", c_int), ("did_swap", c_int),
                ("nelems_in", c_int), ("nelems_out", c_int), ("refine_keys", c_int),
                ("coarsen_keys", c_int), ("swap_keys", c_int), ("indset_rounds", c_int),
                ("min_quality", c_double), ("ms_refine", ctypes.c_float),
                ("ms_coarsen", ctypes.c_float), ("ms_swap", ctypes.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# name -> argument types (restype is int unless listed in _RESTYPE)
SIGNATURES = {
    "ohg_last_error": [],
    "ohg_context_create": [c_int, P(c_void_p)],
    "ohg_context_destroy": [c_void_p],
    "ohg_context_launches": [c_void_p, P(c_ull)],
    "ohg_context_syncs": [c_void_p, P(c_ull)],
    "ohg_context_allocations": [c_void_p, P(c_ull)],
    "ohg_context_pool_bytes": [c_void_p, c_int, P(c_ll), P(c_ll), P(c_ll)],
    "ohg_mesh_device_bytes": [c_void_p, P(c_ll)],
    "ohg_fp64_peak": [c_void_p, c_int, P(c_double)],
    "ohg_context_autotune": [c_void_p, c_int],
    "ohg_context_force_variant": [c_void_p, c_int],
    "ohg_context_tuning": [c_void_p, P(c_int)],
    "ohg_context_stream": [c_void_p, P(c_void_p)],
    "ohg_build_box": [c_void_p, c_int, c_int, P(c_void_p)],
    "ohg_mesh_from_arrays": [c_void_p, c_int, P(c_int), P(c_void_p), P(c_void_p), P(c_void_p),
                             P(c_void_p), c_void_p, c_void_p, P(c_void_p)],
    "ohg_mesh_clone": [c_void_p, P(c_void_p)],
    "ohg_mesh_clone_to": [c_void_p, c_void_p, P(c_void_p)],
    "ohg_mesh_write_osh": [c_void_p, c_char_p, c_int],
    "ohg_mesh_read_osh": [c_void_p, c_char_p, P(c_void_p)],
    "ohg_osh_zlib": [P(c_int)],
    "ohg_intersect_metrics": [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p],
    "ohg_cubic_roots": [c_void_p, c_int, c_void_p, c_double, c_void_p, c_void_p, c_void_p],
    "ohg_decompose_eigen": [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p],
    "ohg_clamp_metrics": [c_void_p, c_int, c_int, c_void_p, c_double, c_double, c_void_p],
    "ohg_hessian_metrics": [c_void_p, c_int, c_int, c_void_p, c_double, c_void_p],
    "ohg_mesh_implied_metrics": [c_void_p, c_void_p],
    "ohg_mesh_limit_metric_gradation": [c_void_p, c_void_p, c_double, c_double, c_void_p, P(c_int)],
    "ohg_mesh_expected_nelems": [c_void_p, c_void_p, P(c_double)],
    "ohg_metric_input_default": [P(MetricInput)],
    "ohg_mesh_generate_metrics": [c_void_p, P(MetricInput), c_void_p, P(c_int)],
    "ohg_mesh_apply_workload": [c_void_p, c_int, c_ull, c_int],
    "ohg_mesh_from_elems": [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, P(c_void_p)],
    "ohg_mesh_destroy": [c_void_p],
    "ohg_mesh_dim": [c_void_p, P(c_int)],
    "ohg_mesh_nents": [c_void_p, c_int, P(c_int)],
    "ohg_mesh_array_bytes": [c_void_p, c_char_p, P(c_ll)],
    "ohg_mesh_get_array": [c_void_p, c_char_p, c_void_p, c_ll],
    "ohg_mesh_get_arrays": [c_void_p, c_int, c_void_p, c_void_p, c_void_p],
    "ohg_mesh_set_array": [c_void_p, c_char_p, c_void_p, c_ll],
    "ohg_adapt_opts_default": [c_int, P(AdaptOpts)],
    "ohg_adapt_pass": [c_void_p, P(AdaptOpts), P(PassStats)],
    "ohg_adapt": [c_void_p, P(AdaptOpts), P(AdaptResult)],
    "ohg_coarsen_slivers": [c_void_p, P(AdaptOpts), P(c_int)],
    "ohg_mesh_concat": [c_void_p, P(c_void_p), c_int, P(c_void_p)],
    "ohg_mesh_split": [c_void_p, c_int, P(c_void_p)],
    "ohg_adapt_pass_batch": [c_void_p, P(c_void_p), c_int, P(AdaptOpts), P(PassStats)],
    "ohg_refine_by_size": [c_void_p, P(AdaptOpts), P(c_int)],
    "ohg_coarsen_by_size": [c_void_p, P(AdaptOpts), P(c_int)],
    "ohg_swap_edges": [c_void_p, P(AdaptOpts), P(c_int)],
    "ohg_measure_edges_metric": [c_void_p, c_void_p, c_int, c_void_p],
    "ohg_measure_qualities": [c_void_p, c_void_p, c_int, c_void_p],
    "ohg_get_mident_metrics": [c_void_p, c_void_p, c_int, c_void_p],
    "ohg_refine_qualities": [c_void_p, c_void_p, c_int, c_void_p],
    "ohg_check_collapse_class": [c_void_p, c_void_p, c_int, c_void_p, c_void_p],
    "ohg_check_collapse_exposure": [c_void_p, c_void_p, c_int, c_void_p, c_void_p],
    "ohg_prevent_coarsen_overshoot": [c_void_p, c_double, c_void_p, c_int, c_void_p, c_void_p],
    "ohg_coarsen_qualities": [c_void_p, c_void_p, c_int, c_void_p, c_void_p],
    "ohg_choose_rails": [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
    "ohg_mark_sliver_layers": [c_void_p, c_double, c_int, c_void_p],
    "ohg_swap2d_qualities": [c_void_p, c_double, c_void_p, c_int, c_void_p],
    "ohg_swap3d_qualities": [c_void_p, c_double, c_void_p, c_int, c_void_p, c_void_p],
    "ohg_swap3d_find_loops": [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p],
    "ohg_find_indset": [c_void_p, c_int, c_void_p, c_void_p, c_void_p, P(c_int)],
    "ohg_time_stage": [c_void_p, c_char_p, c_int, P(ctypes.c_float), P(c_double)],
    "ohg_invert_adj": [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p],
    "ohg_reflect_down": [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_void_p,
                         c_void_p, c_void_p, c_int, c_void_p, c_void_p],
    "ohg_find_indset_graph": [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, P(c_int)],
    "ohg_sort_by_keys": [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p],
    "ohg_hilbert_sort": [c_void_p, c_void_p, c_int, c_int, c_void_p],
    "ohg_hilbert_transpose": [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p],
    "ohg_offset_scan": [c_void_p, c_void_p, c_int, c_void_p],
    "ohg_collect_marked": [c_void_p, c_void_p, c_int, c_void_p, c_void_p],
    "ohg_selftest_scan_wait_limit": [c_void_p, c_void_p, c_int, c_void_p],
    "ohg_screen_tet_qualities": [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p],
    "ohg_screen_tet_qualities_face": [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p,
                                      c_void_p, c_void_p],
    "ohg_screen_edge_lengths": [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p],
    "ohg_context_set_screening": [c_void_p, c_int],
    "ohg_context_time_kernels": [c_void_p, c_int],
    "ohg_context_kernel_time": [c_void_p, c_char_p, P(c_double), P(c_double), P(c_int), c_int],
    "ohg_context_screen_counts": [c_void_p, P(ctypes.c_ulonglong), c_int],
    "ohg_offset_scan_noalloc": [c_void_p, c_void_p, c_int, c_void_p],
    "ohg_offset_scan_noalloc_limit": [P(c_int)],
}
_RESTYPE = {"ohg_last_error": c_char_p}

_lib = None


def load():
    """Loads libohg.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} is missing: run omega_h_gb300.build.build() first")
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPE.get(name, c_int)
    _lib = lib
    return lib


def call(name, *args):
    """Calls a C-ABI function, raising OhgError on a nonzero status."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        raise OhgError(rc, lib.ohg_last_error().decode(errors="replace"))
    return rc
