"""ctypes binding of libsamoa_swe.so (the C ABI declared in include/samoa_swe.h).

The library is loaded from this package directory only. If it is missing the
import fails loudly: there is no CPU fallback for the step.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsamoa_swe.so")

SWE_OK = 0
ERRORS = {-1: "SWE_E_INVALID", -2: "SWE_E_CUDA", -3: "SWE_E_NOMESH", -4: "SWE_E_NOMEM", -5: "SWE_E_STATE",
          -6: "SWE_E_DEVICE"}

# every entry point declared in include/samoa_swe.h
EXPORTS = [
    "swe_create", "swe_destroy", "swe_set_stream", "swe_set_params", "swe_mesh_upload", "swe_state_upload",
    "swe_state_download", "swe_state_device", "swe_set_time", "swe_get_time", "swe_traverse",
    "swe_get_refinements", "swe_get_step_count", "swe_synchronize", "swe_last_error", "swe_set_tiling",
    "swe_get_tiling", "swe_mesh_uniform", "swe_mesh_validate", "swe_riemann_batch", "swe_ensemble_mesh_upload",
    "swe_ensemble_set_params", "swe_ensemble_set_time", "swe_ensemble_get_time", "swe_ensemble_get_refinements",
    "swe_traverse_graph", "swe_set_dt_sequence", "swe_step_noalloc", "swe_snapshot_store", "swe_snapshot_restore",
    "swe_sample_gauges", "swe_adjoint_step", "swe_set_arith", "swe_traverse_branches", "swe_step_back",
    "swe_division_check", "swe_step_host", "swe_gauge_gradient",
    "swe_traverse_gauges", "swe_mesh_uniform_vertices", "swe_mesh_build", "swe_mesh_adapt",
    "swe_set_staging", "swe_get_task_counts", "swe_set_cross_pass", "swe_traverse_frozen",
    "swe_set_segment_order", "swe_set_fault_injection",
]


class SweParams(C.Structure):
    _fields_ = [("solver", C.c_int32), ("bc", C.c_int32), ("dry_tolerance", C.c_double), ("courant", C.c_double),
                ("scaling", C.c_double), ("min_depth", C.c_int32), ("max_depth", C.c_int32),
                ("max_time", C.c_double), ("output_time_step", C.c_double)]


class SweError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


_lib = None


def load():
    """Load the library (it must have been built: samoa_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libsamoa_swe.so is not built (run samoa_gb300.build.build()); "
                          "the SWE step has no CPU fallback")
    L = C.CDLL(LIB_PATH)
    P, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int32, C.c_double
    sig = {
        "swe_create": [P, C.c_int],
        "swe_destroy": [P],
        "swe_set_stream": [P, P],
        "swe_set_params": [P, P],
        "swe_mesh_upload": [P, i64, P, P, i64, P, P, i64, P, P],
        "swe_state_upload": [P, P, P, P, P],
        "swe_state_download": [P, P, P, P, P],
        "swe_state_device": [P, P, P, P, P],
        "swe_set_time": [P, dbl, dbl],
        "swe_get_time": [P, P, P, P],
        "swe_traverse": [P, i64],
        "swe_get_refinements": [P, P, P],
        "swe_get_step_count": [P, P],
        "swe_synchronize": [P],
        "swe_last_error": [P, C.c_size_t],
        "swe_set_tiling": [P, i32, i32],
        "swe_get_tiling": [P, P, P],
        "swe_get_task_counts": [P, P, P, P, P],
        "swe_set_cross_pass": [P, i32],
        "swe_set_segment_order": [P, i32],
        "swe_traverse_frozen": [P, i64, i32, P, i64, P, i64, i64, P, P],
        "swe_mesh_uniform": [i32, P, P, P, P, P, P, P, P, P, P],
        "swe_mesh_validate": [i64, P, P, i64, P, P, i64, P, P],
        "swe_riemann_batch": [i32, i64, P, P, P, dbl, P, P],
        "swe_ensemble_mesh_upload": [P, i64, P, P, P, P, P, P, P, P, P],
        "swe_ensemble_set_params": [P, P],
        "swe_ensemble_set_time": [P, P, P],
        "swe_ensemble_get_time": [P, P, P, P],
        "swe_ensemble_get_refinements": [P, P, P],
        "swe_traverse_graph": [P, i64],
        "swe_set_dt_sequence": [P, i64, P],
        "swe_set_fault_injection": [P, i32],
        "swe_step_noalloc": [P, i64, P, P, i64, P, P, i64, P, P, P, P, P, P, P, P, P, P, dbl, i32, P, P, P],
        "swe_snapshot_store": [P, P, P, P, P],
        "swe_snapshot_restore": [P, P, P, P, i64],
        "swe_sample_gauges": [P, i64, P, P],
        "swe_adjoint_step": [P, P, P, P, P, P, P, P, P],
        "swe_traverse_branches": [P, i64, P, i64],
        "swe_step_back": [P],
        "swe_set_arith": [P, i32],
        "swe_division_check": [i64, C.c_uint64, i32, P],
        "swe_step_host": [P, P, P, P, P, P, P, P, P],
        "swe_gauge_gradient": [P, i64, P, i32, i64, P, P, P, P, P, P, P, P, P],
        "swe_traverse_gauges": [P, i64, i64, P, P],
        "swe_mesh_uniform_vertices": [i32, P],
        "swe_mesh_build": [i64, P, P, P, P, P, P, P, P, P, P],
        "swe_set_staging": [P, i32],
        "swe_mesh_adapt": [i64, P, P, P, P, P, P, i64, P, P, P, P, P, P, P],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    _lib = L
    return L


def last_error():
    buf = C.create_string_buffer(512)
    load().swe_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc):
    if rc != SWE_OK:
        raise SweError(rc, last_error())
    return rc
