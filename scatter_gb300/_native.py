"""ctypes binding of ``libscatter_gb300.so`` (declared in include/scatter_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is present, every
entry point raises.  Pointers are passed as integers taken from torch tensors
(``tensor.data_ptr()``); the stream is torch's current CUDA stream.
"""
import ctypes
import os

from . import build as _build

_lib = None

P = ctypes.c_void_p
I = ctypes.c_int
L = ctypes.c_int64
D = ctypes.c_double

# name -> (restype, argtypes); the C-ABI surface, kept in step with include/scatter_gb300.h
SIGNATURES = {
    "sc_version": (I, []),
    "sc_status_string": (ctypes.c_char_p, [I]),
    "sc_last_error": (ctypes.c_char_p, []),
    "sc_element_matrices": (I, [I, I, I, P, P, P, P, P, P, P]),
    "sc_face_matrices": (I, [I, I, I, P, P, P]),
    "sc_node_incidence": (I, [I, I, I, P, P, P, P, P]),
    "sc_node_adjacency": (I, [I, I, P, P, P, P, P, P, P]),
    "sc_scan_work_size": (L, [L]),
    "sc_exclusive_scan_i64": (I, [L, P, P, P, P]),
    "sc_exclusive_scan_i64_noalloc": (I, [L, P, P, P]),
    "sc_csr_pattern": (I, [I, I, P, P, P, P, P, P, P]),
    "sc_assemble_values": (I, [I, I, I, P, P, P, P, P, P, P, P, P, P, P, P, P]),
    "sc_group_rows": (I, [I, I, P, I, P, P, P, P]),
    "sc_lysmer_values": (I, [I, I, P, P, P, P, I, P, P, P, P, P, P, P]),
    "sc_combine": (I, [L, D, P, D, P, D, P, P, P]),
    "sc_csr_row_sums": (I, [L, P, P, I, P, P]),
    "sc_newmark_workspace_doubles": (L, [L, L]),
    "sc_newmark_create": (I, [ctypes.POINTER(P), L, P, P, P, P, P, P, D, D, I, P, P, P, P, L, P]),
    "sc_newmark_set_force": (I, [P, I, P, P, P]),
    "sc_newmark_set_output": (I, [P, I, I, P, P, P, P, L]),
    "sc_newmark_initial_acceleration": (I, [P]),
    "sc_newmark_run": (I, [P, I, I]),
    "sc_newmark_set_predictor": (I, [P, I]),
    "sc_newmark_set_options": (I, [P, I]),
    "sc_newmark_warm_start_status": (I, [P, ctypes.POINTER(I), ctypes.POINTER(L)]),
    "sc_newmark_status": (I, [P, ctypes.POINTER(L), ctypes.POINTER(I)]),
    "sc_newmark_time_spmv": (I, [P, I, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(L)]),
    "sc_newmark_destroy": (I, [P]),
    "sc_rf_modes_model": (I, [ctypes.c_uint64, I, I, I, D, D, D, D, P, P, P]),
    "sc_rf_modes": (I, [ctypes.c_uint64, I, I, D, D, D, P, P]),
    "sc_rf_lognormal": (I, [I, P, I, I, P, D, D, P, P]),
    "sc_batch_create": (I, [ctypes.POINTER(P), P, P, P, P]),
    "sc_batch_config": (I, [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(ctypes.c_float),
                            ctypes.POINTER(I)]),
    "sc_batch_set_hex8_grid": (I, [P, I, P, P]),
    "sc_batch_set_shape": (I, [P, I, I]),
    "sc_batch_set_grid_shape": (I, [P, I, I]),
    "sc_batch_set_node_shape": (I, [P, I, I]),
    "sc_batch_set_node_shape_budget": (I, [P, I, I, I]),
    "sc_batch_set_hex8_columns": (I, [P, I, I, P, P]),
    "sc_batch_set_tc_shape": (I, [P, I]),
    "sc_batch_status": (I, [P]),
    "sc_batch_set_force": (I, [P, I, P, P, P]),
    "sc_batch_set_output": (I, [P, I, I, P, P, L]),
    "sc_batch_run": (I, [P, I, I]),
    "sc_batch_destroy": (I, [P]),
    "sc_nb_workspace_bytes": (L, [I, I, L]),
    "sc_nb_create": (I, [ctypes.POINTER(P), I, I, P, P, P, L, P, P, P, P, P, L, P, P, P, D, D, D, D, I, I, P, P, P, P,
                         L, P]),
    "sc_nb_set_options": (I, [P, I]),
    "sc_nb_warm_start_status": (I, [P, ctypes.POINTER(I), ctypes.POINTER(L)]),
    "sc_nb_status_to": (I, [P, P]),
    "sc_newmark_status_to": (I, [P, P]),
    "sc_nb_a32_status": (I, [P, ctypes.POINTER(L), ctypes.POINTER(L), ctypes.POINTER(L),
                             ctypes.POINTER(ctypes.c_double)]),
    "sc_nb_residual_fp64": (I, [P, ctypes.POINTER(I)]),
    "sc_nb_set_predictor": (I, [P, I]),
    "sc_nb_set_force": (I, [P, I, P, P, P]),
    "sc_nb_set_output": (I, [P, I, I, P, P, P, P, L]),
    "sc_nb_run": (I, [P, I, I]),
    "sc_nb_status": (I, [P, ctypes.POINTER(L), ctypes.POINTER(I), ctypes.POINTER(I)]),
    "sc_nb_time_spmv": (I, [P, I, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(L)]),
    "sc_nb_time_spmv_a32": (I, [P, I, I, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(L)]),
    "sc_nb_explicit_run": (I, [P, I, I]),
    "sc_nb_set_lumped_mass": (I, [P, P]),
    "sc_nb_time_explicit": (I, [P, I, ctypes.POINTER(ctypes.c_float)]),
    "sc_nb_tune_explicit": (I, [P, I, ctypes.POINTER(I), ctypes.POINTER(ctypes.c_float)]),
    "sc_nb_apply": (I, [P, I, P, P]),
    "sc_nb_adjoint": (I, [P, P, ctypes.POINTER(D), P, P]),
    "sc_nb_adjoint_timings": (I, [P, ctypes.POINTER(ctypes.c_float)]),
    "sc_nb_destroy": (I, [P]),
}

ELEMENT_CODES = {"hexa8": 0, "hexa20": 1, "tetra4": 2, "tetra10": 3, "quad4": 4, "quad8": 5, "tri3": 6, "tri6": 7}


class ScatterGpuError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, fn, code, text, detail):
        super().__init__(f"{fn} failed: status {code} ({text}){': ' + detail if detail else ''}")
        self.code = code


def library_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load the shared library (building it first when asked and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"scatter_gb300 CUDA library not built ({path}); run scatter_gb300.build.build()")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def call(name, *args):
    """Call entry point ``name``; raise ScatterGpuError on a non-zero status."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        text = lib.sc_status_string(rc).decode()
        detail = lib.sc_last_error().decode()
        raise ScatterGpuError(name, rc, text, detail if rc == 5 else "")
    return rc


def value(name, *args):
    return getattr(load(), name)(*args)
