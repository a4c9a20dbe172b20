"""ctypes binding of ``libspmv_gb300.so`` (the C ABI of include/spmv_gb300.h,
include/spmv_gen.h, include/spmv_mtx.h and include/spmv_compare.h).

The library is built in-tree by :mod:`benchmark_spmv_using_csr_gb300.build`.  If it
is missing this module raises at load time: there is no fallback path.
"""
from __future__ import annotations

import ctypes
import os
import threading

from .build import LIB_PATH

_lock = threading.Lock()
_lib = None

c_int, c_int64, c_uint64, c_size_t, c_double = (ctypes.c_int, ctypes.c_int64, ctypes.c_uint64,
                                                 ctypes.c_size_t, ctypes.c_double)
c_void_p, c_char_p = ctypes.c_void_p, ctypes.c_char_p
P_int = ctypes.POINTER(ctypes.c_int)
P_void = ctypes.POINTER(ctypes.c_void_p)

# name -> (restype, argtypes); every entry is a symbol declared in include/*.h
SIGNATURES = {
    # handle API (spmv_gb300.h)
    "bhsp_create": (c_int, [P_void, c_int]),
    "bhsp_destroy": (None, [c_void_p]),
    "bhsp_init_platform": (c_int, [c_void_p]),
    "bhsp_free_platform": (c_int, [c_void_p]),
    "bhsp_prepare_mem": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                 c_void_p, c_void_p]),
    "bhsp_run_benchmark": (c_int, [c_void_p]),
    "bhsp_get_y": (c_int, [c_void_p]),
    "bhsp_free_mem": (c_int, [c_void_p]),
    "bhsp_last_error": (c_char_p, [c_void_p]),
    "bhsp_set_device": (c_int, [c_void_p, c_int]),
    "bhsp_set_config": (c_int, [c_void_p, c_int, c_int, c_int, c_int]),
    "bhsp_set_tuner": (c_int, [c_void_p, c_char_p]),
    "bhsp_get_schedule_source": (c_int, [c_void_p, P_int, ctypes.POINTER(ctypes.c_float)]),
    "bhsp_get_config": (c_int, [c_void_p, P_int, P_int, P_int, P_int]),
    "bhsp_set_x": (c_int, [c_void_p, c_void_p]),
    "bhsp_run_stream": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "bhsp_run_async": (c_int, [c_void_p, c_void_p]),
    "bhsp_check": (c_int, [c_void_p]),
    "bhsp_run_phase": (c_int, [c_void_p, c_void_p, c_int]),
    "bhsp_device_buffers": (c_int, [c_void_p, P_void, P_void, P_void, P_void, P_void]),
    "bhsp_device_bytes": (c_size_t, [c_void_p]),
    # plan API
    "bhsp_plan_create": (c_int, [P_void, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int,
                                 c_int, c_int, c_int, c_void_p]),
    "bhsp_plan_execute": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "bhsp_plan_execute_phase": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int]),
    "bhsp_plan_check": (c_int, [c_void_p, c_void_p]),
    "bhsp_plan_launches": (c_int, [c_void_p]),
    "bhsp_plan_tiles": (c_int, [c_void_p, P_void, P_int, P_int]),
    "bhsp_plan_chunk_form": (c_int, [c_void_p, P_int, P_int]),
    "bhsp_plan_gather_path": (c_int, [c_void_p, P_int, P_int, P_int]),
    "bhsp_plan_set_variant": (c_int, [c_void_p, c_int, c_int]),
    "bhsp_plan_set_grid": (c_int, [c_void_p, c_int]),
    "bhsp_plan_last_error": (c_char_p, [c_void_p]),
    "bhsp_plan_destroy": (None, [c_void_p]),
    # partition primitives
    "bhsp_partition": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p]),
    "bhsp_bitflags": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "bhsp_validate_csr": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p]),
    "bhsp_version": (c_char_p, []),
    # batched form
    "bhsp_batch_create": (c_int, [P_void, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int,
                                  c_int, c_int, c_int, c_void_p]),
    "bhsp_batch_execute": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "bhsp_batch_check": (c_int, [c_void_p, c_void_p]),
    "bhsp_batch_info": (c_int, [c_void_p, P_int, P_int, P_int, P_int]),
    "bhsp_batch_last_error": (c_char_p, [c_void_p]),
    "bhsp_batch_variant": (c_int, [c_void_p, P_int, P_int]),
    "bhsp_batch_set_variant": (c_int, [c_void_p, c_int, c_int]),
    "bhsp_batch_tune_num_candidates": (c_int, []),
    "bhsp_batch_tune_candidate": (c_int, [c_int, P_int, P_int, P_int]),
    "bhsp_batch_autotune": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int,
                                    c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, P_int,
                                    c_void_p]),
    "bhsp_batch_destroy": (None, [c_void_p]),
    # learned tuner network
    "bhsp_mlp_create": (c_int, [P_void, c_int, c_int, c_int, c_int]),
    "bhsp_mlp_num_params": (c_size_t, [c_void_p]),
    "bhsp_mlp_set_params": (c_int, [c_void_p, c_void_p, c_size_t]),
    "bhsp_mlp_get_params": (c_int, [c_void_p, c_void_p, c_size_t]),
    "bhsp_mlp_set_normalization": (c_int, [c_void_p, c_void_p, c_void_p]),
    "bhsp_mlp_forward": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "bhsp_mlp_gradients": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p,
                                   c_void_p]),
    "bhsp_mlp_train_step": (c_int, [c_void_p, c_void_p, c_void_p, c_int, ctypes.c_float,
                                    ctypes.c_float, c_void_p, c_void_p]),
    "bhsp_mlp_destroy": (None, [c_void_p]),
    # tuning
    "bhsp_tune_num_candidates": (c_int, []),
    "bhsp_tune_candidate": (c_int, [c_int, P_int, P_int, P_int, P_int]),
    "bhsp_autotune": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                              c_void_p, c_int, c_int, c_void_p, P_int, c_void_p]),
    "bhsp_row_features": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p]),
    "bhsp_choose_schedule": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_void_p, c_char_p, P_int, P_int, P_int, P_int,
                                     P_int, ctypes.POINTER(ctypes.c_float), c_void_p]),
    "bhsp_features_from_counts": (None, [c_int, c_int, c_void_p, c_void_p]),
    "bhsp_spmv_f64_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                      c_int, c_int, c_int, c_void_p]),
    # generators (spmv_gen.h)
    "bhsp_gen_uniform": (c_int, [c_int64, c_uint64, c_double, c_double, c_void_p]),
    "bhsp_gen_uniform_int": (c_int, [c_int64, c_uint64, c_int, c_void_p]),
    "bhsp_gen_stencil2d_nnz": (c_int64, [c_int, c_int]),
    "bhsp_gen_stencil2d": (c_int, [c_int, c_int, c_double, c_uint64, c_void_p, c_void_p, c_void_p]),
    "bhsp_gen_stencil3d_nnz": (c_int64, [c_int, c_int, c_int]),
    "bhsp_gen_stencil3d": (c_int, [c_int, c_int, c_int, c_double, c_uint64, c_void_p, c_void_p,
                                   c_void_p]),
    "bhsp_gen_powerlaw_rows": (c_int64, [c_int, c_double, c_double, c_int, c_double, c_uint64,
                                         c_void_p]),
    "bhsp_gen_density_rows": (c_int64, [c_int, c_int, c_double, c_uint64, c_void_p]),
    "bhsp_gen_mixed_rows": (c_int64, [c_int, c_int, c_int, c_double, c_double, c_uint64,
                                      c_void_p]),
    "bhsp_gen_random_fill": (c_int, [c_int, c_int, c_void_p, c_double, c_double, c_uint64,
                                     c_void_p, c_void_p]),
    "bhsp_gen_blockdiag_rows": (c_int64, [c_int, c_int, c_int, c_void_p]),
    "bhsp_gen_blockdiag_fill": (c_int, [c_int, c_int, c_int, c_double, c_double, c_uint64,
                                        c_void_p, c_void_p, c_void_p]),
    # Matrix Market loading (spmv_mtx.h)
    "bhsp_mtx_load": (c_int, [c_char_p, P_void]),
    "bhsp_mtx_get_info": (c_int, [c_void_p, c_void_p]),
    "bhsp_mtx_row_ptr": (c_void_p, [c_void_p]),
    "bhsp_mtx_col_idx": (c_void_p, [c_void_p]),
    "bhsp_mtx_val": (c_void_p, [c_void_p]),
    "bhsp_mtx_free": (None, [c_void_p]),
    # comparators (spmv_compare.h)
    "bhsp_csr_vector_width": (c_int, [c_int, c_int]),
    "bhsp_csr_vector": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_int, c_void_p]),
    "bhsp_cusparse_create": (c_int, [P_void, c_int, c_int, c_int, c_int, c_void_p, c_void_p,
                                     c_void_p, c_void_p, c_void_p, c_void_p]),
    "bhsp_cusparse_run": (c_int, [c_void_p]),
    "bhsp_cusparse_destroy": (None, [c_void_p]),
}


def lib() -> ctypes.CDLL:
    """Load the library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with "
                    "`python -m benchmark_spmv_using_csr_gb300.build` (no fallback path exists)")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
        return _lib
