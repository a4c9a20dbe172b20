"""GB300-native speculative segmented-sum CSR SpMV (y = A.x) for one sm_103a GPU.

Drop-in for the host API of weifengliu-ssslab/Benchmark_SpMV_using_CSR
(``bhsparse_spmv_cuda``: init_platform / prepare_mem / run_benchmark / get_y /
free_platform / free_mem), backed by a C ABI (include/spmv_gb300.h) and hand-written
CUDA kernels in ``csrc/``.
"""
from .api import (  # noqa: F401
    BHSPARSE_CUDA_ERROR, BHSPARSE_DEVICE_CHECK_FAILED, BHSPARSE_INVALID_ARGUMENT,
    BHSPARSE_INVALID_CSR, BHSPARSE_NOALLOC_TOO_LARGE, BHSPARSE_NOT_PREPARED, BHSPARSE_OUT_OF_MEMORY,
    BHSPARSE_SUCCESS, SCHEDULE_CALLER, SCHEDULE_DEFAULT, SCHEDULE_LEARNED, SCHEDULE_SWEEP,
    BHSPARSE_UNSUPPORTED_VALUE_TYPE, DEFAULT_CONFIG, VALUE_F32, VALUE_F64, VALUE_MIXED_BF16,
    VALUE_MIXED_F32, VALUE_NAMES, BhsparseSpmvCuda, Plan, SpmvError, bitflags, host_dtype,
    partition, validate_csr, version)
from .build import LIB_PATH, build  # noqa: F401
