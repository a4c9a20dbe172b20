/*
 * spmv_compare.h -- comparators timed beside the tile kernel (C ABI, device buffers).
 *
 * The reference driver times two other GPU SpMVs on the same matrix:
 *   - the CSR-vector kernel of CUSP v0.4.0 (spmv_cuda/kernels_cuda.h:273-342), one vector of
 *     2, 4, 8, 16 or 32 threads per row, the width picked from nnz / m
 *     (spmv_cuda/main.cu:236-286): here a kernel of this library with the same schedule and
 *     a shuffle reduction;
 *   - cuSPARSE's CSR SpMV, cusparse{S,D}csrmv (spmv_cuda/main.cu:49-183), which CUDA 12
 *     removed: here its successor, the generic cusparseSpMV with CUSPARSE_SPMV_CSR_ALG1,
 *     loaded at run time (no link-time dependency; status BHSP_CMP_UNAVAILABLE when the
 *     library cannot be loaded).
 * Both compute y = A.x (alpha = 1, beta = 0) in the value type (F64 or F32 of spmv_gb300.h)
 * and are comparators only: the product path is spmv_gb300.h.
 */
#ifndef SPMV_COMPARE_H
#define SPMV_COMPARE_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    BHSP_CMP_OK = 0,
    BHSP_CMP_INVALID_ARGUMENT = -1,
    BHSP_CMP_CUDA_ERROR = -2,
    BHSP_CMP_UNAVAILABLE = -3, /* the cuSPARSE library could not be loaded */
    BHSP_CMP_LIBRARY_ERROR = -4
};

/* Vector width the reference picks for a matrix: 2, 4, 8, 16 or 32 from nnz / m. */
int bhsp_csr_vector_width(int m, int nnz);
/* CSR-vector SpMV; threads_per_vector 0 picks bhsp_csr_vector_width.  Asynchronous on
 * `stream` (a cudaStream_t, NULL = default stream). */
int bhsp_csr_vector(int value_type, int m, const int* d_row_ptr, const int* d_col_idx,
                    const void* d_val, const void* d_x, void* d_y, int threads_per_vector,
                    void* stream);

/* cuSPARSE generic SpMV bound to fixed device buffers (a handle, the matrix and vector
 * descriptors and the work buffer are set up once). */
typedef struct bhsp_cusparse bhsp_cusparse;
int bhsp_cusparse_create(bhsp_cusparse** out, int value_type, int m, int n, int nnz,
                         const int* d_row_ptr, const int* d_col_idx, const void* d_val,
                         const void* d_x, void* d_y, void* stream);
int bhsp_cusparse_run(bhsp_cusparse* c);
void bhsp_cusparse_destroy(bhsp_cusparse* c);

#ifdef __cplusplus
}
#endif

#endif /* SPMV_COMPARE_H */
