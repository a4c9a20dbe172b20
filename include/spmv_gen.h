/*
 * spmv_gen.h -- seeded synthetic CSR matrices and vectors (host code, C ABI).
 *
 * These replace the benchmark driver's matrix set-up (spmv_cuda/main.cu:570-743: a Matrix
 * Market file converted to CSR, then rand()%10 values and x seeded from the clock) with
 * reproducible generators for the benchmark workloads.  Every random draw is a
 * counter-based hash of (seed, index), so the output does not depend on the number of
 * host threads.  Columns are sorted and distinct within each row; indices are int32.
 * All functions return 0 on success and a negative value on bad arguments.
 */
#ifndef SPMV_GEN_H
#define SPMV_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* out[i] = uniform in [lo, hi) drawn from (seed, i), i = 0..count-1. */
int bhsp_gen_uniform(int64_t count, uint64_t seed, double lo, double hi, double* out);
/* out[i] = integer uniform in [0, modulus) from (seed, i), stored as double (the
 * reference's rand()%10 data, spmv_cuda/main.cu:736-743, made reproducible). */
int bhsp_gen_uniform_int(int64_t count, uint64_t seed, int modulus, double* out);

/* 2D 5-point Laplacian on an nx x ny grid (m = nx*ny): 4 on the diagonal, -1 off it, each
 * plus uniform[-noise, noise].  nnz = m + 2(nx-1)ny + 2nx(ny-1). */
int64_t bhsp_gen_stencil2d_nnz(int nx, int ny);
int bhsp_gen_stencil2d(int nx, int ny, double noise, uint64_t seed, int* row_ptr, int* col,
                       double* val);

/* 3D 27-point stencil on an nx x ny x nz grid: weight 26 on the diagonal and -1 for the 26
 * neighbours, each times (1 + uniform[-noise, noise]).  nnz = (3nx-2)(3ny-2)(3nz-2). */
int64_t bhsp_gen_stencil3d_nnz(int nx, int ny, int nz);
int bhsp_gen_stencil3d(int nx, int ny, int nz, double noise, uint64_t seed, int* row_ptr,
                       int* col, double* val);

/* Power-law row lengths: L = floor(xmin * U^(-1/(alpha-1))) clipped to [1, max_len] (a
 * Zipf(alpha) tail), then a fraction empty_frac of rows forced empty.  Fills row_ptr[0..m]
 * and returns nnz (-1 if it would exceed INT32_MAX). */
int64_t bhsp_gen_powerlaw_rows(int m, double alpha, double xmin, int max_len, double empty_frac,
                               uint64_t seed, int* row_ptr);
/* Uniform-density row lengths: Poisson(n * density) per row, clipped to n. */
int64_t bhsp_gen_density_rows(int m, int n, double density, uint64_t seed, int* row_ptr);
/* Row lengths of a matrix with one dense row (row `dense_row`, all n columns) and
 * Poisson(mean_len) elsewhere; with empty_frac of the other rows forced empty. */
int64_t bhsp_gen_mixed_rows(int m, int n, int dense_row, double mean_len, double empty_frac,
                            uint64_t seed, int* row_ptr);
/* Given row_ptr, fill each row with distinct sorted uniform random columns in [0, n) and
 * values uniform in [lo, hi). */
int bhsp_gen_random_fill(int m, int n, const int* row_ptr, double lo, double hi, uint64_t seed,
                         int* col, double* val);

/* Block-diagonal matrix of dense bs x bs blocks (the last block clipped to m, n). */
int64_t bhsp_gen_blockdiag_rows(int m, int n, int bs, int* row_ptr);
int bhsp_gen_blockdiag_fill(int m, int n, int bs, double lo, double hi, uint64_t seed,
                            const int* row_ptr, int* col, double* val);

#ifdef __cplusplus
}
#endif
#endif /* SPMV_GEN_H */
