/*
 * spmv_mtx.h -- Matrix Market coordinate files to CSR (host code, C ABI).
 *
 * Replaces the benchmark driver's matrix loading, spmv_cuda/main.cu:570-733 (the NIST reader
 * calls mm_read_banner, spmv_cuda/mmio.h:249, and mm_read_mtx_crd_size, mmio.h:334, then a
 * counting sort of the entries by row), with the same result:
 *   - fields real (strtod), integer (read as int) and pattern (value 1.0); complex is refused;
 *   - 1-based indices made 0-based;
 *   - symmetric and hermitian files have every off-diagonal entry (i, j, v) mirrored to
 *     (j, i, v); skew-symmetric files are loaded as stored, unmirrored, as the reference does
 *     (main.cu:608-612 tests symmetric and hermitian only);
 *   - rows are filled in file order (a stable counting sort, main.cu:668-716), each mirrored
 *     entry placed right after the entry that produced it; columns are not sorted in a row.
 * Unlike the reference, indices are range-checked, a truncated entry list is an error and
 * array (dense) storage is refused instead of being misread.  The driver's value overwrite
 * with rand()%10 (main.cu:735-739) is not part of loading (see bhsp_gen_uniform_int).
 *
 * Status codes: the reference's own for its failure points, then the added checks.
 */
#ifndef SPMV_MTX_H
#define SPMV_MTX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    BHSP_MTX_OK = 0,
    BHSP_MTX_OPEN_FAILED = -1,    /* fopen failed (main.cu:582-583) */
    BHSP_MTX_BAD_BANNER = -2,     /* mm_read_banner failed (main.cu:585-589) */
    BHSP_MTX_COMPLEX = -3,        /* complex field (main.cu:591-595) */
    BHSP_MTX_BAD_SIZE = -4,       /* mm_read_mtx_crd_size failed (main.cu:602-604) */
    BHSP_MTX_UNSUPPORTED = -5,    /* array (dense) storage */
    BHSP_MTX_BAD_ENTRY = -6,      /* index out of range, unparsable or missing entry */
    BHSP_MTX_TOO_LARGE = -7,      /* more than INT32_MAX non-zeros after mirroring */
    BHSP_MTX_NO_MEMORY = -8
};

/* field: 0 real, 1 integer, 2 pattern; symmetry: 0 general, 1 symmetric, 2 hermitian,
 * 3 skew-symmetric. */
typedef struct bhsp_mtx_info {
    int m, n;
    int nnz_file; /* entries listed in the file */
    int nnz;      /* entries in the CSR (after mirroring) */
    int field;
    int symmetry;
} bhsp_mtx_info;

typedef struct bhsp_mtx bhsp_mtx;

/* Load a file into a host CSR owned by *out (freed by bhsp_mtx_free).  On failure *out is
 * NULL and the status says why. */
int bhsp_mtx_load(const char* path, bhsp_mtx** out);
int bhsp_mtx_get_info(const bhsp_mtx* a, bhsp_mtx_info* info);
const int* bhsp_mtx_row_ptr(const bhsp_mtx* a);   /* [m + 1] */
const int* bhsp_mtx_col_idx(const bhsp_mtx* a);   /* [nnz] */
const double* bhsp_mtx_val(const bhsp_mtx* a);    /* [nnz] */
void bhsp_mtx_free(bhsp_mtx* a);

#ifdef __cplusplus
}
#endif

#endif /* SPMV_MTX_H */
