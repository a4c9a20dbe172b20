/*
 * oracle.c -- CPU oracle for the speculative segmented-sum CSR SpMV.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library calls, links or
 * loads this file: it is the checker that the parity tests, the smoke check
 * and the benchmark's CPU-baseline leg compare the CUDA path against.
 *
 * Contents (every function cites the reference code it restates; paths are
 * relative to the reference project, weifengliu-ssslab/Benchmark_SpMV_using_CSR):
 *
 *   oracle_search_right     binary_search_right_boundary_kernel, spmv_cuda/utils_cuda.h:6-31
 *   oracle_partition        per-tile row boundaries, spmv_cuda/kernels_cuda.h:39-53, plus the
 *                           dirty (empty-row) test of kernels_cuda.h:114-145, packed CSR5-style
 *                           as tile_ptr[t] = row | dirty<<31
 *   oracle_bitflags         raw bit-flag words, spmv_cuda/kernels_cuda.h:114-148 (before the
 *                           lane-0 head bit is forced at :172)
 *   oracle_bhsparse_{f64,f32}
 *                           a lane-by-lane simulation of SpMV_kernel
 *                           (spmv_cuda/kernels_cuda.h:7-269) followed by the host calibration
 *                           of run_benchmark (spmv_cuda/bhsparse_spmv_cuda.h:166-222), for the
 *                           first call with y zeroed, as spmv_cuda/main.cu:769-806 checks it.
 *                           The out-of-range read of row_ptr[m+1] that the host fix-up makes
 *                           when the last tile is dirty (bhsparse_spmv_cuda.h:199-216) is
 *                           guarded here and reported through a flag.
 *   oracle_csr_serial_{f64,f32}
 *                           the serial CPU loop, spmv_cuda/main.cu:755-761
 *   oracle_csr_omp_{f64,f32}
 *                           the OpenMP loop, spmv_cuda/main.cu:370-393
 *   oracle_csr_dot2         FP64 compensated row dot products (Ogita, Rump and Oishi, "Accurate
 *                           sum and dot product", SIAM J. Sci. Comput. 26(6), 2005, Algorithm
 *                           Dot2): the high-accuracy reference y* for error statements.
 *   oracle_csr_absrow       (|A|.|x|)_i, the scale of the componentwise tolerance.
 *
 * Build with -ffp-contract=off: the reference rounds every product before it is
 * added (products are parked in shared memory, kernels_cuda.h:161), and the
 * restatement must not be fused into FMAs by the host compiler (aarch64 gcc
 * contracts by default).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_LANES 32 /* THREADBUNCH, spmv_cuda/common.h:39 */

/* spmv_cuda/utils_cuda.h:6-31: first index i in [0,size) with row_ptr[i] > key
 * (returns size when there is none). */
int oracle_search_right(const int *row_ptr, int key, int size)
{
    int start = 0, stop = size - 1;
    while (stop >= start) {
        int median = (stop + start) / 2;
        if (key >= row_ptr[median])
            start = median + 1;
        else
            stop = median - 1;
    }
    return start;
}

/* Number of tiles of ps non-zeros: spmv_cuda/bhsparse_spmv_cuda.h:327. */
int oracle_num_tiles(int nnz, int ps)
{
    return (int)(((long long)nnz + ps - 1) / ps);
}

/* Row of tile boundary t: kernels_cuda.h:45-48 (boundary clamped to nnz). */
static int tile_row(const int *row_ptr, int m, int nnz, int ps, long long t)
{
    long long b = t * (long long)ps;
    if (b > nnz)
        b = nnz;
    return oracle_search_right(row_ptr, (int)b, m + 1) - 1;
}

/* Dirty test of one tile whose row span is [lo, hi]: kernels_cuda.h:119-145.
 * A fast-track tile (lo == hi) is never dirty (it `continue`s at :111). */
static int tile_dirty(const int *row_ptr, int m, int lo, int hi)
{
    if (lo == hi)
        return 0;
    int stop = hi == m ? m - 1 : hi;
    for (int r = lo; r <= stop; r++)
        if (row_ptr[r] == row_ptr[r + 1])
            return 1;
    return 0;
}

/* tile_ptr[t], t = 0..ntiles: the row found for boundary t*ps, with bit 31 set
 * when tile t is dirty.  tile_ptr[ntiles] never carries the bit. */
void oracle_partition(const int *row_ptr, int m, int nnz, int ps, uint32_t *tile_ptr)
{
    int nt = oracle_num_tiles(nnz, ps);
    for (int t = 0; t <= nt; t++)
        tile_ptr[t] = (uint32_t)tile_row(row_ptr, m, nnz, ps, t);
    for (int t = 0; t < nt; t++)
        if (tile_dirty(row_ptr, m, (int)tile_ptr[t], (int)(tile_ptr[t + 1] & 0x7fffffffu)))
            tile_ptr[t] |= 0x80000000u;
}

/* Raw bit-flag words of one tile (lanes words, the top s bits of each used):
 * kernels_cuda.h:116-143.  For every non-empty row r of the span, offset
 * o = row_ptr[r] - tile_start; 0 <= o < lanes*s sets bit 31 - o%s of word o/s;
 * o >= lanes*s is a no-op (:132-133). */
static void tile_bitflags(const int *row_ptr, int m, int lanes, int s, long long tile_start,
                          int lo, int hi, uint32_t *words)
{
    memset(words, 0, sizeof(uint32_t) * lanes);
    int stop = hi == m ? m - 1 : hi;
    for (int r = lo; r <= stop; r++) {
        if (row_ptr[r] == row_ptr[r + 1])
            continue;
        long long off = (long long)row_ptr[r] - tile_start;
        if (off < 0)
            continue;
        long long slice = off / s;
        if (slice < lanes)
            words[slice] |= 1u << (31 - (int)(off % s));
    }
}

/* Bit-flag words of every tile, lanes words per tile, geometry lanes x s
 * (the reference geometry is 32 x SEG_H).  tile_ptr is oracle_partition's
 * output for ps = lanes*s. */
void oracle_bitflags(const int *row_ptr, int m, int nnz, int lanes, int s,
                     const uint32_t *tile_ptr, uint32_t *words)
{
    int ps = lanes * s;
    int nt = oracle_num_tiles(nnz, ps);
    for (int t = 0; t < nt; t++)
        tile_bitflags(row_ptr, m, lanes, s, (long long)t * ps, (int)(tile_ptr[t] & 0x7fffffffu),
                      (int)(tile_ptr[t + 1] & 0x7fffffffu), words + (size_t)t * lanes);
}

/* ------------------------------------------------------------------------- */
/* Lane-by-lane simulation of SpMV_kernel + run_benchmark's host calibration. */
/* One body, instantiated for double and float (USE_DOUBLE, common.h:27-31).   */
/* ------------------------------------------------------------------------- */

#define ORACLE_KERNEL(NAME, VT)                                                                \
int NAME(int m, int n, int nnz, const int *row_ptr, const int *col, const VT *val,             \
         const VT *x, int seg_h, int step, VT *y, int *sync_idx, VT *sync_val,                 \
         int *spec, int *ndirty)                                                               \
{                                                                                              \
    (void)n;                                                                                   \
    const int L = ORACLE_LANES;                                                                \
    if (seg_h < 1 || seg_h > 32 || (L % seg_h) != 0 || step < 1 || step >= L)                  \
        return -1;                                                                             \
    const int ps = L * seg_h;                          /* bhsparse_spmv_cuda.h:326 */         \
    const int pnum = oracle_num_tiles(nnz, ps);        /* :327 */                             \
    const int nwarps = (pnum + step - 1) / step;       /* :328 */                             \
    VT *inter = (VT *)malloc(sizeof(VT) * seg_h * (L + 1));                                    \
    int *bs = (int *)malloc(sizeof(int) * (step + 1));                                         \
    uint32_t bfw[ORACLE_LANES];                                                                \
    int lstart[ORACLE_LANES], lstop[ORACLE_LANES], segn[ORACLE_LANES];                         \
    unsigned char present[ORACLE_LANES + 1];                                                   \
    VT head[ORACLE_LANES], fs[ORACLE_LANES], tmp[ORACLE_LANES];                                \
    int nd = 0;                                                                                \
    for (int w = 0; w < nwarps; w++) {                                                         \
        const long long poff = (long long)w * step * ps;               /* :39 */              \
        for (int i = 0; i <= step; i++) {                              /* :43-49 */           \
            long long b = poff + (long long)i * ps;                                            \
            if (b > nnz) b = nnz;                                                              \
            bs[i] = oracle_search_right(row_ptr, (int)b, m + 1) - 1;                           \
        }                                                                                      \
        int bs_stop = bs[0];                                                                   \
        const int tb_start = bs_stop;                                  /* :53 */              \
        VT s_tail = 0;                                                 /* :58 */              \
        present[L] = 1;                                                /* :57 */              \
        for (int i = 0; i < step; i++) {                                                       \
            if (i + w * step >= pnum) break;                           /* :67-68 */           \
            int dirty = 0;                                                                     \
            int bs_start = bs_stop;                                                            \
            bs_stop = bs[i + 1];                                                               \
            const long long tstart = poff + (long long)i * ps;                                 \
            if (bs_start == bs_stop) {                                 /* fast track :79 */   \
                for (int l = 0; l < L; l++) {                                                  \
                    VT f = 0;                                                                  \
                    for (int j = 0; j < seg_h; j++) {                                          \
                        long long e = tstart + (long long)j * L + l;                           \
                        VT p = e < nnz ? val[e] * x[col[e]] : (VT)0;                           \
                        f += p;                                        /* :88 */              \
                    }                                                                          \
                    fs[l] = f;                                                                 \
                }                                                                              \
                for (int mask = L / 2; mask > 0; mask >>= 1) {         /* utils_cuda.h:69-78 */\
                    VT nf[ORACLE_LANES];                                                       \
                    for (int l = 0; l < L; l++) nf[l] = fs[l] + fs[l ^ mask];                  \
                    memcpy(fs, nf, sizeof(nf));                                                \
                }                                                                              \
                VT fsum = ((long long)row_ptr[bs_start] == tstart) ? fs[0] : s_tail + fs[0];   \
                if (bs_start == tb_start) { sync_idx[w] = bs_start; sync_val[w] = fsum; }      \
                else y[bs_start] = fsum;                                                       \
                s_tail = fsum;                                                                 \
                continue;                                                                      \
            }                                                                                  \
            /* step 2: bit flags (:116-148) */                                                 \
            tile_bitflags(row_ptr, m, L, seg_h, tstart, bs_start, bs_stop, bfw);               \
            dirty = tile_dirty(row_ptr, m, bs_start, bs_stop);                                 \
            /* step 3: products, transposed so lane l owns tile slots [l*seg_h,(l+1)*seg_h) */ \
            for (int q = 0; q < ps; q++) {                             /* :152-162 */         \
                long long e = tstart + q;                                                      \
                inter[(q % seg_h) * (L + 1) + q / seg_h] = e < nnz ? val[e] * x[col[e]] : (VT)0;\
            }                                                                                  \
            if (!((bfw[0] >> 31) & 1u)) inter[0] = inter[0] + s_tail;  /* :165-170 */         \
            bfw[0] |= 0x80000000u;                                     /* :172 */             \
            /* step 4-0: per-lane segmented reduction (:177-199) */                            \
            for (int l = 0; l < L; l++) {                                                      \
                uint32_t bf = bfw[l];                                                          \
                int bit = (bf >> 31) & 1u;                                                     \
                lstart[l] = !bit;                                                              \
                lstop[l] = 0;                                                                  \
                VT sum = inter[l];                                                             \
                int pr = (l == 0) | bit;                                                       \
                for (int j = 1; j < seg_h; j++) {                                              \
                    bit = (bf >> (31 - j)) & 1u;                                               \
                    if (bit) { inter[lstop[l] * (L + 1) + l] = sum; sum = 0; lstop[l]++; }     \
                    sum += inter[j * (L + 1) + l];                                             \
                    pr |= bit;                                                                 \
                }                                                                              \
                inter[lstop[l] * (L + 1) + l] = sum;                                           \
                present[l] = (unsigned char)pr;                                                \
                int c = lstop[l] - lstart[l] + pr;                     /* :201-202 */         \
                segn[l] = c > 0 ? c : 0;                                                       \
            }                                                                                  \
            /* exclusive scan of segment counts (:205-207) */                                  \
            { int run = 0; for (int l = 0; l < L; l++) { int c = segn[l]; segn[l] = run; run += c; } }\
            /* head-less partial of lane l+1, pulled down by one lane (:210-216) */            \
            for (int l = 0; l < L; l++) head[l] = (VT)lstart[l] * inter[l];                  \
            for (int l = 0; l < L; l++) tmp[l] = (l == L - 1) ? (VT)0 : head[l + 1];           \
            /* step 4-1: spanning segments (:219-230) */                                       \
            for (int l = 0; l < L; l++) {                                                      \
                VT t = 0;                                                                      \
                if (present[l]) {                                                              \
                    t = tmp[l];                                                                \
                    int id = l + 1;                                                            \
                    while (!present[id]) { t += tmp[id]; id++; }                               \
                }                                                                              \
                inter[lstop[l] * (L + 1) + l] += t;                    /* :235 */             \
            }                                                                                  \
            /* steps 5-6: compacted scatter, synchronizer, carry (:239-257) */                 \
            for (int l = 0; l < L; l++) {                                                      \
                int loc = bs_start + segn[l];                                                  \
                for (int j = lstart[l]; j <= lstop[l]; j++) {                                  \
                    VT v = inter[j * (L + 1) + l];                                             \
                    if (loc == tb_start) { sync_idx[w] = tb_start; sync_val[w] = v; }          \
                    else y[loc] = v;                                                           \
                    if (loc == bs_stop) s_tail = v;                                            \
                    loc++;                                                                     \
                }                                                                              \
            }                                                                                  \
            /* step 7: dirty tile recorded, carry dropped (:261-267) */                        \
            if (dirty) { s_tail = 0; spec[2 * nd] = bs_start; spec[2 * nd + 1] = bs_stop; nd++; }\
        }                                                                                      \
    }                                                                                          \
    if (ndirty) *ndirty = nd;                                                                  \
    free(inter); free(bs);                                                                     \
    return nwarps;                                                                             \
}

/* The host steps of run_benchmark after the kernel (bhsparse_spmv_cuda.h:166-222) on the   */
/* kernel's compacted y, synchronizer and speculator.  *flags bit 0: the fix-up would read   */
/* row_ptr[m+1] (last tile dirty); that read and the write of y[m] are skipped.              */
#define ORACLE_CALIB(NAME, VT)                                                                 \
void NAME(int m, const int *row_ptr, int nwarps, const int *sync_idx, const VT *sync_val,      \
          int nd, const int *spec, VT *y, int *flags)                                          \
{                                                                                              \
    int fl = 0;                                                                                \
    /* host step 8: inter-warp calibration, bhsparse_spmv_cuda.h:170-173 */                    \
    for (int w = 0; w < nwarps; w++) y[sync_idx[w]] += sync_val[w];                            \
    /* host step 9: speculative check, :184-222 */                                             \
    if (nd) {                                                                                  \
        VT *yt = (VT *)malloc(sizeof(VT) * (m > 0 ? m : 1));                                   \
        memcpy(yt, y, sizeof(VT) * m);                                                         \
        for (int d = 0; d < nd; d++) {                                                         \
            int s0 = spec[2 * d], s1 = spec[2 * d + 1];                                        \
            int yp = s0;                                                                       \
            int ro = row_ptr[s0];                                                              \
            for (int j = s0 + 1; j <= s1 + 1; j++) {                                           \
                if (j > m) { fl |= 1; break; }   /* row_ptr[m+1] would be read: guarded */     \
                int rn = row_ptr[j];                                                           \
                if (ro != rn) {                                                                \
                    if (j - 1 == s1) { y[j - 1] += yt[yp]; yt[j - 1] += yt[yp]; }              \
                    else y[j - 1] = yt[yp];                                                    \
                    yp++;                                                                      \
                } else {                                                                       \
                    y[j - 1] = 0;                                                              \
                }                                                                              \
                ro = rn;                                                                       \
            }                                                                                  \
        }                                                                                      \
        free(yt);                                                                              \
    }                                                                                          \
    if (flags) *flags = fl;                                                                    \
}

/* SpMV_kernel followed by the host calibration: what run_benchmark leaves in y. */
#define ORACLE_BHSPARSE(NAME, KNAME, CNAME, VT)                                                \
int NAME(int m, int n, int nnz, const int *row_ptr, const int *col, const VT *val,             \
         const VT *x, int seg_h, int step, VT *y, int *sync_idx, VT *sync_val,                 \
         int *spec, int *ndirty, int *flags)                                                   \
{                                                                                              \
    int nd = 0;                                                                                \
    const int nwarps = KNAME(m, n, nnz, row_ptr, col, val, x, seg_h, step, y, sync_idx,        \
                             sync_val, spec, &nd);                                             \
    if (flags) *flags = 0;                                                                     \
    if (nwarps < 0) return nwarps;                                                             \
    CNAME(m, row_ptr, nwarps, sync_idx, sync_val, nd, spec, y, flags);                         \
    if (ndirty) *ndirty = nd;                                                                  \
    return nwarps;                                                                             \
}

ORACLE_KERNEL(oracle_bhsparse_kernel_f64, double)
ORACLE_KERNEL(oracle_bhsparse_kernel_f32, float)
ORACLE_CALIB(oracle_calibrate_f64, double)
ORACLE_CALIB(oracle_calibrate_f32, float)
ORACLE_BHSPARSE(oracle_bhsparse_f64, oracle_bhsparse_kernel_f64, oracle_calibrate_f64, double)
ORACLE_BHSPARSE(oracle_bhsparse_f32, oracle_bhsparse_kernel_f32, oracle_calibrate_f32, float)

/* Number of warps (thread bunches) of the reference launch: bhsparse_spmv_cuda.h:326-328. */
int oracle_num_warps(int nnz, int seg_h, int step)
{
    int pnum = oracle_num_tiles(nnz, ORACLE_LANES * seg_h);
    return (pnum + step - 1) / step;
}

/* ------------------------------------------------------------------------- */
/* Serial and OpenMP CSR loops: spmv_cuda/main.cu:755-761 and :377-393.       */
/* ------------------------------------------------------------------------- */

void oracle_csr_serial_f64(int m, const int *row_ptr, const int *col, const double *val,
                           const double *x, double *y)
{
    for (int i = 0; i < m; i++) {
        double sum = 0;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++)
            sum += x[col[j]] * val[j];
        y[i] = sum;
    }
}

void oracle_csr_serial_f32(int m, const int *row_ptr, const int *col, const float *val,
                           const float *x, float *y)
{
    for (int i = 0; i < m; i++) {
        float sum = 0;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++)
            sum += x[col[j]] * val[j];
        y[i] = sum;
    }
}

/* Rows [r0, r1) only: the bounded sample the benchmark's CPU leg times. */
void oracle_csr_serial_rows_f64(int r0, int r1, const int *row_ptr, const int *col,
                                const double *val, const double *x, double *y)
{
    for (int i = r0; i < r1; i++) {
        double sum = 0;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++)
            sum += x[col[j]] * val[j];
        y[i] = sum;
    }
}

void oracle_csr_omp_f64(int m, const int *row_ptr, const int *col, const double *val,
                        const double *x, double *y, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < m; i++) {
        double sum = 0;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++)
            sum += x[col[j]] * val[j];
        y[i] = sum;
    }
    (void)nthreads;
}

void oracle_csr_omp_f32(int m, const int *row_ptr, const int *col, const float *val,
                        const float *x, float *y, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < m; i++) {
        float sum = 0;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++)
            sum += x[col[j]] * val[j];
        y[i] = sum;
    }
    (void)nthreads;
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* FP64 compensated oracle (Ogita-Rump-Oishi Dot2) and |A||x|.                */
/* ------------------------------------------------------------------------- */

static inline void two_sum(double a, double b, double *s, double *e)
{
    double ss = a + b;
    double z = ss - a;
    *e = (a - (ss - z)) + (b - z);
    *s = ss;
}

static inline void two_prod(double a, double b, double *p, double *e)
{
    double pp = a * b;
    *e = fma(a, b, -pp);
    *p = pp;
}

/* y*_i = Dot2(val[row i], x[col[row i]]): about twice the working precision,
 * so its own error is far below the 1e-12 / 1e-6 tolerances it judges. */
void oracle_csr_dot2(int m, const int *row_ptr, const int *col, const double *val,
                     const double *x, double *y, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1024)
#endif
    for (int i = 0; i < m; i++) {
        double p = 0, s = 0;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++) {
            double h, r, q;
            two_prod(val[j], x[col[j]], &h, &r);
            two_sum(p, h, &p, &q);
            s += q + r;
        }
        y[i] = p + s;
    }
    (void)nthreads;
}

void oracle_csr_absrow(int m, const int *row_ptr, const int *col, const double *val,
                       const double *x, double *out, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1024)
#endif
    for (int i = 0; i < m; i++) {
        double s = 0;
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; j++)
            s += fabs(val[j]) * fabs(x[col[j]]);
        out[i] = s;
    }
    (void)nthreads;
}
