/*
 * spmv_gb300.h -- C ABI of the GB300 speculative segmented-sum CSR SpMV (y = A.x).
 *
 * Plain C: opaque handles, plain pointers and sizes.  Every function returns an int
 * status (0 = success) and never aborts the process; the text of the last failure of a
 * handle is available from bhsp_last_error().
 *
 * The handle API mirrors, call for call, the host class bhsparse_spmv_cuda of the
 * reference (spmv_cuda/bhsparse_spmv_cuda.h:7-55); include/bhsparse_spmv_cuda.h wraps
 * it back into that class.  The plan API below it runs the same kernels on buffers that
 * the caller already holds in device memory.
 */
#ifndef SPMV_GB300_H
#define SPMV_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The first two keep the reference's values (spmv_cuda/common.h:24-25). */
#define BHSPARSE_SUCCESS 0
#define BHSPARSE_UNSUPPORTED_VALUE_TYPE -1
#define BHSPARSE_INVALID_ARGUMENT -2     /* bad size, null pointer, unknown config */
#define BHSPARSE_INVALID_CSR -3          /* row_ptr not monotone / not ending at nnz, col out of range */
#define BHSPARSE_CUDA_ERROR -4           /* a CUDA runtime call failed (see bhsp_last_error) */
#define BHSPARSE_NOT_PREPARED -5         /* run/get before prepare_mem */
#define BHSPARSE_DEVICE_CHECK_FAILED -6  /* a kernel's own bounds check fired */
#define BHSPARSE_OUT_OF_MEMORY -7
#define BHSPARSE_NOALLOC_TOO_LARGE -8    /* matrix too large for the fixed scratch of bhsp_spmv_f64_noalloc */

/* Largest nnz accepted (int32 indices with one tile of head-room). */
#define BHSP_MAX_NNZ 2147479551

/* Value types.  F64 / F32 are the reference's USE_DOUBLE=1 / USE_DOUBLE=0 builds
 * (spmv_cuda/common.h:27-31).  The mixed forms take and return FP64 on the host side,
 * store the matrix values in FP32 or BF16 and x / y in FP32, accumulate with a
 * compensated (TwoSum) FP32 segmented sum and carry between tiles in FP64. */
typedef enum {
    BHSP_VALUE_F64 = 0,
    BHSP_VALUE_F32 = 1,
    BHSP_VALUE_MIXED_F32 = 2,
    BHSP_VALUE_MIXED_BF16 = 3
} bhsp_value_type;

/* ------------------------------------------------------------------------------------ */
/* Handle API: one object of the reference class bhsparse_spmv_cuda.                     */
/* ------------------------------------------------------------------------------------ */
typedef struct bhsp_spmv bhsp_spmv;

/* Constructor, spmv_cuda/bhsparse_spmv_cuda.h:10, 57-59 (value type = the USE_DOUBLE choice). */
int bhsp_create(bhsp_spmv** out, int value_type);
/* Destructor (the reference object is deleted by the caller; frees whatever is left). */
void bhsp_destroy(bhsp_spmv* h);
/* init_platform, spmv_cuda/bhsparse_spmv_cuda.h:61-75: selects the device (0 unless
 * bhsp_set_device chose another) and records its name. */
int bhsp_init_platform(bhsp_spmv* h);
/* free_platform, spmv_cuda/bhsparse_spmv_cuda.h:77-82. */
int bhsp_free_platform(bhsp_spmv* h);
/* prepare_mem, spmv_cuda/bhsparse_spmv_cuda.h:238-351: copies A (row_ptr, col_idx, val),
 * x and the initial y into device memory, validates the CSR, builds the tile partition
 * and keeps the caller's y pointer for get_y (the caller's y must outlive the object, as
 * in the reference).  val / x / y are double* for F64 and the mixed forms, float* for F32. */
int bhsp_prepare_mem(bhsp_spmv* h, int m, int n, int nnz, const int* row_ptr,
                     const int* col_idx, const void* val, const void* x, void* y);
/* run_benchmark, spmv_cuda/bhsparse_spmv_cuda.h:121-228: y = A.x on the device, including
 * the calibration of rows that cross tiles and of empty rows; returns when done.  Unlike
 * the reference, the result does not depend on y's previous contents and repeated calls
 * give the same y. */
int bhsp_run_benchmark(bhsp_spmv* h);
/* get_y, spmv_cuda/bhsparse_spmv_cuda.h:230-236: copies y into the pointer given to
 * prepare_mem.  Returns a status (the CUDA twin returns void; the OpenCL twin returns int,
 * spmv_opencl_amd/bhsparse_spmv_opencl.h:401). */
int bhsp_get_y(bhsp_spmv* h);
/* free_mem, spmv_cuda/bhsparse_spmv_cuda.h:84-118. */
int bhsp_free_mem(bhsp_spmv* h);
/* Text of the last failure on this handle ("" if none). */
const char* bhsp_last_error(const bhsp_spmv* h);

/* -- additions with no counterpart in the reference -- */
/* Choose the CUDA device used by init_platform (default 0, as the reference hard-codes). */
int bhsp_set_device(bhsp_spmv* h, int device);
/* Tile schedule: seg = non-zeros per lane (8, 16 or 32), tiles_per_worker >= 1,
 * warps_per_cta 4 or 8, stages = 0 (each lane streams its values with 256-bit loads) or
 * 2 / 3 / 4 (values and column indices staged in a shared-memory ring of that many tiles by
 * 2D tensor copies; a matrix with no full tile runs the direct-load kernel).  Before
 * prepare_mem; 0 for seg / tiles_per_worker / warps_per_cta and -1 for stages take the fixed
 * default (16, 8, 4, 0; stages 2 for BHSP_VALUE_MIXED_BF16, whose staged schedule is the faster
 * one).  Rejected if the staged ring does not fit in shared memory.  Without this call
 * prepare_mem chooses the schedule itself (bhsp_choose_schedule with the handle's network,
 * see bhsp_set_tuner), which is what the reference's callers get: its geometry is a compile-
 * time constant (spmv_cuda/common.h:39-48, spmv_cuda/bhsparse_spmv_cuda.h:323-328). */
int bhsp_set_config(bhsp_spmv* h, int seg, int tiles_per_worker, int warps_per_cta, int stages);
/* The network prepare_mem consults when bhsp_set_config was not called: NULL = the library's
 * network for the handle's value type (the default; see bhsp_choose_schedule), "" = none (the
 * fixed default schedule), else the path of a network file.  Before prepare_mem. */
int bhsp_set_tuner(bhsp_spmv* h, const char* path);
/* How prepare_mem chose the schedule in use: *source = one of BHSP_SCHEDULE_*, *confidence =
 * the network's probability of its pick (0 when no network ran).  With the environment
 * variable BHSP_LOG_SCHEDULE set (not "0"), prepare_mem also prints the schedule and its
 * source to stderr, so a caller that cannot be changed shows what it got. */
int bhsp_get_schedule_source(const bhsp_spmv* h, int* source, float* confidence);
int bhsp_get_config(const bhsp_spmv* h, int* seg, int* tiles_per_worker, int* warps_per_cta,
                    int* stages);
/* Replace x (host pointer, same type as in prepare_mem) without rebuilding anything; returns
 * once x has been read, so the caller may reuse its buffer.  As prepare_mem does, it reads
 * pageable host memory with a copy kernel where the device accesses pageable memory through the
 * host's page tables (a Grace host: 197 against 168 GB/s for cudaMemcpy), and pinned memory with
 * cudaMemcpy. */
int bhsp_set_x(bhsp_spmv* h, const void* x);
/* Streamed SpMVs over many right-hand sides held in host memory: y_host[i] = A x_host[i] for
 * i = 0..count-1, with the upload of x_{i+1} and the download of y_{i-1} overlapping the SpMV of
 * x_i (two device x / y buffer pairs of its own, separate upload, compute and download streams).
 * Blocks until every y_host[i] is written, or, on a failure, until none of its copies and
 * kernels is still running.  The handle's own x and y (prepare_mem / set_x / run_benchmark)
 * are not touched: a later run_benchmark computes with the x it held before.  The extra buffers
 * (2 x (n + m) vector entries) are allocated on the first call and kept until free_mem.  F64
 * and F32 forms; host vectors in the handle's value type, pinned (cudaHostAlloc /
 * cudaHostRegister) for the copies to overlap.  No counterpart in the reference, whose driver
 * runs one SpMV per prepared x (spmv_cuda/main.cu:811-817). */
int bhsp_run_stream(bhsp_spmv* h, int count, const void* const* x_host, void* const* y_host);
/* Enqueue y = A.x on `stream` (a cudaStream_t, NULL = the legacy default stream) and
 * return at once; bhsp_check() synchronises and reports a kernel-side failure. */
int bhsp_run_async(bhsp_spmv* h, void* stream);
int bhsp_check(bhsp_spmv* h);
/* One phase of bhsp_run_async: 1 = the tile kernel, 2 = the calibration kernel that adds
 * the per-worker carry records, 3 = both.  Phase 2 must follow phase 1 on the same stream;
 * exists so that the two kernels can be timed apart. */
int bhsp_run_phase(bhsp_spmv* h, void* stream, int phase);
/* Device pointers of the handle's buffers (for callers that keep working on the device). */
int bhsp_device_buffers(const bhsp_spmv* h, const int** row_ptr, const int** col_idx,
                        const void** val, void** x, void** y);
/* Bytes of device memory the handle holds. */
size_t bhsp_device_bytes(const bhsp_spmv* h);

/* ------------------------------------------------------------------------------------ */
/* Plan API: the same kernels over device buffers the caller owns.                       */
/* ------------------------------------------------------------------------------------ */
typedef struct bhsp_plan bhsp_plan;

/* Validates the CSR on the device, builds tile_ptr and allocates the carry records.
 * row_ptr / col_idx stay owned by the caller and must outlive the plan; col_idx must be
 * 32-byte aligned.  The schedule fields are as in bhsp_set_config. */
int bhsp_plan_create(bhsp_plan** out, int value_type, int m, int n, int nnz,
                     const int* d_row_ptr, const int* d_col_idx, int seg, int tiles_per_worker,
                     int warps_per_cta, int stages, void* stream);
/* y = A.x, enqueued on `stream`.  d_val in the storage type of value_type (double, float,
 * float, __nv_bfloat16), 32-byte aligned; d_x / d_y in the x/y type (double for F64, float
 * otherwise).  A plan runs one SpMV at a time: its tile kernel's work queue and carry records
 * are the plan's own, so calls on one plan must follow each other on one stream (or be ordered
 * by events); separate plans run concurrently. */
int bhsp_plan_execute(bhsp_plan* p, const void* d_val, const void* d_x, void* d_y, void* stream);
/* One phase of bhsp_plan_execute (1 = tile kernel, 2 = calibration, 3 = both). */
int bhsp_plan_execute_phase(bhsp_plan* p, const void* d_val, const void* d_x, void* d_y,
                            void* stream, int phase);
/* Synchronise `stream` and report (then clear) any kernel-side check that fired. */
int bhsp_plan_check(bhsp_plan* p, void* stream);
/* Number of device kernels one bhsp_plan_execute launches. */
int bhsp_plan_launches(const bhsp_plan* p);
/* tile_ptr of the plan (device pointer, ntiles+1 entries) and its tile size. */
int bhsp_plan_tiles(const bhsp_plan* p, const uint32_t** d_tile_ptr, int* ntiles, int* tile_nnz);
/* The chunk form the plan's tile kernel takes, fixed when the plan is built: *short_rows =
 * non-empty rows shorter than one chunk of a lane's slots (4 at seg 8, else 8), *one_head = 1
 * when they are few enough (at most 1/4 of the warp-chunks) for the branch-free one-head form. */
int bhsp_plan_chunk_form(const bhsp_plan* p, int* short_rows, int* one_head);
/* The x gather path the plan's tile kernels take, fixed when the plan is built: of *sampled
 * non-zeros (every nnz / 2^20-th), *near have a column within 4 of the previous entry of their
 * row or of the same-position entry of the previous row; *l2_only = 1 (x gathered from L2
 * only, ld.global.cg) when fewer than half do, else x goes through L1. */
int bhsp_plan_gather_path(const bhsp_plan* p, int* sampled, int* near, int* l2_only);
/* Overrides the kernel variant the plan's rules chose: one_head (the chunk form above) and
 * l2_only (the gather path) = 1 or 0 to force it, -1 to keep the rule's choice.  Every variant
 * gives the same y; only the speed differs.  Takes effect at the next bhsp_plan_execute. */
int bhsp_plan_set_variant(bhsp_plan* p, int one_head, int l2_only);
/* Overrides the grid of the direct-load tile kernel: 1 = the persistent kernel (warps draw
 * workers from the plan's work queue), 0 = a static grid of one warp per worker, -1 = the rule
 * (persistent when the workers exceed one wave of the static grid, except plain FP64 in the
 * one-head form, which always runs the static grid and ignores 1).  Same y either way. */
int bhsp_plan_set_grid(bhsp_plan* p, int persistent);
const char* bhsp_plan_last_error(const bhsp_plan* p);
void bhsp_plan_destroy(bhsp_plan* p);

/* ------------------------------------------------------------------------------------ */
/* Partition primitives (device pointers), exposed for parity checks.                    */
/* ------------------------------------------------------------------------------------ */
/* tile_ptr[t], t = 0..ceil(nnz/tile_nnz): the row of boundary min(t*tile_nnz, nnz) found by
 * the right-boundary binary search (spmv_cuda/utils_cuda.h:6-31, kernels_cuda.h:39-53),
 * bit 31 set when tile t holds an empty row (kernels_cuda.h:119-145). */
int bhsp_partition(const int* d_row_ptr, int m, int nnz, int tile_nnz, uint32_t* d_tile_ptr,
                   void* stream);
/* Raw bit-flag words, 32 per tile of 32*seg non-zeros (kernels_cuda.h:114-148, before the
 * lane-0 head bit is forced at :172).  seg in {1,2,4,8,16,32}; d_words may be NULL when
 * nnz == 0 (there are no tiles). */
int bhsp_bitflags(const int* d_row_ptr, int m, int nnz, int seg, const uint32_t* d_tile_ptr,
                  uint32_t* d_words, void* stream);
/* 0 if the CSR is valid, else BHSPARSE_INVALID_CSR (synchronises `stream`). */
int bhsp_validate_csr(const int* d_row_ptr, const int* d_col_idx, int m, int n, int nnz,
                      void* stream);

/* ------------------------------------------------------------------------------------ */
/* Batched multi-RHS form (no counterpart in the reference).                             */
/* ------------------------------------------------------------------------------------ */
/* Many CSR matrices and k in {1,2,4,8} right-hand sides per launch, FP32 storage, compensated
 * FP32 accumulation (the mixed form's arithmetic), FP64 carry records.  The batch is passed as
 * one block-diagonal CSR (device pointers, kept by the caller):
 *   d_row_ptr[m_total+1]: the matrices' row pointers concatenated, with global non-zero offsets;
 *   d_col_idx[nnz_total]: each matrix's column indices plus the offset of its x block
 *                         (32-byte aligned).
 * x is [n_total][k] and y is [m_total][k], the k values of a row interleaved.  One persistent
 * kernel hands out tile ranges from a global ticket; schedule fields as in bhsp_set_config
 * (0 = default: seg 16, or 32 for k = 4; 4 tiles per worker; 4 warps per CTA).  Validates the
 * CSR and builds the partition (synchronous). */
typedef struct bhsp_batch bhsp_batch;
int bhsp_batch_create(bhsp_batch** out, int count, int m_total, int n_total, int nnz_total,
                      const int* d_row_ptr, const int* d_col_idx, int k, int seg,
                      int tiles_per_worker, int warps_per_cta, void* stream);
/* y = A.x for all matrices and right-hand sides, enqueued on `stream`.  use_graph != 0 replays a
 * CUDA graph of the persistent kernel and the calibration (captured on the
 * first call and again whenever the buffers change); use_graph == 0 launches them directly.
 * d_val 32-byte aligned, d_x / d_y aligned to 4*k bytes. */
int bhsp_batch_execute(bhsp_batch* b, const float* d_val, const float* d_x, float* d_y,
                       int use_graph, void* stream);
int bhsp_batch_check(bhsp_batch* b, void* stream);
int bhsp_batch_info(const bhsp_batch* b, int* ntiles, int* nworkers, int* grid, int* launches);
/* The kernel variant bhsp_batch_create chose for the batch, as bhsp_plan_chunk_form /
 * bhsp_plan_gather_path do for one matrix: *one_head = 1 for the branch-free one-head chunk form
 * (one right-hand side and few rows shorter than a chunk), *l2_only = 1 when x is gathered from
 * L2 only (fewer than half of about 2^20 sampled columns lie near their neighbours). */
int bhsp_batch_variant(const bhsp_batch* b, int* one_head, int* l2_only);
/* Overrides that choice: one_head / l2_only = 1 or 0 to force, -1 to keep.  The one-head form
 * exists for one right-hand side only (one_head = 1 with k > 1 is rejected).  Every variant
 * gives the same y; the next bhsp_batch_execute with use_graph captures the graph again. */
int bhsp_batch_set_variant(bhsp_batch* b, int one_head, int l2_only);
/* The batched form's schedule tuner.  Candidates: S 8 / 16 / 32 x 1 / 2 / 4 / 8 tiles per
 * worker x 4 / 8 warps per CTA.  bhsp_batch_autotune builds the batch at every candidate and
 * times bhsp_batch_execute (graph replay; `warmup` untimed runs, then the median of `reps`
 * CUDA-event-timed runs, each after a write of twice the L2 size) on the caller's buffers,
 * writing ms_out[bhsp_batch_tune_num_candidates()] and the fastest's index to *best; pass the
 * pick to bhsp_batch_create.  Synchronous. */
int bhsp_batch_tune_num_candidates(void);
int bhsp_batch_tune_candidate(int index, int* seg, int* tiles_per_worker, int* warps_per_cta);
int bhsp_batch_autotune(int count, int m_total, int n_total, int nnz_total, const int* d_row_ptr,
                        const int* d_col_idx, int k, const float* d_val, const float* d_x,
                        float* d_y, int warmup, int reps, float* ms_out, int* best, void* stream);
const char* bhsp_batch_last_error(const bhsp_batch* b);
void bhsp_batch_destroy(bhsp_batch* b);

/* ------------------------------------------------------------------------------------ */
/* Schedule tuning (no counterpart in the reference, whose tile geometry is fixed at     */
/* compile time: spmv_cuda/common.h:39-48).                                              */
/* ------------------------------------------------------------------------------------ */
/* The candidate schedules: index -> (non-zeros per lane, tiles per worker, warps per CTA,
 * stages): 24 direct-load schedules (S 8 / 16 / 32 x 1 / 4 / 8 / 16 tiles per worker x 4 / 8
 * warps) and 8 TMA-staged ones (S 8 / 16 x 4 / 8 tiles per worker x 2 / 3 stages, 4 warps). */
int bhsp_tune_num_candidates(void);
int bhsp_tune_candidate(int index, int* seg, int* tiles_per_worker, int* warps_per_cta,
                        int* stages);
/* Autotuner: validates the CSR, then times y = A.x for every candidate on the given device
 * buffers (`warmup` untimed runs, then the median of `reps` CUDA-event-timed runs, each
 * preceded by a write of twice the L2 size so that it starts with the matrix and x out of L2)
 * and writes ms_out[bhsp_tune_num_candidates()] and the index of the fastest to *best.  A
 * staged candidate whose ring does not fit in shared memory for this value type is not run and
 * gets +infinity.  Synchronous. */
int bhsp_autotune(int value_type, int m, int n, int nnz, const int* d_row_ptr,
                  const int* d_col_idx, const void* d_val, const void* d_x, void* d_y, int warmup,
                  int reps, float* ms_out, int* best, void* stream);
/* Where a schedule came from (bhsp_choose_schedule, bhsp_get_schedule_source). */
#define BHSP_SCHEDULE_CALLER 0  /* bhsp_set_config */
#define BHSP_SCHEDULE_DEFAULT 1 /* the fixed default: no network for this value type */
#define BHSP_SCHEDULE_LEARNED 2 /* the learned network's pick */
#define BHSP_SCHEDULE_SWEEP 3   /* the full autotune sweep: the network was below its threshold */
/* The schedule for a matrix held on the device: the 16 row features (bhsp_row_features) go
 * through the learned network's forward kernels, and its most probable candidate is taken
 * unless a second, small risk network (the features and the first network's top two
 * probabilities and entropy in, the probability that the pick is below 95 % of the best time
 * out) rates the pick as likely slow, or the pick's probability is below the file's confidence
 * threshold; then the full autotune sweep (bhsp_autotune, 1 warm-up and the median of 3
 * flushed-L2 runs per candidate, writing d_y) decides.  *confidence is the first network's
 * probability of its pick.  tuner_path: NULL = the library's network for value_type, the file
 * tuner_data/gb300_<f64|f32|mixed_f32|mixed_bf16>_tuner.bin next to the library (or in the
 * directory named by the BHSP_TUNER_DIR environment variable); with no such file the fixed
 * default is returned (*source = BHSP_SCHEDULE_DEFAULT).  "" = no network (the fixed default).
 * Another path must name a network file trained for value_type.  The network only picks a
 * schedule: every schedule computes the same y up to the summation order.  d_val / d_x / d_y
 * are needed only by the sweep.  Synchronous. */
int bhsp_choose_schedule(int value_type, int m, int n, int nnz, const int* d_row_ptr,
                         const int* d_col_idx, const void* d_val, const void* d_x, void* d_y,
                         const char* tuner_path, int* seg, int* tiles_per_worker,
                         int* warps_per_cta, int* stages, int* source, float* confidence,
                         void* stream);
/* The 16 row-length statistics the learned tuner reads, computed on the device in one pass
 * over row_ptr:  0 log2(m+1), 1 log2(n+1), 2 log2(nnz+1), 3 log2(1+mean length),
 * 4 log2(1+std), 5 log2(1+max), 6 empty-row fraction, 7..15 fraction of rows whose length is
 * 1, 2-3, 4-7, 8-15, 16-31, 32-63, 64-255, 256-4095, >= 4096.  Synchronous. */
int bhsp_row_features(const int* d_row_ptr, int m, int n, float* features16, void* stream);
/* The same features from the 13 accumulated counts (sum, sum of squares, max, empty rows,
 * 9 bin counts); host arithmetic shared by the device path and CPU checks. */
void bhsp_features_from_counts(int m, int n, const unsigned long long* counts13, float* features16);

/* ------------------------------------------------------------------------------------ */
/* Learned tuner network (no counterpart in the reference): I -> H -> H -> K, ReLU, softmax, */
/* trained with soft cross-entropy and Adam by hand-written CUDA kernels (FP32).          */
/* It only chooses a schedule; it never changes the SpMV arithmetic.                     */
/* ------------------------------------------------------------------------------------ */
typedef struct bhsp_mlp bhsp_mlp;
int bhsp_mlp_create(bhsp_mlp** out, int n_in, int n_hidden, int n_out, int max_batch);
/* Flat parameter vector W1[H][I] b1[H] W2[H][H] b2[H] W3[K][H] b3[K] (host copies). */
size_t bhsp_mlp_num_params(const bhsp_mlp* m);
int bhsp_mlp_set_params(bhsp_mlp* m, const float* host_params, size_t count);
int bhsp_mlp_get_params(const bhsp_mlp* m, float* host_params, size_t count);
/* Inputs are standardised as (f - mean) / std on the device (host arrays of n_in). */
int bhsp_mlp_set_normalization(bhsp_mlp* m, const float* mean, const float* std);
/* Probabilities [batch][K] of d_features [batch][I] (device pointers), enqueued on stream. */
int bhsp_mlp_forward(bhsp_mlp* m, const float* d_features, int batch, float* d_probs, void* stream);
/* Gradient of the mean soft cross-entropy against d_targets [batch][K] (rows sum to 1) into
 * d_grads_out (device, num_params; may be NULL) and the loss into *loss_out (host; may be
 * NULL).  Synchronous. */
int bhsp_mlp_gradients(bhsp_mlp* m, const float* d_features, const float* d_targets, int batch,
                       float* d_grads_out, float* loss_out, void* stream);
/* One Adam step (beta 0.9 / 0.999, decoupled weight decay added to the gradient). */
int bhsp_mlp_train_step(bhsp_mlp* m, const float* d_features, const float* d_targets, int batch,
                        float lr, float weight_decay, float* loss_out, void* stream);
void bhsp_mlp_destroy(bhsp_mlp* m);

/* ------------------------------------------------------------------------------------ */
/* Allocation-free entry point (no counterpart in the reference).                        */
/* ------------------------------------------------------------------------------------ */
/* Size of the fixed device scratch array behind bhsp_spmv_f64_noalloc: 2 MiB, held on every GPU
 * that loads the library until the process exits.  With the entry point's schedule (16
 * non-zeros per lane, 8 tiles per worker) it covers matrices of up to about 195 million
 * non-zeros; larger ones are rejected with BHSPARSE_NOALLOC_TOO_LARGE before any work. */
#define BHSP_NOALLOC_SCRATCH_BYTES (2u << 20)
/* y = A.x in plain FP64 for callers that must not allocate device memory: code that runs
 * inside a host framework which owns all device memory through its own caching allocator,
 * real-time loops that cannot afford cudaMalloc / cudaFree (both may synchronise the whole
 * device), or processes whose device footprint must not grow after start-up.  All buffers are
 * the caller's device pointers (d_val and d_col_idx 32-byte aligned); the kernels' scratch
 * (tile partition, carry records, error word, the tile kernel's work queue) lives in the fixed
 * array above, so the call performs no cudaMalloc, cudaFree or other allocating routine.
 *   - The first call on each device looks up the array's device address (with that device
 *     current) and caches it for the rest of the process; make that first call before any
 *     stream capture.  The cached address does not survive a reset of the device's primary
 *     context (cudaDeviceReset): do not call this entry point across one.
 *   - It always runs the tile kernel's per-slot chunk form with x gathered through L1 at a
 *     fixed schedule (16 non-zeros per lane, 8 tiles per worker, 4 warps): the plan-time
 *     choices of the other entry points (one-head form, L2-only gathers, learned or tuned
 *     schedule) need counts read back from the device, which this call skips.
 *   - Every call shares the one array: calls whose work overlaps on the GPU (two streams, two
 *     host threads) race and must not be issued; calls in sequence are safe.
 *   - The call enqueues on `stream` and synchronises it before returning; it returns
 *     BHSPARSE_DEVICE_CHECK_FAILED if a kernel's own check fired.
 *   - validate != 0 first checks the CSR (synchronously) and returns BHSPARSE_INVALID_CSR
 *     instead of running on invalid input; with validate == 0 the CSR must be valid. */
int bhsp_spmv_f64_noalloc(const int* d_row_ptr, const int* d_col_idx, const double* d_val,
                          const double* d_x, double* d_y, int m, int n, int nnz, int validate,
                          void* stream);

/* Library version string and the compute capability it was built for. */
const char* bhsp_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SPMV_GB300_H */
