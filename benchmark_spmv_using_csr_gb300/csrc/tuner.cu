// tuner.cu -- schedule autotuner and the row-length features the learned tuner reads.
//
// The autotuner times every candidate schedule (non-zeros per lane S, tiles per worker,
// warps per CTA, direct or TMA-staged stream) of the tile kernel on the caller's matrix and reports the per-candidate time
// and the fastest.  It only picks a schedule; every candidate computes the same y (the
// arithmetic does not depend on the schedule beyond summation order).  No counterpart in the
// reference, whose tile geometry is fixed at compile time (spmv_cuda/common.h:39-48).
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/spmv_gb300.h"
#include "internal.h"
#include "tile.cuh"

namespace {

struct Cand {
    int seg, tpw, warps, stages;
};
// Direct loads: S in {8,16,32} x tiles-per-worker in {1,4,8,16} x warps-per-CTA in {4,8}; then
// the TMA-staged ring (2 or 3 tiles) at S in {8,16} x tiles-per-worker in {4,8}, 4 warps.
const Cand kCands[] = {
    {8, 1, 4, 0},  {8, 1, 8, 0},  {8, 4, 4, 0},  {8, 4, 8, 0},  {8, 8, 4, 0},  {8, 8, 8, 0},
    {8, 16, 4, 0}, {8, 16, 8, 0}, {16, 1, 4, 0}, {16, 1, 8, 0}, {16, 4, 4, 0}, {16, 4, 8, 0},
    {16, 8, 4, 0}, {16, 8, 8, 0}, {16, 16, 4, 0}, {16, 16, 8, 0}, {32, 1, 4, 0}, {32, 1, 8, 0},
    {32, 4, 4, 0}, {32, 4, 8, 0}, {32, 8, 4, 0}, {32, 8, 8, 0}, {32, 16, 4, 0}, {32, 16, 8, 0},
    {8, 4, 4, 2},  {8, 8, 4, 2},  {8, 4, 4, 3},  {8, 8, 4, 3},  {16, 4, 4, 2}, {16, 8, 4, 2},
    {16, 4, 4, 3}, {16, 8, 4, 3},
};
constexpr int kNumCands = sizeof(kCands) / sizeof(kCands[0]);

}  // namespace

extern "C" int bhsp_tune_num_candidates(void) { return kNumCands; }

extern "C" int bhsp_tune_candidate(int index, int* seg, int* tiles_per_worker, int* warps_per_cta,
                                   int* stages) {
    if (index < 0 || index >= kNumCands) return BHSPARSE_INVALID_ARGUMENT;
    if (seg) *seg = kCands[index].seg;
    if (tiles_per_worker) *tiles_per_worker = kCands[index].tpw;
    if (warps_per_cta) *warps_per_cta = kCands[index].warps;
    if (stages) *stages = kCands[index].stages;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_autotune(int value_type, int m, int n, int nnz, const int* d_row_ptr,
                             const int* d_col_idx, const void* d_val, const void* d_x, void* d_y,
                             int warmup, int reps, float* ms_out, int* best, void* stream) {
    if (warmup < 0 || reps < 1 || !ms_out) return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = bhsp_validate_csr(d_row_ptr, d_col_idx, m, n, nnz, stream);
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return BHSPARSE_CUDA_ERROR;
    }
    // a scratch buffer of twice the L2 size, written before every timed run so that each run
    // starts with the matrix and x out of L2 (skipped if it cannot be allocated)
    void* flush = nullptr;
    size_t flush_bytes = 0;
    {
        int dev = 0, l2 = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) == cudaSuccess && l2 > 0) {
            flush_bytes = 2 * (size_t)l2;
            if (cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
                flush = nullptr;
                cudaGetLastError();  // clear the failed allocation
            }
        }
    }
    int best_i = -1;
    float best_ms = 0.f;
    std::vector<float> t((size_t)reps);
    for (int i = 0; i < kNumCands && rc == BHSPARSE_SUCCESS; ++i) {
        const spmv::TileConfig c{kCands[i].seg, kCands[i].tpw, kCands[i].warps, kCands[i].stages};
        const int smem = spmv::tile_config_smem_bytes(value_type, c);
        if (smem < 0 || smem > 227 * 1024) {  // a staged ring this value type cannot hold
            ms_out[i] = INFINITY;
            continue;
        }
        bhsp_plan* p = nullptr;
        rc = spmv::plan_create_impl(&p, value_type, m, n, nnz, d_row_ptr, d_col_idx, c.seg,
                                    c.tiles_per_worker, c.warps_per_cta, c.stages, stream, false);
        if (rc) break;
        for (int w = 0; w < warmup && rc == 0; ++w) rc = bhsp_plan_execute(p, d_val, d_x, d_y, stream);
        for (int r = 0; r < reps && rc == 0; ++r) {
            if (flush && cudaMemsetAsync(flush, r & 0xff, flush_bytes, st) != cudaSuccess)
                rc = BHSPARSE_CUDA_ERROR;
            if (!rc && cudaEventRecord(e0, st) != cudaSuccess) rc = BHSPARSE_CUDA_ERROR;
            if (!rc) rc = bhsp_plan_execute(p, d_val, d_x, d_y, stream);
            if (!rc && cudaEventRecord(e1, st) != cudaSuccess) rc = BHSPARSE_CUDA_ERROR;
            if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = BHSPARSE_CUDA_ERROR;
            if (!rc && cudaEventElapsedTime(&t[r], e0, e1) != cudaSuccess) rc = BHSPARSE_CUDA_ERROR;
        }
        if (!rc) rc = bhsp_plan_check(p, stream);
        bhsp_plan_destroy(p);
        if (rc) break;
        std::sort(t.begin(), t.end());
        ms_out[i] = t[(size_t)reps / 2];
        if (best_i < 0 || ms_out[i] < best_ms) {
            best_i = i;
            best_ms = ms_out[i];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (flush) cudaFree(flush);
    if (best) *best = best_i;
    return rc;
}

// ---------------------------------------------------------------------------------------
// Row-length features: 16 cheap statistics of a matrix, computed from row_ptr in one pass
// ---------------------------------------------------------------------------------------
namespace spmv {

// acc[0] = sum of lengths, acc[1] = sum of squares, acc[2] = max, acc[3] = empty rows,
// acc[4 + b] = rows in length bin b (1, 2-3, 4-7, 8-15, 16-31, 32-63, 64-255, 256-4095, >=4096)
__global__ void k_row_features(const int* __restrict__ row_ptr, int m,
                               unsigned long long* __restrict__ acc) {
    __shared__ unsigned long long s[13];
    if (threadIdx.x < 13) s[threadIdx.x] = 0ull;
    __syncthreads();
    unsigned long long sum = 0, sq = 0, mx = 0, empty = 0;
    unsigned long long bins[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;  // 64-bit: m may be near 2^31
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < m; r += stride) {
        const unsigned long long L = (unsigned long long)(__ldg(row_ptr + r + 1) - __ldg(row_ptr + r));
        sum += L;
        sq += L * L;
        mx = L > mx ? L : mx;
        if (L == 0) {
            ++empty;
            continue;
        }
        const int lg = 63 - __clzll((long long)L);  // floor(log2 L)
        const int b = lg <= 5 ? lg : (lg < 8 ? 6 : (lg < 12 ? 7 : 8));
        ++bins[b];
    }
    atomicAdd(&s[0], sum);
    atomicAdd(&s[1], sq);
    atomicMax(&s[2], mx);
    atomicAdd(&s[3], empty);
#pragma unroll
    for (int b = 0; b < 9; ++b)
        if (bins[b]) atomicAdd(&s[4 + b], bins[b]);
    __syncthreads();
    if (threadIdx.x < 13) {
        if (threadIdx.x == 2)
            atomicMax(&acc[2], s[2]);
        else
            atomicAdd(&acc[threadIdx.x], s[threadIdx.x]);
    }
}

}  // namespace spmv

extern "C" int bhsp_row_features(const int* d_row_ptr, int m, int n, float* features16,
                                 void* stream) {
    if (!d_row_ptr || !features16 || m < 0 || n < 0) return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned long long* acc = nullptr;
    if (cudaMalloc(&acc, 13 * sizeof(unsigned long long)) != cudaSuccess) return BHSPARSE_OUT_OF_MEMORY;
    unsigned long long h[13] = {0};
    int rc = BHSPARSE_SUCCESS;
    if (cudaMemsetAsync(acc, 0, sizeof h, st) != cudaSuccess) rc = BHSPARSE_CUDA_ERROR;
    if (!rc && m > 0) {
        const int blocks = spmv::grid_for(m, 256, 8);
        spmv::k_row_features<<<blocks, 256, 0, st>>>(d_row_ptr, m, acc);
        if (cudaGetLastError() != cudaSuccess) rc = BHSPARSE_CUDA_ERROR;
    }
    if (!rc && (cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = BHSPARSE_CUDA_ERROR;
    cudaFree(acc);
    if (rc) return rc;
    bhsp_features_from_counts(m, n, h, features16);
    return BHSPARSE_SUCCESS;
}

// The 16 features from the accumulated counts (host arithmetic, shared with the CPU path):
//  0 log2(m+1)  1 log2(n+1)  2 log2(nnz+1)  3 log2(1+mean)  4 log2(1+std)  5 log2(1+max)
//  6 empty-row fraction  7..15 fraction of rows with length in 1, 2-3, 4-7, 8-15, 16-31, 32-63,
//  64-255, 256-4095, >=4096
extern "C" void bhsp_features_from_counts(int m, int n, const unsigned long long* c, float* f) {
    const double mm = m > 0 ? (double)m : 1.0;
    const double sum = (double)c[0];
    const double mean = sum / mm;
    double var = (double)c[1] / mm - mean * mean;
    if (var < 0) var = 0;
    f[0] = (float)std::log2((double)m + 1.0);
    f[1] = (float)std::log2((double)n + 1.0);
    f[2] = (float)std::log2(sum + 1.0);
    f[3] = (float)std::log2(1.0 + mean);
    f[4] = (float)std::log2(1.0 + std::sqrt(var));
    f[5] = (float)std::log2(1.0 + (double)c[2]);
    f[6] = (float)((double)c[3] / mm);
    for (int b = 0; b < 9; ++b) f[7 + b] = (float)((double)c[4 + b] / mm);
}
