// internal.h -- launchers shared between the library's translation units (not installed).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace spmv {

inline int num_tiles(int nnz, int tile) { return (int)(((long long)nnz + tile - 1) / tile); }

// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount, looked up
// once per device; 152 on a GB300).  Grid-stride launchers cap their grids at a multiple of it.
int device_sm_count();
// min(ceil(work / threads), cap_per_sm * SMs), at least 1: the grid of a grid-stride launch
int grid_for(long long work, int threads, int cap_per_sm);

// hostcopy.cu: host <-> device copies for the handle API.  The device reads pageable host
// memory coherently where it has pageable memory access through the host's page tables (Grace);
// host_copy then reads pageable, 16-byte-aligned host buffers with a copy kernel (faster than
// the driver's staged cudaMemcpy there) and uses cudaMemcpyAsync for everything else, including
// every device -> host copy (cudaMemcpy is the faster writer).
bool host_direct_access();
bool is_pageable_host(const void* p);
cudaError_t host_copy(void* dst, const void* src, size_t bytes, bool device_to_host,
                      cudaStream_t st);

// Schedule of the plain / mixed tile kernels: S non-zeros per lane (tile = 32*S), a worker
// (one warp) walks `tiles_per_worker` consecutive tiles, `warps_per_cta` workers per CTA.
struct TileConfig {
    int seg;               // S in {8, 16, 32}
    int tiles_per_worker;  // >= 1
    int warps_per_cta;     // 4 or 8
    int stages;            // 0: direct 256-bit loads; 2, 3 or 4: TMA-staged ring of that depth
};

// partition.cu
cudaError_t launch_partition(const int* row_ptr, int m, int nnz, int tile, uint32_t* tile_ptr,
                             cudaStream_t st);
cudaError_t launch_bitflags(const int* row_ptr, int m, int nnz, int seg, const uint32_t* tile_ptr,
                            uint32_t* words, cudaStream_t st);
// *count = non-empty rows shorter than cw non-zeros (zeroed first)
cudaError_t launch_short_rows(const int* row_ptr, int m, int cw, uint32_t* count, cudaStream_t st);
// counts[0] = sampled non-zeros (every step-th), counts[1] = those whose column lies within 4 of
// the previous entry of its row or of the entry at the same position of the previous row
// (zeroed first)
cudaError_t launch_x_locality(const int* row_ptr, const int* col, int m, int nnz, int step,
                              uint32_t* counts, cudaStream_t st);
// Whether the x gathers bypass L1: less than half of the sampled non-zeros have such a near
// column (stencils and block matrices ~0.99, random columns <= 0.15).
inline bool x_l2_pays(long long sampled, long long near) { return 2 * near < sampled; }
// Whether the tile kernels take the one-head chunk form: the short rows can break at most 1/4
// of the warp-chunks (32 lanes x cw slots).  Measured on rows of 27 non-zeros with a share of
// 1-3-entry rows: the form still wins where they could break half of the chunks (1.00-1.06x),
// loses where they can break all of them, and is mixed in between.
inline bool one_head_pays(long long short_rows, long long nnz, int cw) {
    const long long chunks = (nnz + 32LL * cw - 1) / (32LL * cw);
    return 4 * short_rows <= chunks;
}
cudaError_t launch_validate(const int* row_ptr, const int* col, int m, int n, int nnz,
                            uint32_t* bad, cudaStream_t st);

// spmv_plain.cu: plain forms (value type = accumulate type = FP64 or FP32)
struct PlainLaunch {
    const int* row_ptr;
    const int* col;
    const void* val;
    const void* x;
    void* y;
    const uint32_t* tile_ptr;
    int* rec_row;     // [nworkers]
    void* rec_val;    // [nworkers] of the value type
    uint32_t* err;
    int m, n, nnz;
    int phase;  // bit 0: tile kernel, bit 1: calibration kernel
    bool one_head = false;  // the plan's choice of the one-head chunk form
    bool x_l2 = false;      // the plan's choice of L2-only x gathers
    int* ticket = nullptr;  // [2] the persistent kernel's work queue, zero between launches
    int grid_mode = -1;     // -1 the launcher's rule, 0 static grid, 1 persistent
};
cudaError_t launch_plain_f64(const PlainLaunch& a, const TileConfig& cfg, cudaStream_t st);
cudaError_t launch_plain_f32(const PlainLaunch& a, const TileConfig& cfg, cudaStream_t st);
int plain_f32_smem_bytes(const TileConfig& cfg);

// spmv_mixed.cu: mixed forms (FP32 / BF16 values, FP32 x and y, compensated FP32
// accumulation, FP64 carries and records)
struct MixedLaunch {
    const int* row_ptr;
    const int* col;
    const void* val;  // float or __nv_bfloat16
    const float* x;
    float* y;
    const uint32_t* tile_ptr;
    int* rec_row;
    double* rec_val;
    uint32_t* err;
    int m, n, nnz;
    bool bf16;
    int phase;  // bit 0: tile kernel, bit 1: calibration kernel
    bool one_head = false;  // the plan's choice of the one-head chunk form
    bool x_l2 = false;      // the plan's choice of L2-only x gathers
    int* ticket = nullptr;  // [2] the persistent kernel's work queue, zero between launches
    int grid_mode = -1;     // -1 the launcher's rule, 0 static grid, 1 persistent
};
cudaError_t launch_mixed(const MixedLaunch& a, const TileConfig& cfg, cudaStream_t st);
cudaError_t launch_mixed_bf16(const MixedLaunch& a, const TileConfig& cfg, cudaStream_t st);
int mixed_bf16_smem_bytes(const TileConfig& cfg);
cudaError_t launch_convert_from_f64(const double* src, void* dst, size_t n, bool to_bf16,
                                    cudaStream_t st);
cudaError_t launch_convert_to_f64(const float* src, double* dst, size_t n, cudaStream_t st);

inline bool is_supported_value_type(int vt) { return vt >= 0 && vt <= 3; }

}  // namespace spmv
struct bhsp_plan;
namespace spmv {
// bhsp_plan_create with the device-side CSR validation made optional (the autotuner validates
// once and then builds one plan per candidate schedule).
int plan_create_impl(bhsp_plan** out, int value_type, int m, int n, int nnz, const int* d_row_ptr,
                     const int* d_col_idx, int seg, int tiles_per_worker, int warps_per_cta,
                     int stages, void* stream, bool validate);

// Dynamic shared memory one CTA of the TMA-staged kernel needs (0 for the direct kernel);
// value_type as in bhsp_value_type.  Configurations above 227 KB cannot run.
int tile_config_smem_bytes(int value_type, const TileConfig& cfg);
int plain_smem_bytes(bool f64, const TileConfig& cfg);
int mixed_smem_bytes(bool bf16, const TileConfig& cfg);

}  // namespace spmv
