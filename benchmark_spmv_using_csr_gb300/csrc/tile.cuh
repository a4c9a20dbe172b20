// tile.cuh -- tile partition and bit-flag generation shared by every kernel.
//
// Geometry: a tile is 32 lanes x S consecutive non-zeros, lane l owning tile slots
// [l*S, (l+1)*S) -- the transposed ownership of spmv_cuda/kernels_cuda.h:152-162, but
// realised by each lane loading its own contiguous run instead of a shared-memory
// transpose.
//
// tile_ptr[t] (t = 0..ntiles) is the row found for boundary min(t*TILE, nnz) by the
// right-boundary binary search of spmv_cuda/utils_cuda.h:6-31 (called at
// spmv_cuda/kernels_cuda.h:43-49), with bit 31 set when tile t contains an empty row
// (the dirty test of spmv_cuda/kernels_cuda.h:119-145; the reference keeps it as a
// per-warp flag and a speculator entry, here it is packed into tile_ptr).
#pragma once
#include "common.cuh"

namespace spmv {

constexpr uint32_t DIRTY_BIT = 0x80000000u;
constexpr uint32_t ROW_MASK = 0x7fffffffu;

// spmv_cuda/utils_cuda.h:6-31: first index in [0, size) whose row_ptr entry exceeds key.
__device__ __forceinline__ int search_right(const int* __restrict__ row_ptr, int key, int size) {
    int start = 0, stop = size - 1;
    while (stop >= start) {
        const int median = (stop + start) >> 1;
        if (key >= __ldg(row_ptr + median))
            start = median + 1;
        else
            stop = median - 1;
    }
    return start;
}

// First 64 row_ptr entries of a span (two batches of 32 rows, row_ptr[r] and row_ptr[r+1]),
// loaded one tile ahead of their use.
struct RowBatch {
    int a0, b0, a1, b1;
};
__device__ __forceinline__ RowBatch prefetch_rows(const int* __restrict__ row_ptr, int m, int lo) {
    RowBatch rb{0, 0, 0, 0};
    const int r = lo + lane_id();
    if (r < m) {
        rb.a0 = __ldg(row_ptr + r);
        rb.b0 = __ldg(row_ptr + r + 1);
    }
    if (r + 32 < m) {
        rb.a1 = __ldg(row_ptr + r + 32);
        rb.b1 = __ldg(row_ptr + r + 33);
    }
    return rb;
}

// Bit-flag word of this lane for tile [e0, e0+32*S) with span [lo, hi] -- the words of
// spmv_cuda/kernels_cuda.h:116-148: for every non-empty row r of the span whose offset
// o = row_ptr[r] - e0 lies in [0, 32*S), bit 31 - o%S of word o/S; offsets past the tile are
// ignored (:131-133) and the word is the raw one, before the reference forces lane 0's head
// bit (:172) -- plus s_rowof[o] = r for
// every non-empty row r starting at tile slot o, and y[r] = 0 for every empty row of the
// span -- each empty row lies strictly inside exactly one span, so it is written once.  The
// slot -> row map replaces the compacted scatter of kernels_cuda.h:239-257 and the host
// fix-up of bhsparse_spmv_cuda.h:184-222: a dirty tile writes its rows at their true index.
template <int S, typename YT>
__device__ __forceinline__ uint32_t tile_rows(const int* __restrict__ row_ptr, int m, int e0,
                                              int lo, int hi, const RowBatch& rb,
                                              uint32_t* s_words, int* s_rowof, YT* y) {
    constexpr int TILE = 32 * S;
    const int lane = lane_id();
    s_words[lane] = 0u;
    __syncwarp();
    const int stop = hi == m ? m - 1 : hi;
    for (int base = lo, i = 0; base <= stop; base += 32, ++i) {
        const int r = base + lane;
        const bool valid = r <= stop;
        int A, B;
        if (i == 0) {
            A = rb.a0;
            B = rb.b0;
        } else if (i == 1) {
            A = rb.a1;
            B = rb.b1;
        } else {
            A = valid ? __ldg(row_ptr + r) : 0;
            B = valid ? __ldg(row_ptr + r + 1) : 0;
        }
        if (valid) {
            if (A != B) {
                const int off = A - e0;
                if (off >= 0 && off < TILE) {
                    atomicOr(&s_words[off / S], 1u << (31 - off % S));
                    s_rowof[off] = r;
                }
            } else if (y != nullptr) {
                y[r] = YT(0);
            }
        }
    }
    __syncwarp();
    const uint32_t w = s_words[lane];
    __syncwarp();
    return w;
}

}  // namespace spmv
