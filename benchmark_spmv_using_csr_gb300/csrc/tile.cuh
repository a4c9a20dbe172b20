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

// Bit-flag word of this lane for tile [e0, e0 + 32*S) whose row span is [lo, hi]
// (spmv_cuda/kernels_cuda.h:116-148): for every non-empty row r of the span with offset
// o = row_ptr[r] - e0 in [0, 32*S), bit 31 - o%S of word o/S is set.  The word is in the
// reference's bit order (slot k of a lane is bit 31-k) and is the raw word, before the
// reference forces lane 0's head bit (:172).
//
// When `dirty` is set the same pass also (a) writes y[r] = 0 for every empty row of the
// span -- each empty row lies strictly inside exactly one tile span, so it is written once
// -- and (b) lists the span's non-empty rows in order in s_list, so that the k-th row head
// of the tile can be mapped to its row.  This is the empty-row calibration of
// spmv_cuda/bhsparse_spmv_cuda.h:184-222, done at the point where the rows are known
// instead of by a host pass over a compacted y.
template <int S, typename VT>
__device__ __forceinline__ uint32_t tile_flags(const int* __restrict__ row_ptr, int m, int e0,
                                               int lo, int hi, bool dirty, uint32_t* s_words,
                                               int* s_list, int list_cap, VT* y,
                                               uint32_t* err) {
    constexpr int TILE = 32 * S;
    const int lane = lane_id();
    s_words[lane] = 0u;
    __syncwarp();
    const int stop = hi == m ? m - 1 : hi;
    int nlist = 0;
    for (int base = lo; base <= stop; base += 32) {
        const int r = base + lane;
        const bool valid = r <= stop;
        int a = 0, b = 0;
        if (valid) {
            a = __ldg(row_ptr + r);
            b = __ldg(row_ptr + r + 1);
        }
        const bool nonempty = valid && a != b;
        if (nonempty) {
            const int off = a - e0;
            if (off >= 0 && off < TILE) atomicOr(&s_words[off / S], 1u << (31 - off % S));
        }
        if (dirty) {
            if (valid && !nonempty && y != nullptr) y[r] = VT(0);
            const uint32_t bal = __ballot_sync(SPMV_FULL_MASK, nonempty);
            if (nonempty && s_list != nullptr) {
                const int idx = nlist + __popc(bal & ((1u << lane) - 1u));
                if (idx < list_cap)
                    s_list[idx] = r;
                else if (err)
                    atomicOr(err, ERR_LIST_OVERFLOW);
            }
            nlist += __popc(bal);
        }
    }
    __syncwarp();
    const uint32_t w = s_words[lane];
    __syncwarp();
    return w;
}

}  // namespace spmv
