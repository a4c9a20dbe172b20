// partition.cu -- tile_ptr construction (binary-search partition + dirty bits), the
// bit-flag parity kernel, and the CSR validation pass run before a matrix is accepted.
#include <atomic>

#include "internal.h"
#include "tile.cuh"

namespace spmv {

// One thread per tile boundary: tile_ptr[t] = search_right(min(t*TILE, nnz)) - 1
// (spmv_cuda/kernels_cuda.h:43-49).  The reference searches each boundary inside every
// SpMV launch (twice for boundaries shared by adjacent warps); here it is done once per
// matrix and reused by every call.
__global__ void k_tile_rows(const int* __restrict__ row_ptr, int m, int nnz, int tile,
                            int ntiles, uint32_t* __restrict__ tile_ptr) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > ntiles) return;
    long long b = (long long)t * tile;
    if (b > nnz) b = nnz;
    tile_ptr[t] = (uint32_t)(search_right(row_ptr, (int)b, m + 1) - 1);
}

// One thread per row: an empty row r with o = row_ptr[r] lies strictly inside the span of
// tile (o % TILE == 0 ? o/TILE - 1 : o/TILE) (clamped to the last tile), which is exactly
// the tile whose span the reference scans and finds it in (kernels_cuda.h:119-145).
// Leading empty rows (o == 0) belong to no tile.  Setting a bit is idempotent, so the
// result does not depend on the order of the atomics.
__global__ void k_mark_dirty(const int* __restrict__ row_ptr, int m, int tile, int ntiles,
                             uint32_t* __restrict__ tile_ptr) {
    const long long stride = (long long)gridDim.x * blockDim.x;  // 64-bit: m may be near 2^31
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < m; r += stride) {
        const int o = __ldg(row_ptr + r);
        if (o != __ldg(row_ptr + r + 1)) continue;
        int t = (o % tile == 0) ? o / tile - 1 : o / tile;
        if (t > ntiles - 1) t = ntiles - 1;
        if (t >= 0) atomicOr(tile_ptr + t, DIRTY_BIT);
    }
}

// One warp per tile: the raw bit-flag words of every tile, produced by the same tile_rows()
// the SpMV kernels use (exposed for parity against the reference's words).
template <int S>
__global__ void k_bitflags(const int* __restrict__ row_ptr, int m, int nnz, int ntiles,
                           const uint32_t* __restrict__ tile_ptr, uint32_t* __restrict__ words) {
    __shared__ uint32_t s_words[8][32];
    __shared__ int s_rowof[8][32 * S];
    const int warp = threadIdx.x >> 5;
    const int t = blockIdx.x * 8 + warp;
    if (t >= ntiles) return;
    const uint32_t tp0 = tile_ptr[t], tp1 = tile_ptr[t + 1];
    const int lo = (int)(tp0 & ROW_MASK);
    const RowBatch rb = prefetch_rows(row_ptr, m, lo);
    const uint32_t w = tile_rows<S, double>(row_ptr, m, t * 32 * S, lo, (int)(tp1 & ROW_MASK), rb,
                                            s_words[warp], s_rowof[warp], nullptr);
    words[(size_t)t * 32 + lane_id()] = w;
    (void)nnz;
}

// CSR validation: row_ptr[0] == 0, non-decreasing, row_ptr[m] == nnz, 0 <= col < n.
// Any violation sets a bit in *bad (bit0 row_ptr, bit1 col_idx).
__global__ void k_validate(const int* __restrict__ row_ptr, const int* __restrict__ col, int m,
                           int n, int nnz, uint32_t* bad) {
    // 64-bit counters: m and nnz may be within one stride of 2^31
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid == 0 && (row_ptr[0] != 0 || row_ptr[m] != nnz)) atomicOr(bad, 1u);
    for (long long r = tid; r < m; r += stride)
        if (__ldg(row_ptr + r) > __ldg(row_ptr + r + 1)) atomicOr(bad, 1u);
    for (long long e = tid; e < nnz; e += stride) {
        const int c = __ldg(col + e);
        if (c < 0 || c >= n) atomicOr(bad, 2u);
    }
}


int device_sm_count() {
    static std::atomic<int> cache[64];  // zero: not looked up yet
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
    if (dev < 64) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c > 0) return c;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        return 1;
    if (dev < 64) cache[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

int grid_for(long long work, int threads, int cap_per_sm) {
    long long g = (work + threads - 1) / threads;
    const long long cap = (long long)cap_per_sm * device_sm_count();
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

cudaError_t launch_partition(const int* row_ptr, int m, int nnz, int tile, uint32_t* tile_ptr,
                             cudaStream_t st) {
    const int nt = num_tiles(nnz, tile);
    k_tile_rows<<<(unsigned)(((long long)nt + 1 + 255) / 256), 256, 0, st>>>(row_ptr, m, nnz, tile, nt,
                                                                tile_ptr);
    if (m > 0 && nt > 0)
        k_mark_dirty<<<grid_for(m, 256, 16), 256, 0, st>>>(row_ptr, m, tile, nt, tile_ptr);
    return cudaGetLastError();
}

cudaError_t launch_bitflags(const int* row_ptr, int m, int nnz, int seg, const uint32_t* tile_ptr,
                            uint32_t* words, cudaStream_t st) {
    const int nt = num_tiles(nnz, 32 * seg);
    if (nt == 0) return cudaSuccess;
    const int blocks = (nt + 7) / 8;
    switch (seg) {
        case 1: k_bitflags<1><<<blocks, 256, 0, st>>>(row_ptr, m, nnz, nt, tile_ptr, words); break;
        case 2: k_bitflags<2><<<blocks, 256, 0, st>>>(row_ptr, m, nnz, nt, tile_ptr, words); break;
        case 4: k_bitflags<4><<<blocks, 256, 0, st>>>(row_ptr, m, nnz, nt, tile_ptr, words); break;
        case 8: k_bitflags<8><<<blocks, 256, 0, st>>>(row_ptr, m, nnz, nt, tile_ptr, words); break;
        case 16: k_bitflags<16><<<blocks, 256, 0, st>>>(row_ptr, m, nnz, nt, tile_ptr, words); break;
        case 32: k_bitflags<32><<<blocks, 256, 0, st>>>(row_ptr, m, nnz, nt, tile_ptr, words); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Non-empty rows shorter than cw non-zeros.  Only such a row puts two row heads into one
// lane's chunk of cw slots (heads at s and s + len share an aligned chunk only if len < cw), and
// it does so in at most one chunk.
__global__ void k_short_rows(const int* __restrict__ row_ptr, int m, int cw,
                             uint32_t* __restrict__ count) {
    const long long stride = (long long)gridDim.x * blockDim.x;  // 64-bit: m may be near 2^31
    uint32_t c = 0;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < m; r += stride) {
        const int len = __ldg(row_ptr + r + 1) - __ldg(row_ptr + r);
        c += (len > 0 && len < cw) ? 1u : 0u;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(SPMV_FULL_MASK, c, d);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// Locality of the columns for the x gathers, on every step-th non-zero: near when its column is
// within 4 of the previous entry of its row, or of the entry at the same position of the
// previous row (a stencil's neighbour rows reuse the same x lines).
__global__ void k_x_locality(const int* __restrict__ row_ptr, const int* __restrict__ col, int m,
                             int nnz, int step, uint32_t* __restrict__ counts) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    uint32_t seen = 0, near = 0;
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s * step < nnz;
         s += stride) {
        const int j = (int)(s * step);
        // the row of non-zero j: the last r with row_ptr[r] <= j (rows 0..m-1)
        int lo = 0, hi = m - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(row_ptr + mid) <= j)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int r = lo;
        const int start = __ldg(row_ptr + r);
        const int c = __ldg(col + j);
        bool is_near = false;
        if (j > start) is_near = abs(c - __ldg(col + j - 1)) <= 4;
        if (!is_near && r > 0) {
            const int ps = __ldg(row_ptr + r - 1);
            if (ps + (j - start) < start) is_near = abs(c - __ldg(col + ps + (j - start))) <= 4;
        }
        ++seen;
        near += is_near ? 1u : 0u;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        seen += __shfl_xor_sync(SPMV_FULL_MASK, seen, d);
        near += __shfl_xor_sync(SPMV_FULL_MASK, near, d);
    }
    if ((threadIdx.x & 31) == 0 && seen) {
        atomicAdd(counts, seen);
        atomicAdd(counts + 1, near);
    }
}

cudaError_t launch_x_locality(const int* row_ptr, const int* col, int m, int nnz, int step,
                              uint32_t* counts, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(counts, 0, 2 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    if (m > 0 && nnz > 0 && step > 0) {
        const long long samples = ((long long)nnz + step - 1) / step;
        k_x_locality<<<grid_for(samples, 256, 8), 256, 0, st>>>(row_ptr, col, m, nnz, step,
                                                                       counts);
    }
    return cudaGetLastError();
}

cudaError_t launch_short_rows(const int* row_ptr, int m, int cw, uint32_t* count, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    if (m > 0) k_short_rows<<<grid_for(m, 256, 8), 256, 0, st>>>(row_ptr, m, cw, count);
    return cudaGetLastError();
}

cudaError_t launch_validate(const int* row_ptr, const int* col, int m, int n, int nnz,
                            uint32_t* bad, cudaStream_t st) {
    long long work = (long long)(m > nnz ? m : nnz);
    k_validate<<<grid_for(work, 256, 8), 256, 0, st>>>(row_ptr, col, m, n, nnz, bad);
    return cudaGetLastError();
}

}  // namespace spmv
