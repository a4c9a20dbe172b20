// noalloc.cu -- plain FP64 y = A.x for callers that cannot allocate device memory.
//
// The kernels are the library's own (partition, tile kernel, calibration); only their scratch
// moves: tile_ptr, the per-worker carry records and the error word live in one file-scope
// device array of BHSP_NOALLOC_SCRATCH_BYTES instead of buffers from cudaMalloc.  Every GPU
// that loads the library holds that array until the process exits.
#include <cstdint>
#include <mutex>

#include "../../include/spmv_gb300.h"
#include "internal.h"

namespace {

using namespace spmv;

static __device__ __align__(256) unsigned char g_scratch[BHSP_NOALLOC_SCRATCH_BYTES];

// Device address of g_scratch, looked up once per device (host code may not use the symbol
// itself: on the host it names a stand-in, not device memory).
std::mutex g_mu;
void* g_scratch_addr[64] = {};

struct Layout {
    size_t err, ticket, tile_ptr, rec_row, rec_val, total;
};

size_t up256(size_t v) { return (v + 255) & ~size_t(255); }

// Fixed schedule of this entry point: 16 non-zeros per lane, 8 tiles per worker, 4 warps.
TileConfig noalloc_config() {
    TileConfig c;
    c.seg = 16;
    c.tiles_per_worker = 8;
    c.warps_per_cta = 4;
    c.stages = 0;
    return c;
}

Layout layout_for(int nnz, const TileConfig& c) {
    const size_t nt = (size_t)num_tiles(nnz, 32 * c.seg);
    const size_t nw = (nt + c.tiles_per_worker - 1) / c.tiles_per_worker;
    Layout L;
    L.err = 0;
    L.ticket = 8;  // two ints beside the error word
    L.tile_ptr = 256;
    L.rec_row = up256(L.tile_ptr + 4 * (nt + 1));
    L.rec_val = up256(L.rec_row + 4 * (nw > 0 ? nw : 1));
    L.total = L.rec_val + 8 * (nw > 0 ? nw : 1);
    return L;
}

}  // namespace

extern "C" int bhsp_spmv_f64_noalloc(const int* d_row_ptr, const int* d_col_idx,
                                     const double* d_val, const double* d_x, double* d_y, int m,
                                     int n, int nnz, int validate, void* stream) {
    if (m < 0 || n < 0 || nnz < 0 || nnz > BHSP_MAX_NNZ || (nnz > 0 && n == 0))
        return BHSPARSE_INVALID_ARGUMENT;
    if (m == 0) return BHSPARSE_SUCCESS;
    if (!d_row_ptr || !d_y || (nnz > 0 && (!d_col_idx || !d_val || !d_x)))
        return BHSPARSE_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(d_val) % 32 != 0 || reinterpret_cast<uintptr_t>(d_col_idx) % 32 != 0)
        return BHSPARSE_INVALID_ARGUMENT;
    const TileConfig cfg = noalloc_config();
    const Layout L = layout_for(nnz, cfg);
    if (L.total > (size_t)BHSP_NOALLOC_SCRATCH_BYTES) return BHSPARSE_NOALLOC_TOO_LARGE;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return BHSPARSE_CUDA_ERROR;
    if (dev < 0 || dev >= 64) return BHSPARSE_INVALID_ARGUMENT;
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return BHSPARSE_CUDA_ERROR;
            g_scratch_addr[dev] = p;
        }
        base = static_cast<unsigned char*>(g_scratch_addr[dev]);
    }
    uint32_t* err = reinterpret_cast<uint32_t*>(base + L.err);
    uint32_t* tile_ptr = reinterpret_cast<uint32_t*>(base + L.tile_ptr);
    int* rec_row = reinterpret_cast<int*>(base + L.rec_row);
    double* rec_val = reinterpret_cast<double*>(base + L.rec_val);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t h = 0;

    if (validate) {  // optional CSR check, synchronous, through the same error word
        if (cudaMemsetAsync(err, 0, sizeof(uint32_t), st) != cudaSuccess ||
            launch_validate(d_row_ptr, d_col_idx, m, n, nnz, err, st) != cudaSuccess ||
            cudaMemcpyAsync(&h, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return BHSPARSE_CUDA_ERROR;
        if (h) return BHSPARSE_INVALID_CSR;
    }
    // the array keeps the previous call's contents: the error word and the tile kernel's work
    // queue must start at zero (tile_ptr is rewritten in full by the partition, and every
    // worker writes its record); one write covers both
    if (cudaMemsetAsync(err, 0, L.ticket + 2 * sizeof(int), st) != cudaSuccess)
        return BHSPARSE_CUDA_ERROR;
    if (launch_partition(d_row_ptr, m, nnz, 32 * cfg.seg, tile_ptr, st) != cudaSuccess)
        return BHSPARSE_CUDA_ERROR;
    PlainLaunch a;
    a.row_ptr = d_row_ptr;
    a.col = d_col_idx;
    a.val = d_val;
    a.x = d_x;
    a.y = d_y;
    a.tile_ptr = tile_ptr;
    a.rec_row = rec_row;
    a.rec_val = rec_val;
    a.err = err;
    a.m = m;
    a.n = n;
    a.nnz = nnz;
    a.phase = 3;
    a.ticket = reinterpret_cast<int*>(base + L.ticket);
    if (launch_plain_f64(a, cfg, st) != cudaSuccess) return BHSPARSE_CUDA_ERROR;
    if (cudaMemcpyAsync(&h, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return BHSPARSE_CUDA_ERROR;
    return h ? BHSPARSE_DEVICE_CHECK_FAILED : BHSPARSE_SUCCESS;
}
