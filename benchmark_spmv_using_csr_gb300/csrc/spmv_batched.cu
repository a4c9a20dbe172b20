// spmv_batched.cu -- the batched multi-RHS form: many CSR matrices of uneven size, k in
// {1, 2, 4, 8} right-hand sides, FP32 storage with the compensated FP32 arithmetic of the mixed
// form, in one persistent launch replayed from a CUDA graph.  No counterpart in the reference.
//
// The batch is one block-diagonal CSR: the matrices' rows are concatenated (row_ptr carries
// global non-zero offsets) and their column indices are offset into one concatenated x.  x and
// y hold the k right-hand sides interleaved ([row][k]), so one gather brings all k values of an
// x entry (k*4 bytes, one 256-bit load at k = 8).  One tile partition covers the whole batch;
// the per-matrix tile counts are its segments.  A persistent kernel sized to the GPU's resident
// capacity hands out workers (consecutive tile ranges) from a global atomic ticket, so the
// uneven matrices load-balance over the SMs; the calibration kernel then adds the carry
// records.  The ticket reset, the persistent kernel and the calibration are captured once in a
// CUDA graph and replayed by every call.
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/spmv_gb300.h"
#include "internal.h"
#include "tile_kernel.cuh"

namespace spmv {

// ---- k interleaved FP32 values, accumulators and FP64 records ----
template <int K>
struct alignas(4 * K) VecF {
    float v[K];
    __device__ VecF() {}
    __device__ explicit VecF(int z) {
#pragma unroll
        for (int j = 0; j < K; ++j) v[j] = (float)z;
    }
};
template <int K>
struct VecD {
    double v[K];
};
template <int K>
struct AccK {
    float2 v[K];
};

__device__ __forceinline__ VecF<1> ld_x(const VecF<1>* p, uint64_t) {
    VecF<1> r;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(r.v[0]) : "l"(p));
    return r;
}
__device__ __forceinline__ VecF<2> ld_x(const VecF<2>* p, uint64_t) {
    VecF<2> r;
    asm volatile("ld.global.nc.v2.f32 {%0,%1}, [%2];" : "=f"(r.v[0]), "=f"(r.v[1]) : "l"(p));
    return r;
}
__device__ __forceinline__ VecF<4> ld_x(const VecF<4>* p, uint64_t) {
    VecF<4> r;
    asm volatile("ld.global.nc.v4.f32 {%0,%1,%2,%3}, [%4];"
                 : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3])
                 : "l"(p));
    return r;
}
__device__ __forceinline__ VecF<8> ld_x(const VecF<8>* p, uint64_t) {
    VecF<8> r;
    asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3]), "=f"(r.v[4]),
                   "=f"(r.v[5]), "=f"(r.v[6]), "=f"(r.v[7])
                 : "l"(p));
    return r;
}

template <int K>
__device__ __forceinline__ AccK<K> sh_down(const AccK<K>& a, int d) {
    AccK<K> r;
#pragma unroll
    for (int j = 0; j < K; ++j) r.v[j] = sh_down(a.v[j], d);
    return r;
}
template <int K>
__device__ __forceinline__ AccK<K> sh_idx(const AccK<K>& a, int s) {
    AccK<K> r;
#pragma unroll
    for (int j = 0; j < K; ++j) r.v[j] = sh_idx(a.v[j], s);
    return r;
}
template <int K>
__device__ __forceinline__ AccK<K> sh_xor(const AccK<K>& a, int d) {
    AccK<K> r;
#pragma unroll
    for (int j = 0; j < K; ++j) r.v[j] = sh_xor(a.v[j], d);
    return r;
}

// compensated float-float steps (TwoProduct by FMA + Knuth TwoSum), rounded explicitly
__device__ __forceinline__ float2 ffk_add_product(float v, float x, float2 a) {
    const float p = __fmul_rn(v, x);
    const float ep = __fmaf_rn(v, x, -p);
    const float s = __fadd_rn(a.x, p);
    const float bb = __fsub_rn(s, a.x);
    const float es = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    return make_float2(s, __fadd_rn(a.y, __fadd_rn(es, ep)));
}
__device__ __forceinline__ float2 ffk_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float bb = __fsub_rn(s, a.x);
    const float es = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
    return make_float2(s, __fadd_rn(__fadd_rn(a.y, b.y), es));
}

// The mixed-FP32 arithmetic of spmv_mixed.cu applied to k right-hand sides at once.
template <int K>
struct PolMixedK {
    using VS = float;
    using VC = float;
    using XT = VecF<K>;
    using YT = VecF<K>;
    using Acc = AccK<K>;
    using Carry = AccK<K>;
    using Rec = VecD<K>;
    __device__ static Acc zero() {
        Acc r;
#pragma unroll
        for (int j = 0; j < K; ++j) r.v[j] = make_float2(0.f, 0.f);
        return r;
    }
    __device__ static Carry carry_zero() { return zero(); }
    __device__ static Acc fma(float v, const XT& x, const Acc& a) {
        Acc r;
#pragma unroll
        for (int j = 0; j < K; ++j) r.v[j] = ffk_add_product(v, x.v[j], a.v[j]);
        return r;
    }
    __device__ static Acc add(const Acc& a, const Acc& b) {
        Acc r;
#pragma unroll
        for (int j = 0; j < K; ++j) r.v[j] = ffk_add(a.v[j], b.v[j]);
        return r;
    }
    __device__ static Carry carry_from(const Acc& a) { return a; }
    __device__ static Acc carry_to_acc(const Carry& c) { return c; }
    __device__ static Carry carry_add(const Carry& c, const Acc& a) { return add(c, a); }
    __device__ static YT out_acc(const Acc& a) {
        YT r;
#pragma unroll
        for (int j = 0; j < K; ++j) r.v[j] = __fadd_rn(a.v[j].x, a.v[j].y);
        return r;
    }
    __device__ static YT out_carry(const Carry& c) { return out_acc(c); }
    __device__ static Rec rec_from(const Carry& c) {
        Rec r;
#pragma unroll
        for (int j = 0; j < K; ++j) r.v[j] = (double)c.v[j].x + (double)c.v[j].y;
        return r;
    }
    __device__ static Rec rec_add(const Rec& a, const Rec& b) {
        Rec r;
#pragma unroll
        for (int j = 0; j < K; ++j) r.v[j] = a.v[j] + b.v[j];
        return r;
    }
    __device__ static Rec rec_of_y(const YT& y) {
        Rec r;
#pragma unroll
        for (int j = 0; j < K; ++j) r.v[j] = (double)y.v[j];
        return r;
    }
    __device__ static YT out_rec(const Rec& r) {
        YT y;
#pragma unroll
        for (int j = 0; j < K; ++j) y.v[j] = __double2float_rn(r.v[j]);
        return y;
    }
};

// the persistent kernel for K right-hand sides: register-capped from 4 on
template <int K, int S, int WARPS>
constexpr auto persistent_kernel() {
    if constexpr (K >= 4)
        return &k_tiles_persistent_capped<PolMixedK<K>, S, WARPS>;
    else
        return &k_tiles_persistent<PolMixedK<K>, S, WARPS>;
}

template <int K, int S, int WARPS>
static cudaError_t enqueue_batched(const TileArgs<PolMixedK<K>>& a, int tpw, int nworkers,
                                   int ntiles, int* ticket, int grid, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    if (nworkers > 0)
        persistent_kernel<K, S, WARPS>()<<<grid, WARPS * 32, 0, st>>>(a, tpw, nworkers, ntiles,
                                                                     ticket);
    const int cb = grid_for(nworkers, 256, 8);
    k_calibrate<PolMixedK<K>><<<cb, 256, 0, st>>>(a.rec_row, a.rec_val, nworkers, a.y, a.tile_ptr,
                                                  a.m, a.err);
    return cudaGetLastError();
}

template <int K, int S, int WARPS>
static int persistent_grid() {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, persistent_kernel<K, S, WARPS>(), WARPS * 32, 0) != cudaSuccess)
        return 0;
    return sms * (per_sm > 0 ? per_sm : 1);
}

struct BatchLaunch {
    const int* row_ptr;
    const int* col;
    const float* val;
    const void* x;
    void* y;
    const uint32_t* tile_ptr;
    int* rec_row;
    void* rec_val;
    uint32_t* err;
    int* ticket;
    int m, n, nnz;
};

template <int K, int S, int WARPS>
static cudaError_t enqueue_k(const BatchLaunch& l, int tpw, int grid, cudaStream_t st) {
    TileArgs<PolMixedK<K>> a;
    a.row_ptr = l.row_ptr;
    a.col = l.col;
    a.val = l.val;
    a.x = static_cast<const VecF<K>*>(l.x);
    a.y = static_cast<VecF<K>*>(l.y);
    a.tile_ptr = l.tile_ptr;
    a.rec_row = l.rec_row;
    a.rec_val = static_cast<VecD<K>*>(l.rec_val);
    a.err = l.err;
    a.m = l.m;
    a.n = l.n;
    a.nnz = l.nnz;
    a.phase = 3;
    const int nt = num_tiles(l.nnz, 32 * S);
    const int nw = (nt + tpw - 1) / tpw;
    return enqueue_batched<K, S, WARPS>(a, tpw, nw, nt, l.ticket, grid, st);
}

// dispatch over k (1,2,4,8) x S (8,16,32) x warps (4,8)
#define SPMV_BATCH_DISPATCH(FN, K, ...)                                                     \
    switch (K) {                                                                            \
        case 1: return FN<1>(__VA_ARGS__);                                                  \
        case 2: return FN<2>(__VA_ARGS__);                                                  \
        case 4: return FN<4>(__VA_ARGS__);                                                  \
        case 8: return FN<8>(__VA_ARGS__);                                                  \
        default: return cudaErrorInvalidValue;                                              \
    }

template <int K>
static cudaError_t enqueue_any(const BatchLaunch& l, const TileConfig& c, int grid, cudaStream_t st) {
    const bool w8 = c.warps_per_cta == 8;
    switch (c.seg) {
        case 8: return w8 ? enqueue_k<K, 8, 8>(l, c.tiles_per_worker, grid, st) : enqueue_k<K, 8, 4>(l, c.tiles_per_worker, grid, st);
        case 16: return w8 ? enqueue_k<K, 16, 8>(l, c.tiles_per_worker, grid, st) : enqueue_k<K, 16, 4>(l, c.tiles_per_worker, grid, st);
        case 32: return w8 ? enqueue_k<K, 32, 8>(l, c.tiles_per_worker, grid, st) : enqueue_k<K, 32, 4>(l, c.tiles_per_worker, grid, st);
        default: return cudaErrorInvalidValue;
    }
}
static cudaError_t enqueue_batch(const BatchLaunch& l, int k, const TileConfig& c, int grid,
                                 cudaStream_t st) {
    SPMV_BATCH_DISPATCH(enqueue_any, k, l, c, grid, st)
}

template <int K>
static int grid_any(const TileConfig& c) {
    const bool w8 = c.warps_per_cta == 8;
    switch (c.seg) {
        case 8: return w8 ? persistent_grid<K, 8, 8>() : persistent_grid<K, 8, 4>();
        case 16: return w8 ? persistent_grid<K, 16, 8>() : persistent_grid<K, 16, 4>();
        case 32: return w8 ? persistent_grid<K, 32, 8>() : persistent_grid<K, 32, 4>();
        default: return 0;
    }
}
static int batch_grid(int k, const TileConfig& c) {
    switch (k) {
        case 1: return grid_any<1>(c);
        case 2: return grid_any<2>(c);
        case 4: return grid_any<4>(c);
        case 8: return grid_any<8>(c);
        default: return 0;
    }
}

}  // namespace spmv

using namespace spmv;

struct bhsp_batch {
    int count = 0, k = 1;
    int m = 0, n = 0, nnz = 0;  // totals of the concatenated block-diagonal matrix
    TileConfig cfg{};
    int ntiles = 0, nworkers = 0, grid = 0;
    const int* row_ptr = nullptr;
    const int* col = nullptr;
    uint32_t* tile_ptr = nullptr;
    int* rec_row = nullptr;
    void* rec_val = nullptr;
    uint32_t* err = nullptr;
    int* ticket = nullptr;
    // the graph and the buffers it was captured with
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const float* g_val = nullptr;
    const void* g_x = nullptr;
    void* g_y = nullptr;
    std::string last_error;
};

static void batch_release(bhsp_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFree(b->tile_ptr);
    cudaFree(b->rec_row);
    cudaFree(b->rec_val);
    cudaFree(b->err);
    cudaFree(b->ticket);
    b->exec = nullptr;
    b->graph = nullptr;
}

static int batch_cuda(bhsp_batch* b, cudaError_t e, const char* what) {
    b->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? BHSPARSE_OUT_OF_MEMORY : BHSPARSE_CUDA_ERROR;
}

extern "C" int bhsp_batch_create(bhsp_batch** out, int count, int m_total, int n_total,
                                 int nnz_total, const int* d_row_ptr, const int* d_col_idx, int k,
                                 int seg, int tiles_per_worker, int warps_per_cta, void* stream) {
    if (!out) return BHSPARSE_INVALID_ARGUMENT;
    *out = nullptr;
    if (count < 1 || m_total < 1 || n_total < 1 || nnz_total < 0 || nnz_total > BHSP_MAX_NNZ ||
        !d_row_ptr || (nnz_total > 0 && !d_col_idx) || (k != 1 && k != 2 && k != 4 && k != 8))
        return BHSPARSE_INVALID_ARGUMENT;
    if ((long long)m_total * k > 0x7fffffffLL || (long long)n_total * k > 0x7fffffffLL)
        return BHSPARSE_INVALID_ARGUMENT;
    TileConfig c;
    // default schedule: S = 16, except S = 32 for 4 right-hand sides (+1.7 % on the batched workload)
    c.seg = seg > 0 ? seg : (k == 4 ? 32 : 16);
    c.tiles_per_worker = tiles_per_worker > 0 ? tiles_per_worker : 4;
    c.warps_per_cta = warps_per_cta > 0 ? warps_per_cta : 4;
    c.stages = 0;
    if ((c.seg != 8 && c.seg != 16 && c.seg != 32) || (c.warps_per_cta != 4 && c.warps_per_cta != 8))
        return BHSPARSE_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(d_col_idx) % 32 != 0) return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = bhsp_validate_csr(d_row_ptr, d_col_idx, m_total, n_total, nnz_total, stream);
    if (rc) return rc;
    bhsp_batch* b = new bhsp_batch;
    b->count = count;
    b->k = k;
    b->m = m_total;
    b->n = n_total;
    b->nnz = nnz_total;
    b->cfg = c;
    b->row_ptr = d_row_ptr;
    b->col = d_col_idx;
    b->ntiles = num_tiles(nnz_total, 32 * c.seg);
    b->nworkers = (b->ntiles + c.tiles_per_worker - 1) / c.tiles_per_worker;
    b->grid = batch_grid(k, c);
    cudaError_t e = cudaSuccess;
    const size_t nw = b->nworkers > 0 ? (size_t)b->nworkers : 1;
    if (b->grid <= 0) e = cudaErrorInvalidConfiguration;
    if (e == cudaSuccess) e = cudaMalloc(&b->tile_ptr, sizeof(uint32_t) * ((size_t)b->ntiles + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->rec_row, sizeof(int) * nw);
    if (e == cudaSuccess) e = cudaMalloc(&b->rec_val, sizeof(double) * k * nw);
    if (e == cudaSuccess) e = cudaMalloc(&b->err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->ticket, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->err, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = launch_partition(d_row_ptr, m_total, nnz_total, 32 * c.seg, b->tile_ptr, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        rc = batch_cuda(b, e, "batch setup");
        batch_release(b);
        delete b;
        return rc;
    }
    *out = b;
    return BHSPARSE_SUCCESS;
}

static BatchLaunch batch_launch(bhsp_batch* b, const float* val, const void* x, void* y) {
    BatchLaunch l;
    l.row_ptr = b->row_ptr;
    l.col = b->col;
    l.val = val;
    l.x = x;
    l.y = y;
    l.tile_ptr = b->tile_ptr;
    l.rec_row = b->rec_row;
    l.rec_val = b->rec_val;
    l.err = b->err;
    l.ticket = b->ticket;
    l.m = b->m;
    l.n = b->n;
    l.nnz = b->nnz;
    return l;
}

extern "C" int bhsp_batch_execute(bhsp_batch* b, const float* d_val, const float* d_x, float* d_y,
                                  int use_graph, void* stream) {
    if (!b || !d_y || (b->nnz > 0 && (!d_val || !d_x))) return BHSPARSE_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(d_val) % 32 != 0 ||
        reinterpret_cast<uintptr_t>(d_x) % (4 * b->k) != 0 || reinterpret_cast<uintptr_t>(d_y) % (4 * b->k) != 0)
        return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const BatchLaunch l = batch_launch(b, d_val, d_x, d_y);
    if (!use_graph) {
        cudaError_t e = enqueue_batch(l, b->k, b->cfg, b->grid, st);
        return e == cudaSuccess ? BHSPARSE_SUCCESS : batch_cuda(b, e, "batched launch");
    }
    if (!b->exec || b->g_val != d_val || b->g_x != d_x || b->g_y != d_y) {
        // (re)capture the ticket reset, the persistent kernel and the calibration
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        cudaStream_t cs = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e != cudaSuccess) return batch_cuda(b, e, "capture stream");
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e2 = enqueue_batch(l, b->k, b->cfg, b->grid, cs);
            e = cudaStreamEndCapture(cs, &b->graph);
            if (e == cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess) return batch_cuda(b, e, "graph capture");
        b->g_val = d_val;
        b->g_x = d_x;
        b->g_y = d_y;
    }
    cudaError_t e = cudaGraphLaunch(b->exec, st);
    return e == cudaSuccess ? BHSPARSE_SUCCESS : batch_cuda(b, e, "graph launch");
}

extern "C" int bhsp_batch_check(bhsp_batch* b, void* stream) {
    if (!b) return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, b->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return batch_cuda(b, e, "batch check");
    if (h) {
        cudaMemsetAsync(b->err, 0, sizeof(uint32_t), st);
        cudaStreamSynchronize(st);
        char buf[96];
        snprintf(buf, sizeof buf, "device-side check failed (error word 0x%x)", h);
        b->last_error = buf;
        return BHSPARSE_DEVICE_CHECK_FAILED;
    }
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_batch_info(const bhsp_batch* b, int* ntiles, int* nworkers, int* grid,
                               int* launches) {
    if (!b) return BHSPARSE_INVALID_ARGUMENT;
    if (ntiles) *ntiles = b->ntiles;
    if (nworkers) *nworkers = b->nworkers;
    if (grid) *grid = b->grid;
    if (launches) *launches = b->nworkers > 0 ? 2 : 1;
    return BHSPARSE_SUCCESS;
}

extern "C" const char* bhsp_batch_last_error(const bhsp_batch* b) {
    return b ? b->last_error.c_str() : "null batch";
}

extern "C" void bhsp_batch_destroy(bhsp_batch* b) {
    if (!b) return;
    batch_release(b);
    delete b;
}
