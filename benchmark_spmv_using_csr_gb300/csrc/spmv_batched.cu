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
// records.  The persistent kernel and the calibration are captured once in a CUDA graph and
// replayed by every call (the kernel leaves its ticket at zero for the next launch).
#include <algorithm>
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

// the same gathers from L2 only (ld.global.cg), the batch's plan choice when its columns have no
// locality
__device__ __forceinline__ VecF<1> ld_x_l2(const VecF<1>* p) {
    VecF<1> r;
    asm volatile("ld.global.cg.f32 %0, [%1];" : "=f"(r.v[0]) : "l"(p));
    return r;
}
__device__ __forceinline__ VecF<2> ld_x_l2(const VecF<2>* p) {
    VecF<2> r;
    asm volatile("ld.global.cg.v2.f32 {%0,%1}, [%2];" : "=f"(r.v[0]), "=f"(r.v[1]) : "l"(p));
    return r;
}
__device__ __forceinline__ VecF<4> ld_x_l2(const VecF<4>* p) {
    VecF<4> r;
    asm volatile("ld.global.cg.v4.f32 {%0,%1,%2,%3}, [%4];"
                 : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3])
                 : "l"(p));
    return r;
}
__device__ __forceinline__ VecF<8> ld_x_l2(const VecF<8>* p) {
    VecF<8> r;
    asm volatile("ld.global.cg.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
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

// the persistent kernel for K right-hand sides: register-capped from 4 on.  OH (the one-head
// chunk form) exists for one right-hand side only, whose accumulator is scalar.
template <int K, int S, int WARPS, bool OH, bool XL2>
constexpr auto persistent_kernel() {
    if constexpr (K >= 4)
        return &k_tiles_persistent_capped<PolMixedK<K>, S, WARPS, false, XL2>;
    else
        return &k_tiles_persistent<PolMixedK<K>, S, WARPS, OH && K == 1, XL2>;
}

template <int K, int S, int WARPS, bool OH, bool XL2>
static cudaError_t enqueue_batched(const TileArgs<PolMixedK<K>>& a, int tpw, int nworkers,
                                   int ntiles, int grid, cudaStream_t st) {
    if (nworkers > 0)
        persistent_kernel<K, S, WARPS, OH, XL2>()<<<grid, WARPS * 32, 0, st>>>(a, tpw, nworkers,
                                                                               ntiles);
    const int cb = grid_for(nworkers, 256, 8);
    k_calibrate<PolMixedK<K>><<<cb, 256, 0, st>>>(a.rec_row, a.rec_val, nworkers, a.y, a.tile_ptr,
                                                  a.m, a.err);
    return cudaGetLastError();
}

template <int K, int S, int WARPS, bool OH, bool XL2>
static int persistent_grid() {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, persistent_kernel<K, S, WARPS, OH, XL2>(), WARPS * 32, 0) != cudaSuccess)
        return 0;
    return device_sm_count() * (per_sm > 0 ? per_sm : 1);
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

// The plan's kernel variant: the one-head chunk form (one right-hand side, few short rows) and
// L2-only x gathers (columns without locality), both chosen from counts made on the device.
struct BatchVariant {
    bool one_head = false;
    bool x_l2 = false;
};

template <int K, int S, int WARPS, bool OH, bool XL2>
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
    a.ticket = l.ticket;
    const int nt = num_tiles(l.nnz, 32 * S);
    const int nw = (nt + tpw - 1) / tpw;
    return enqueue_batched<K, S, WARPS, OH, XL2>(a, tpw, nw, nt, grid, st);
}

// dispatch over the variant (one-head form for k = 1 only, L2-only gathers), then S and warps
template <int K, int S, int WARPS>
static cudaError_t enqueue_v(const BatchLaunch& l, const BatchVariant& v, int tpw, int grid,
                             cudaStream_t st) {
    if (K == 1 && v.one_head)
        return v.x_l2 ? enqueue_k<K, S, WARPS, true, true>(l, tpw, grid, st)
                      : enqueue_k<K, S, WARPS, true, false>(l, tpw, grid, st);
    return v.x_l2 ? enqueue_k<K, S, WARPS, false, true>(l, tpw, grid, st)
                  : enqueue_k<K, S, WARPS, false, false>(l, tpw, grid, st);
}
template <int K>
static cudaError_t enqueue_any(const BatchLaunch& l, const TileConfig& c, const BatchVariant& v,
                               int grid, cudaStream_t st) {
    const bool w8 = c.warps_per_cta == 8;
    const int tpw = c.tiles_per_worker;
    switch (c.seg) {
        case 8: return w8 ? enqueue_v<K, 8, 8>(l, v, tpw, grid, st) : enqueue_v<K, 8, 4>(l, v, tpw, grid, st);
        case 16: return w8 ? enqueue_v<K, 16, 8>(l, v, tpw, grid, st) : enqueue_v<K, 16, 4>(l, v, tpw, grid, st);
        case 32: return w8 ? enqueue_v<K, 32, 8>(l, v, tpw, grid, st) : enqueue_v<K, 32, 4>(l, v, tpw, grid, st);
        default: return cudaErrorInvalidValue;
    }
}
static cudaError_t enqueue_batch(const BatchLaunch& l, int k, const TileConfig& c,
                                 const BatchVariant& v, int grid, cudaStream_t st) {
    switch (k) {
        case 1: return enqueue_any<1>(l, c, v, grid, st);
        case 2: return enqueue_any<2>(l, c, v, grid, st);
        case 4: return enqueue_any<4>(l, c, v, grid, st);
        case 8: return enqueue_any<8>(l, c, v, grid, st);
        default: return cudaErrorInvalidValue;
    }
}

template <int K, int S, int WARPS>
static int grid_v(const BatchVariant& v) {
    if (K == 1 && v.one_head)
        return v.x_l2 ? persistent_grid<K, S, WARPS, true, true>()
                      : persistent_grid<K, S, WARPS, true, false>();
    return v.x_l2 ? persistent_grid<K, S, WARPS, false, true>()
                  : persistent_grid<K, S, WARPS, false, false>();
}
template <int K>
static int grid_any(const TileConfig& c, const BatchVariant& v) {
    const bool w8 = c.warps_per_cta == 8;
    switch (c.seg) {
        case 8: return w8 ? grid_v<K, 8, 8>(v) : grid_v<K, 8, 4>(v);
        case 16: return w8 ? grid_v<K, 16, 8>(v) : grid_v<K, 16, 4>(v);
        case 32: return w8 ? grid_v<K, 32, 8>(v) : grid_v<K, 32, 4>(v);
        default: return 0;
    }
}
static int batch_grid(int k, const TileConfig& c, const BatchVariant& v) {
    switch (k) {
        case 1: return grid_any<1>(c, v);
        case 2: return grid_any<2>(c, v);
        case 4: return grid_any<4>(c, v);
        case 8: return grid_any<8>(c, v);
        default: return 0;
    }
}

}  // namespace spmv

using namespace spmv;

struct bhsp_batch {
    int count = 0, k = 1;
    int m = 0, n = 0, nnz = 0;  // totals of the concatenated block-diagonal matrix
    TileConfig cfg{};
    BatchVariant var{};
    int short_rows = 0, x_sampled = 0, x_near = 0;  // the counts the variant came from
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
    cudaError_t e = cudaSuccess;
    {
        // the kernel variant, as for a single matrix's plan: short rows against the chunk
        // width of the batched kernel, and the locality of about 2^20 sampled columns
        const int cw = k == 8 ? 2 : (c.seg == 8 || k == 4) ? 4 : 8;  // chunk_width<S, x entry>
        const int step = nnz_total > (1 << 20) ? nnz_total / (1 << 20) : 1;
        uint32_t* counts = nullptr;
        uint32_t h[3] = {0u, 0u, 0u};
        e = cudaMalloc(&counts, 3 * sizeof(uint32_t));
        if (e == cudaSuccess) e = launch_short_rows(d_row_ptr, m_total, cw, counts, st);
        if (e == cudaSuccess)
            e = launch_x_locality(d_row_ptr, d_col_idx, m_total, nnz_total, step, counts + 1, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, counts, sizeof h, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(counts);
        b->short_rows = (int)h[0];
        b->x_sampled = (int)h[1];
        b->x_near = (int)h[2];
        b->var.one_head = k == 1 && one_head_pays(h[0], nnz_total, cw);
        b->var.x_l2 = x_l2_pays(h[1], h[2]);
    }
    b->grid = e == cudaSuccess ? batch_grid(k, c, b->var) : 0;
    const size_t nw = b->nworkers > 0 ? (size_t)b->nworkers : 1;
    if (e == cudaSuccess && b->grid <= 0) e = cudaErrorInvalidConfiguration;
    if (e == cudaSuccess) e = cudaMalloc(&b->tile_ptr, sizeof(uint32_t) * ((size_t)b->ntiles + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->rec_row, sizeof(int) * nw);
    if (e == cudaSuccess) e = cudaMalloc(&b->rec_val, sizeof(double) * k * nw);
    if (e == cudaSuccess) e = cudaMalloc(&b->err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->ticket, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->err, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->ticket, 0, 2 * sizeof(int), st);
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
        cudaError_t e = enqueue_batch(l, b->k, b->cfg, b->var, b->grid, st);
        return e == cudaSuccess ? BHSPARSE_SUCCESS : batch_cuda(b, e, "batched launch");
    }
    if (!b->exec || b->g_val != d_val || b->g_x != d_x || b->g_y != d_y) {
        // (re)capture the persistent kernel and the calibration
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        cudaStream_t cs = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e != cudaSuccess) return batch_cuda(b, e, "capture stream");
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e2 = enqueue_batch(l, b->k, b->cfg, b->var, b->grid, cs);
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

extern "C" int bhsp_batch_variant(const bhsp_batch* b, int* one_head, int* l2_only) {
    if (!b) return BHSPARSE_INVALID_ARGUMENT;
    if (one_head) *one_head = b->var.one_head ? 1 : 0;
    if (l2_only) *l2_only = b->var.x_l2 ? 1 : 0;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_batch_set_variant(bhsp_batch* b, int one_head, int l2_only) {
    if (!b || one_head < -1 || one_head > 1 || l2_only < -1 || l2_only > 1 ||
        (one_head == 1 && b->k != 1))
        return BHSPARSE_INVALID_ARGUMENT;
    BatchVariant v = b->var;
    if (one_head >= 0) v.one_head = one_head == 1;
    if (l2_only >= 0) v.x_l2 = l2_only == 1;
    const int grid = batch_grid(b->k, b->cfg, v);
    if (grid <= 0) return batch_cuda(b, cudaErrorInvalidConfiguration, "batch variant");
    b->var = v;
    b->grid = grid;
    // the captured graph launches the previous kernel: capture again at the next execute
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    return BHSPARSE_SUCCESS;
}

// ---------------------------------------------------------------------------------------
// Schedule tuner of the batched form
// ---------------------------------------------------------------------------------------
namespace {
struct BatchCand {
    int seg, tpw, warps;
};
// S in {8, 16, 32} x tiles per worker in {1, 2, 4, 8} x warps per CTA in {4, 8}
const BatchCand kBatchCands[] = {
    {8, 1, 4},  {8, 1, 8},  {8, 2, 4},  {8, 2, 8},  {8, 4, 4},  {8, 4, 8},  {8, 8, 4},  {8, 8, 8},
    {16, 1, 4}, {16, 1, 8}, {16, 2, 4}, {16, 2, 8}, {16, 4, 4}, {16, 4, 8}, {16, 8, 4}, {16, 8, 8},
    {32, 1, 4}, {32, 1, 8}, {32, 2, 4}, {32, 2, 8}, {32, 4, 4}, {32, 4, 8}, {32, 8, 4}, {32, 8, 8},
};
constexpr int kNumBatchCands = sizeof(kBatchCands) / sizeof(kBatchCands[0]);
}  // namespace

extern "C" int bhsp_batch_tune_num_candidates(void) { return kNumBatchCands; }

extern "C" int bhsp_batch_tune_candidate(int index, int* seg, int* tiles_per_worker,
                                         int* warps_per_cta) {
    if (index < 0 || index >= kNumBatchCands) return BHSPARSE_INVALID_ARGUMENT;
    if (seg) *seg = kBatchCands[index].seg;
    if (tiles_per_worker) *tiles_per_worker = kBatchCands[index].tpw;
    if (warps_per_cta) *warps_per_cta = kBatchCands[index].warps;
    return BHSPARSE_SUCCESS;
}

extern "C" int bhsp_batch_autotune(int count, int m_total, int n_total, int nnz_total,
                                   const int* d_row_ptr, const int* d_col_idx, int k,
                                   const float* d_val, const float* d_x, float* d_y, int warmup,
                                   int reps, float* ms_out, int* best, void* stream) {
    if (warmup < 0 || reps < 1 || !ms_out) return BHSPARSE_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return BHSPARSE_CUDA_ERROR;
    }
    // a write of twice the L2 size before every timed run (skipped if it cannot be allocated)
    void* flush = nullptr;
    size_t flush_bytes = 0;
    int dev = 0, l2 = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) == cudaSuccess && l2 > 0) {
        flush_bytes = 2 * (size_t)l2;
        if (cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
            flush = nullptr;
            cudaGetLastError();
        }
    }
    int rc = BHSPARSE_SUCCESS, best_i = -1;
    float best_ms = 0.f;
    std::vector<float> t((size_t)reps);
    for (int i = 0; i < kNumBatchCands && rc == BHSPARSE_SUCCESS; ++i) {
        bhsp_batch* b = nullptr;
        rc = bhsp_batch_create(&b, count, m_total, n_total, nnz_total, d_row_ptr, d_col_idx, k,
                               kBatchCands[i].seg, kBatchCands[i].tpw, kBatchCands[i].warps,
                               stream);
        if (rc) break;
        for (int w = 0; w < warmup && rc == 0; ++w) rc = bhsp_batch_execute(b, d_val, d_x, d_y, 1, stream);
        for (int r = 0; r < reps && rc == 0; ++r) {
            if (flush && cudaMemsetAsync(flush, r & 0xff, flush_bytes, st) != cudaSuccess)
                rc = BHSPARSE_CUDA_ERROR;
            if (!rc && cudaEventRecord(e0, st) != cudaSuccess) rc = BHSPARSE_CUDA_ERROR;
            if (!rc) rc = bhsp_batch_execute(b, d_val, d_x, d_y, 1, stream);
            if (!rc && cudaEventRecord(e1, st) != cudaSuccess) rc = BHSPARSE_CUDA_ERROR;
            if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = BHSPARSE_CUDA_ERROR;
            if (!rc && cudaEventElapsedTime(&t[(size_t)r], e0, e1) != cudaSuccess)
                rc = BHSPARSE_CUDA_ERROR;
        }
        if (!rc) rc = bhsp_batch_check(b, stream);
        bhsp_batch_destroy(b);
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
