// common.cuh -- shared device helpers for the GB300 speculative segmented-sum SpMV.
//
// Streaming loads use 256-bit vector loads (ld.global.v4.f64 / v8.b32, sm_100+) with an
// L2 evict-first policy, so that the val / col_idx stream does not push x out of L2;
// x is gathered through the read-only path (ld.global.nc) with an L2 evict-last policy.
#pragma once
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#define SPMV_FULL_MASK 0xffffffffu

namespace spmv {

// Error word bits set by kernels (read back by the host; no __trap anywhere).
enum : uint32_t {
    ERR_NONE = 0,
    ERR_BAD_TILE = 1u << 0,      // a tile row span that cannot come from a valid row_ptr
    ERR_LIST_OVERFLOW = 1u << 1, // more non-empty rows in a dirty tile span than fit in shared memory
    ERR_QUEUE = 1u << 2,         // batched work queue gave out an index out of range
    ERR_WAIT_TIMEOUT = 1u << 3,  // an mbarrier wait ran out of its iteration budget
};

// ---- shared-memory addresses, mbarriers and bulk (TMA) copies ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// make barrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// order this thread's earlier generic-proxy shared-memory accesses before later TMA writes
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait for phase `parity` of the barrier with a bounded number of polls; false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < (1 << 22); ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// 1D bulk copy global -> shared, completing on an mbarrier (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                         uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
        " [%0], [%1], %2, [%3], %4;" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// Cache treatment of the two access streams (compile-time):
//   1: no L2 policy on either (the val / col stream's whole-sector loads skip L1 allocation) --
//      the default: on
//      GB300 it is the fastest on both benchmark matrices (27-point stencil +6 % over 0)
//   0: val/col stream with an L2 evict-first policy, x gathers with an L2 evict-last policy
//   2: evict-first on the stream only
//   3: as 0, plus a 256-byte L2 prefetch hint on the stream
#ifndef SPMV_CACHE_MODE
#define SPMV_CACHE_MODE 1
#endif
#if SPMV_CACHE_MODE == 1
#define SPMV_STREAM_HINT ""
#elif SPMV_CACHE_MODE == 3
#define SPMV_STREAM_HINT ".L2::cache_hint.L2::256B"
#else
#define SPMV_STREAM_HINT ".L2::cache_hint"
#endif
#if SPMV_CACHE_MODE == 1 || SPMV_CACHE_MODE == 2
#define SPMV_X_HINT ""
#else
#define SPMV_X_HINT ".L2::cache_hint"
#endif

// ---- 256-bit streaming loads (address must be 32-byte aligned) ----
__device__ __forceinline__ void ld_stream_f64x4(const double* p, uint64_t pol, double (&v)[4]) {
#if SPMV_CACHE_MODE == 1
    (void)pol;
    asm volatile("ld.global.nc.L1::no_allocate.v4.f64 {%0,%1,%2,%3}, [%4];"
                 : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3])
                 : "l"(p));
#else
    asm volatile("ld.global.nc.L1::no_allocate" SPMV_STREAM_HINT ".v4.f64 {%0,%1,%2,%3}, [%4], %5;"
                 : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3])
                 : "l"(p), "l"(pol));
#endif
}
__device__ __forceinline__ void ld_stream_b32x8(const void* p, uint64_t pol, uint32_t (&v)[8]) {
#if SPMV_CACHE_MODE == 1
    (void)pol;
    asm volatile("ld.global.nc.L1::no_allocate.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                   "=r"(v[7])
                 : "l"(p));
#else
    asm volatile("ld.global.nc.L1::no_allocate" SPMV_STREAM_HINT
                 ".v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                   "=r"(v[7])
                 : "l"(p), "l"(pol));
#endif
}
// 128-bit and 64-bit stream loads serve chunks narrower than a 32-byte sector: the same lane's
// next chunk reads the other half (or quarters) of the sector, so these loads allocate in L1
// and that next read hits there instead of fetching the sector from L2 a second time (column
// indices at S = 8, FP32 / BF16 values at S = 8, BF16 values at S = 16, the batched form's
// column indices at 8 right-hand sides).
// 128-bit stream load (16-byte aligned)
__device__ __forceinline__ void ld_stream_b32x4(const void* p, uint64_t pol, uint32_t (&v)[4]) {
#if SPMV_CACHE_MODE == 1
    (void)pol;
    asm volatile("ld.global.nc.v4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                 : "l"(p));
#else
    asm volatile("ld.global.nc.L1::no_allocate" SPMV_STREAM_HINT ".v4.b32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                 : "l"(p), "l"(pol));
#endif
}

// 64-bit stream load (8-byte aligned)
__device__ __forceinline__ void ld_stream_b32x2(const void* p, uint64_t pol, uint32_t (&v)[2]) {
#if SPMV_CACHE_MODE == 1
    (void)pol;
    asm volatile("ld.global.nc.v2.b32 {%0,%1}, [%2];" : "=r"(v[0]), "=r"(v[1]) : "l"(p));
#else
    asm volatile("ld.global.nc.L1::no_allocate" SPMV_STREAM_HINT ".v2.b32 {%0,%1}, [%2], %3;"
                 : "=r"(v[0]), "=r"(v[1])
                 : "l"(p), "l"(pol));
#endif
}

// N consecutive 32-bit words with one vector load (N = 2, 4 or 8)
__device__ __forceinline__ void ld_stream_u32s(const void* p, uint64_t pol, uint32_t (&v)[8]) {
    ld_stream_b32x8(p, pol, v);
}
__device__ __forceinline__ void ld_stream_u32s(const void* p, uint64_t pol, uint32_t (&v)[4]) {
    ld_stream_b32x4(p, pol, v);
}
__device__ __forceinline__ void ld_stream_u32s(const void* p, uint64_t pol, uint32_t (&v)[2]) {
    ld_stream_b32x2(p, pol, v);
}

// ---- x gathers: read-only path, kept in L2 ----
__device__ __forceinline__ double ld_x(const double* p, uint64_t pol) {
    double v;
#if SPMV_CACHE_MODE == 1 || SPMV_CACHE_MODE == 2
    (void)pol;
    asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
#else
    asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
#endif
    return v;
}
__device__ __forceinline__ float ld_x(const float* p, uint64_t pol) {
    float v;
#if SPMV_CACHE_MODE == 1 || SPMV_CACHE_MODE == 2
    (void)pol;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
#else
    asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
#endif
    return v;
}
// x gathers cached in L2 only (ld.global.cg): for matrices whose columns have no locality, where
// L1 allocation buys almost no hits (the power-law matrix: 6.6 %) and costs L1 throughput.  x is
// not written while a kernel runs, so the coherent path reads the same values.
__device__ __forceinline__ double ld_x_l2(const double* p) {
    double v;
    asm volatile("ld.global.cg.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ float ld_x_l2(const float* p) {
    float v;
    asm volatile("ld.global.cg.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}

// ---- warp helpers ----
template <typename T>
__device__ __forceinline__ T shfl_down(T v, int d) { return __shfl_down_sync(SPMV_FULL_MASK, v, d); }
template <typename T>
__device__ __forceinline__ T shfl_idx(T v, int src) { return __shfl_sync(SPMV_FULL_MASK, v, src); }

// exclusive prefix sum of an int over the warp
__device__ __forceinline__ int warp_exclusive_scan(int v) {
    const int lane = lane_id();
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(SPMV_FULL_MASK, x, d);
        if (lane >= d) x += y;
    }
    return x - v;
}

// longest run of zero bits in a 32-bit mask (warp-uniform integer work)
__device__ __forceinline__ int longest_zero_run(uint32_t mask) {
    uint32_t y = ~mask;
    int r = 0;
    while (y) {
        y &= y << 1;
        ++r;
    }
    return r;
}

}  // namespace spmv
