// hostcopy.cu -- host -> device copies of pageable host memory by a kernel.
//
// On a Grace host the GPU reads the CPU's pageable memory coherently through the host's page
// tables (cudaDevAttrPageableMemoryAccess and cudaDevAttrPageableMemoryAccessUsesHostPageTables
// both 1).  Measured on GB300 for 33.5 MB (python -m benchmark_spmv_using_csr_gb300.probes):
//   pageable -> device: copy kernel 197 GB/s, cudaMemcpy (staged by the driver) 168 GB/s;
//   device -> pageable: copy kernel 168 GB/s, cudaMemcpy 182 GB/s;
//   pinned memory: about 205 / 189 GB/s either way.
// So the handle API reads the caller's pageable arrays with the kernel and writes y back with
// cudaMemcpy.  The reference's callers pass plain malloc'd arrays (spmv_cuda/main.cu:745-746).
#include <atomic>

#include "internal.h"

namespace spmv {
namespace {

__global__ void k_copy16(const int4* __restrict__ src, int4* __restrict__ dst, long long n16,
                         const unsigned char* __restrict__ src_tail,
                         unsigned char* __restrict__ dst_tail, int tail) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (long long i = tid; i < n16; i += stride) dst[i] = src[i];
    if (tid < tail) dst_tail[tid] = src_tail[tid];
}

}  // namespace

bool host_direct_access() {
    static std::atomic<int> cache[64];  // 0: not looked up, 1: no, 2: yes
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return false;
    if (dev < 64) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c) return c == 2;
    }
    int pageable = 0, host_tables = 0;
    const bool ok =
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                               dev) == cudaSuccess &&
        pageable == 1 && host_tables == 1;
    if (dev < 64) cache[dev].store(ok ? 2 : 1, std::memory_order_relaxed);
    return ok;
}

bool is_pageable_host(const void* p) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();  // clear the query's error
        return false;
    }
    return attr.type == cudaMemoryTypeUnregistered;
}

cudaError_t host_copy(void* dst, const void* src, size_t bytes, bool device_to_host,
                      cudaStream_t st) {
    if (bytes == 0) return cudaSuccess;
    const bool aligned = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) &
                          15u) == 0u;
    if (device_to_host || !aligned || !host_direct_access() || !is_pageable_host(src))
        return cudaMemcpyAsync(dst, src, bytes,
                               device_to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice,
                               st);
    const long long n16 = (long long)(bytes / 16);
    const int tail = (int)(bytes % 16);
    const int grid = grid_for(n16 > tail ? n16 : tail, 512, 4);
    k_copy16<<<grid, 512, 0, st>>>(static_cast<const int4*>(src), static_cast<int4*>(dst), n16,
                                   static_cast<const unsigned char*>(src) + 16 * n16,
                                   static_cast<unsigned char*>(dst) + 16 * n16, tail);
    return cudaGetLastError();
}

}  // namespace spmv
