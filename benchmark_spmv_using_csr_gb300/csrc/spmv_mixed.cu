// spmv_mixed.cu -- the mixed-precision form with FP32 storage (policies_mixed.cuh), the dispatch
// of both mixed forms, and the FP64 <-> FP32 / BF16 conversions of the handle API.
#include "policies_mixed.cuh"

namespace spmv {

cudaError_t launch_mixed(const MixedLaunch& l, const TileConfig& cfg, cudaStream_t st) {
    return l.bf16 ? launch_mixed_bf16(l, cfg, st) : launch_mixed_t<float>(l, cfg, st);
}

int mixed_smem_bytes(bool bf16, const TileConfig& cfg) {
    return bf16 ? mixed_bf16_smem_bytes(cfg) : tma_smem_bytes<PolMixed<float>>(cfg);
}

// FP64 -> FP32 or BF16 (round to nearest even), and FP32 -> FP64.
__global__ void k_from_f64(const double* __restrict__ src, void* __restrict__ dst, size_t n,
                           bool to_bf16) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        if (to_bf16)
            static_cast<__nv_bfloat16*>(dst)[i] = __double2bfloat16(src[i]);
        else
            static_cast<float*>(dst)[i] = __double2float_rn(src[i]);
    }
}
__global__ void k_to_f64(const float* __restrict__ src, double* __restrict__ dst, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride)
        dst[i] = (double)src[i];
}

cudaError_t launch_convert_from_f64(const double* src, void* dst, size_t n, bool to_bf16,
                                    cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const int g = grid_for((long long)n, 256, 16);
    k_from_f64<<<(unsigned)g, 256, 0, st>>>(src, dst, n, to_bf16);
    return cudaGetLastError();
}
cudaError_t launch_convert_to_f64(const float* src, double* dst, size_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const int g = grid_for((long long)n, 256, 16);
    k_to_f64<<<(unsigned)g, 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

}  // namespace spmv
