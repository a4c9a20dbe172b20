// spmv_mixed_bf16.cu -- the mixed-precision form with BF16 storage: kernels of
// policies_mixed.cuh instantiated for __nv_bfloat16 values.
#include "policies_mixed.cuh"

namespace spmv {

cudaError_t launch_mixed_bf16(const MixedLaunch& l, const TileConfig& cfg, cudaStream_t st) {
    return launch_mixed_t<__nv_bfloat16>(l, cfg, st);
}

int mixed_bf16_smem_bytes(const TileConfig& cfg) { return tma_smem_bytes<PolMixed<__nv_bfloat16>>(cfg); }

}  // namespace spmv
