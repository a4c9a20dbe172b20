// spmv_plain_f32.cu -- the plain FP32 form (USE_DOUBLE=0): kernels of policies_plain.cuh
// instantiated for PolF32.
#include "policies_plain.cuh"

namespace spmv {

cudaError_t launch_plain_f32(const PlainLaunch& a, const TileConfig& cfg, cudaStream_t st) {
    return launch_plain_any<PolF32>(a, cfg, st);
}

int plain_f32_smem_bytes(const TileConfig& cfg) { return tma_smem_bytes<PolF32>(cfg); }

}  // namespace spmv
