// spmv_plain_f64.cu -- the plain FP64 form (USE_DOUBLE=1): kernels of policies_plain.cuh
// instantiated for PolF64.
#include "policies_plain.cuh"

namespace spmv {

cudaError_t launch_plain_f64(const PlainLaunch& a, const TileConfig& cfg, cudaStream_t st) {
    return launch_plain_any<PolF64>(a, cfg, st);
}

int plain_smem_bytes(bool f64, const TileConfig& cfg) {
    return f64 ? tma_smem_bytes<PolF64>(cfg) : plain_f32_smem_bytes(cfg);
}

}  // namespace spmv
