// tensor_map.cu -- host encoding of the tensor maps of the TMA-staged tile kernel.
//
// val and col_idx are viewed as 2D tensors of 128-byte rows (32 u32 words), so that one tile
// of 32*S non-zeros is a box of whole rows for every value type.  The driver entry point is
// looked up once through the runtime (no link against the driver library); encoded maps are
// kept in a small per-thread cache keyed by (base, bytes, box height), since a plan is
// normally run many times on the same buffers.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "internal.h"
#include "tile_kernel_tma.cuh"

namespace spmv {
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

struct MapEntry {
    const void* base;
    long long bytes;
    int box_rows;
    CUtensorMap map;
};
constexpr int kCache = 8;
thread_local MapEntry g_cache[kCache];
thread_local int g_next = 0;

}  // namespace

bool encode_stream_map(const void* base, long long bytes, int box_rows, CUtensorMap* map) {
    const long long rows = bytes / 128;
    if (base == nullptr || rows < 1 || box_rows < 1 || box_rows > 256 ||
        (reinterpret_cast<uintptr_t>(base) & 15u) != 0u)
        return false;
    for (int i = 0; i < kCache; ++i) {
        const MapEntry& e = g_cache[i];
        if (e.base == base && e.bytes == bytes && e.box_rows == box_rows) {
            std::memcpy(map, &e.map, sizeof(CUtensorMap));
            return true;
        }
    }
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (fn == nullptr) return false;
    const cuuint64_t dims[2] = {32, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {128};
    const cuuint32_t box[2] = {32, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUtensorMap m;
    const CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void*>(base), dims,
                          strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    MapEntry& e = g_cache[g_next];
    g_next = (g_next + 1) % kCache;
    e.base = base;
    e.bytes = bytes;
    e.box_rows = box_rows;
    std::memcpy(&e.map, &m, sizeof(CUtensorMap));
    std::memcpy(map, &m, sizeof(CUtensorMap));
    return true;
}

}  // namespace spmv
