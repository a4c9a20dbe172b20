// gather_rate.cu -- the random-access ceiling behind the power-law matrix's sector roofline.
//
// Times fully random 8-byte gathers from an L2-resident FP64 vector (n = 4,194,304, the
// power-law matrix's x) with their int32 indices streamed beside them, the access mix of the
// tile kernel on a matrix without column locality:
//   * through the LSU with ld.global.nc (read-only path), ld.global.cg (L2 only) and ld.global;
//   * through the texture pipeline (tex1Dfetch on a linear texture);
//   * through the tensor unit: cp.async.bulk.tensor.2d ... tile::gather4 (x viewed as rows of 32
//     or 16 bytes, one-row boxes, four rows per instruction) into an NSTAGE-deep ring of
//     128-byte-aligned shared-memory slots per warp, every mbarrier wait bounded;
//   * through both at once: in every CTA some warps gather through the LSU and the others
//     through the tensor unit, over disjoint shares of the indices;
// and host <-> device copies of x's size: cudaMemcpyAsync against a copy kernel, over pinned
// (mapped) memory and over pageable memory (the kernel only where the device reads pageable
// memory through the host's page tables).  Prints one line per case.  Built and run by
// `python -m benchmark_spmv_using_csr_gb300.probes`.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define CK(x)                                                                         \
    do {                                                                              \
        cudaError_t e_ = (x);                                                         \
        if (e_ != cudaSuccess) {                                                      \
            std::printf("error %s: %s\n", #x, cudaGetErrorString(e_));                \
            std::exit(1);                                                             \
        }                                                                             \
    } while (0)

__device__ __forceinline__ uint32_t mix32(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (uint32_t)(z ^ (z >> 31));
}
__global__ void k_fill_idx(int* idx, long long count, int n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        idx[i] = (int)(mix32((uint64_t)i) % (uint32_t)n);
}
__global__ void k_fill_x(double* x, int n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        x[i] = (double)(i & 1023) * 0.5;
}

template <int MODE>
__device__ __forceinline__ double load_x(const double* p) {
    double v;
    if (MODE == 0)
        asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
    else if (MODE == 1)
        asm volatile("ld.global.cg.f64 %0, [%1];" : "=d"(v) : "l"(p));
    else
        asm volatile("ld.global.f64 %0, [%1];" : "=d"(v) : "l"(p));
    return v;
}

// LSU gathers: every thread keeps 8 in flight; the index reads are coalesced.  out has one
// entry per thread of the grid.
template <int MODE>
__global__ void __launch_bounds__(256) k_gather(const int* __restrict__ idx,
                                                const double* __restrict__ x, long long count,
                                                double* out) {
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    double s = 0.0;
    for (long long i = tid; i < count; i += 8 * stride) {
        int c[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const long long k = i + j * stride;
            c[j] = k < count ? __ldg(idx + k) : -1;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (c[j] >= 0) s += load_x<MODE>(x + c[j]);
    }
    out[tid] = s;
}

// Texture gathers: x bound as a linear 1D texture of int2 texels (one FP64 each), fetched with
// tex1Dfetch through the texture pipeline.
__global__ void __launch_bounds__(256) k_gather_tex(const int* __restrict__ idx,
                                                    cudaTextureObject_t tex, long long count,
                                                    double* out) {
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    double s = 0.0;
    for (long long i = tid; i < count; i += 8 * stride) {
        int c[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const long long k = i + j * stride;
            c[j] = k < count ? __ldg(idx + k) : -1;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (c[j] >= 0) {
                const int2 v = tex1Dfetch<int2>(tex, c[j]);
                s += __hiloint2double(v.y, v.x);
            }
    }
    out[tid] = s;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (int i = 0; i < (1 << 22); ++i)
        if (mbar_try(bar, parity)) return true;
    return false;
}

// TMA gathers.  A warp handles chunks of 32 indices (chunk g = gw, gw + W, ...), each into one
// stage of its ring: 8 gather4 copies of 4 rows, one per lane 0..7, slots G4 bytes apart
// (128-byte aligned); lane l's row lands at (l/4)*G4 + (l%4)*ROWB.  Returns the lane's sum.
template <int ROWB, int NST>
__device__ double tma_gather_warp(const CUtensorMap& map, const int* __restrict__ idx,
                                  long long nchunks, long long gw, long long W,
                                  unsigned char* ring, uint64_t* bar, unsigned* err) {
    constexpr int G4 = 4 * ROWB > 128 ? 4 * ROWB : 128;
    constexpr int STAGE = 8 * G4;
    constexpr int EPR = ROWB / 8;
    const int lane = threadIdx.x & 31;
    if (lane == 0)
        for (int s = 0; s < NST; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar + s))
                         : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncwarp();
    auto issue = [&](long long g, int s) {
        const int c = __ldg(idx + g * 32 + lane);
        const int r = c / EPR;
        if (lane == 0)
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                             smem_addr(bar + s)),
                         "r"(32 * ROWB)
                         : "memory");
        __syncwarp();
        const int base = (lane & 7) * 4;
        const int r0 = __shfl_sync(0xffffffffu, r, base), r1 = __shfl_sync(0xffffffffu, r, base + 1);
        const int r2 = __shfl_sync(0xffffffffu, r, base + 2), r3 = __shfl_sync(0xffffffffu, r, base + 3);
        if (lane < 8)
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cta.global.tile::gather4.mbarrier::complete_tx::"
                "bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(
                    smem_addr(ring + s * STAGE + lane * G4)),
                "l"(reinterpret_cast<uint64_t>(&map)), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3),
                "r"(smem_addr(bar + s))
                : "memory");
        return c;
    };
    int cs[NST];
#pragma unroll
    for (int s = 0; s < NST; ++s) {
        cs[s] = 0;
        if (gw + (long long)s * W < nchunks) cs[s] = issue(gw + (long long)s * W, s);
    }
    double acc = 0.0;
    uint32_t phase = 0;
    int s = 0;
    long long g = gw;
    bool timed_out = false;
    for (; g < nchunks; g += W) {
        if (!mbar_wait(bar + s, phase)) {
            timed_out = true;
            break;
        }
        const double* row =
            reinterpret_cast<const double*>(ring + s * STAGE + (lane >> 2) * G4 + (lane & 3) * ROWB);
        acc += row[cs[s] % EPR];
        __syncwarp();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const long long gn = g + (long long)NST * W;
        if (gn < nchunks) cs[s] = issue(gn, s);
        if (++s == NST) {
            s = 0;
            phase ^= 1u;
        }
    }
    if (timed_out) {  // record it, then wait (bounded) for every copy still in flight
        if (lane == 0) atomicOr(err, 1u);
        for (int k = 0; k < NST && g + (long long)k * W < nchunks; ++k) {
            mbar_wait(bar + s, phase);
            if (++s == NST) {
                s = 0;
                phase ^= 1u;
            }
        }
    }
    return acc;
}

// Shared memory of TW warps' rings (NST stages of 8 * G4 bytes) and their mbarriers, 1024-byte
// aligned inside the dynamic allocation.
template <int ROWB, int NST>
__device__ __forceinline__ void tma_ring(unsigned char* smem_raw, int tw, int TW,
                                         unsigned char** ring, uint64_t** bar) {
    constexpr int G4 = 4 * ROWB > 128 ? 4 * ROWB : 128;
    constexpr int STAGE = 8 * G4;
    const uint32_t raw = smem_addr(smem_raw);
    unsigned char* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    *ring = smem + tw * (NST * STAGE);
    *bar = reinterpret_cast<uint64_t*>(smem + TW * NST * STAGE) + tw * NST;
}

// Every warp gathers through the tensor unit.
template <int ROWB, int NST, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    k_gather4(const __grid_constant__ CUtensorMap map, const int* __restrict__ idx,
              long long nchunks, double* out, unsigned* err) {
    extern __shared__ unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5;
    unsigned char* ring;
    uint64_t* bar;
    tma_ring<ROWB, NST>(smem_raw, warp, WARPS, &ring, &bar);
    const long long gw = (long long)blockIdx.x * WARPS + warp;
    out[gw * 32 + (threadIdx.x & 31)] = tma_gather_warp<ROWB, NST>(
        map, idx, nchunks, gw, (long long)gridDim.x * WARPS, ring, bar, err);
}

// Both paths at once on every SM: per CTA, LW warps gather through the LSU (ld.global.cg) over
// idx[0, count_lsu) and TW warps through the tensor unit over idx[count_lsu, count).
template <int ROWB, int NST, int LW, int TW>
__global__ void __launch_bounds__((LW + TW) * 32)
    k_hybrid(const __grid_constant__ CUtensorMap map, const int* __restrict__ idx,
             const double* __restrict__ x, long long count_lsu, long long nchunks, double* out,
             unsigned* err) {
    extern __shared__ unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5;
    const long long otid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (warp < LW) {
        const long long tid = blockIdx.x * (long long)(LW * 32) + threadIdx.x;
        const long long stride = (long long)gridDim.x * LW * 32;
        double s = 0.0;
        for (long long i = tid; i < count_lsu; i += 8 * stride) {
            int c[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const long long k = i + j * stride;
                c[j] = k < count_lsu ? __ldg(idx + k) : -1;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (c[j] >= 0) s += load_x<1>(x + c[j]);
        }
        out[otid] = s;
        return;
    }
    unsigned char* ring;
    uint64_t* bar;
    tma_ring<ROWB, NST>(smem_raw, warp - LW, TW, &ring, &bar);
    out[otid] = tma_gather_warp<ROWB, NST>(map, idx + count_lsu, nchunks,
                                           (long long)blockIdx.x * TW + (warp - LW),
                                           (long long)gridDim.x * TW, ring, bar, err);
}

__global__ void k_copy(const int4* __restrict__ src, int4* __restrict__ dst, long long n16) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n16;
         i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

static float median_ms(std::vector<float> t) {
    std::sort(t.begin(), t.end());
    return t[t.size() / 2];
}

static const long long kOut = 4ll << 20;  // entries of the output buffer

template <int ROWB>
static bool x_rows_map(PFN_cuTensorMapEncodeTiled_v12000 enc, const double* x, int n,
                       CUtensorMap* map) {
    const cuuint64_t dims[2] = {(cuuint64_t)(ROWB / 8), (cuuint64_t)((long long)n * 8 / ROWB)};
    const cuuint64_t strides[1] = {(cuuint64_t)ROWB};
    const cuuint32_t box[2] = {(cuuint32_t)(ROWB / 8), 1};
    const cuuint32_t es[2] = {1, 1};
    if (enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void*)x, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
        std::printf("gather4 rows=%dB: tensor map rejected\n", ROWB);
        return false;
    }
    return true;
}

// median of 5 timed launches after one untimed
template <class F>
static float time_launch(F launch, cudaEvent_t e0, cudaEvent_t e1) {
    std::vector<float> t;
    for (int rep = 0; rep < 6; ++rep) {
        CK(cudaEventRecord(e0));
        launch();
        CK(cudaEventRecord(e1));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (rep) t.push_back(ms);
    }
    CK(cudaGetLastError());
    return median_ms(t);
}

template <int ROWB, int NST, int WARPS>
static void run_gather4(PFN_cuTensorMapEncodeTiled_v12000 enc, const double* x, int n,
                        const int* idx, long long count, double* out, unsigned* err, int sms,
                        cudaEvent_t e0, cudaEvent_t e1) {
    CUtensorMap map;
    if (!x_rows_map<ROWB>(enc, x, n, &map)) return;
    constexpr int G4 = 4 * ROWB > 128 ? 4 * ROWB : 128;
    const int smem = WARPS * NST * (8 * G4 + 8) + 1024;
    auto kfn = k_gather4<ROWB, NST, WARPS>;
    CK(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, WARPS * 32, smem));
    const int grid = sms * (per_sm > 0 ? per_sm : 1);
    if ((long long)grid * WARPS * 32 > kOut) return;
    CK(cudaMemset(err, 0, sizeof(unsigned)));
    const float ms = time_launch(
        [&] { kfn<<<grid, WARPS * 32, smem>>>(map, idx, count / 32, out, err); }, e0, e1);
    unsigned h = 0;
    CK(cudaMemcpy(&h, err, sizeof h, cudaMemcpyDeviceToHost));
    std::printf("TMA gather4, %2d-byte rows, %2d-stage ring, %d warps x %d CTAs/SM: %7.1f G gathers/s%s\n",
                ROWB, NST, WARPS, per_sm, count / (ms * 1e-3) / 1e9, h ? "  (a wait timed out)" : "");
}

template <int ROWB, int NST, int LW, int TW>
static void run_hybrid(PFN_cuTensorMapEncodeTiled_v12000 enc, const double* x, int n,
                       const int* idx, long long count, double lsu_share, double* out,
                       unsigned* err, int sms, cudaEvent_t e0, cudaEvent_t e1) {
    CUtensorMap map;
    if (!x_rows_map<ROWB>(enc, x, n, &map)) return;
    constexpr int G4 = 4 * ROWB > 128 ? 4 * ROWB : 128;
    const int smem = TW * NST * (8 * G4 + 8) + 1024;
    auto kfn = k_hybrid<ROWB, NST, LW, TW>;
    CK(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, (LW + TW) * 32, smem));
    const int grid = sms * (per_sm > 0 ? per_sm : 1);
    if ((long long)grid * (LW + TW) * 32 > kOut) return;
    const long long count_lsu = (long long)(lsu_share * (double)count) / 32 * 32;
    const long long nchunks = (count - count_lsu) / 32;
    CK(cudaMemset(err, 0, sizeof(unsigned)));
    const float ms = time_launch(
        [&] {
            kfn<<<grid, (LW + TW) * 32, smem>>>(map, idx, x, count_lsu, nchunks, out, err);
        },
        e0, e1);
    unsigned h = 0;
    CK(cudaMemcpy(&h, err, sizeof h, cudaMemcpyDeviceToHost));
    std::printf("LSU + TMA on every SM, %d + %d warps x %d CTAs/SM, %3.0f %% through the LSU: %7.1f G gathers/s%s\n",
                LW, TW, per_sm, 100.0 * lsu_share, (count_lsu + 32 * nchunks) / (ms * 1e-3) / 1e9,
                h ? "  (a wait timed out)" : "");
}

int main() {
    CK(cudaSetDevice(0));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, 0));
    const int sms = prop.multiProcessorCount;
    std::printf("%s, %d SMs, L2 %d MB\n", prop.name, sms, prop.l2CacheSize >> 20);
    const int n = 4194304;
    const long long count = 64ll << 20;
    double *x, *out;
    int* idx;
    unsigned* err;
    CK(cudaMalloc(&x, (size_t)n * 8));
    CK(cudaMalloc(&idx, (size_t)count * 4));
    CK(cudaMalloc(&out, (size_t)kOut * 8));
    CK(cudaMalloc(&err, sizeof(unsigned)));
    k_fill_idx<<<sms * 8, 256>>>(idx, count, n);
    k_fill_x<<<sms * 8, 256>>>(x, n);
    CK(cudaDeviceSynchronize());
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));

    const int grid = sms * 8;  // 311 k threads, each writing one of kOut outputs
    auto lsu = [&](auto kfn, const char* name) {
        const float ms = time_launch([&] { kfn<<<grid, 256>>>(idx, x, count, out); }, e0, e1);
        const double g = count / (ms * 1e-3) / 1e9;
        std::printf("LSU %-13s: %7.1f G gathers/s = %7.1f G sectors/s with the index stream\n",
                    name, g, g * 1.125);
    };
    lsu(k_gather<0>, "ld.global.nc");
    lsu(k_gather<1>, "ld.global.cg");
    lsu(k_gather<2>, "ld.global");
    {
        int max_w = 0;
        CK(cudaDeviceGetAttribute(&max_w, cudaDevAttrMaxTexture1DLinearWidth, 0));
        if (max_w >= n) {
            cudaResourceDesc rd;
            std::memset(&rd, 0, sizeof rd);
            rd.resType = cudaResourceTypeLinear;
            rd.res.linear.devPtr = x;
            rd.res.linear.desc = cudaCreateChannelDesc<int2>();
            rd.res.linear.sizeInBytes = (size_t)n * 8;
            cudaTextureDesc td;
            std::memset(&td, 0, sizeof td);
            td.readMode = cudaReadModeElementType;
            cudaTextureObject_t tex = 0;
            CK(cudaCreateTextureObject(&tex, &rd, &td, nullptr));
            const float ms = time_launch(
                [&] { k_gather_tex<<<grid, 256>>>(idx, tex, count, out); }, e0, e1);
            std::printf("TEX tex1Dfetch   : %7.1f G gathers/s\n", count / (ms * 1e-3) / 1e9);
            CK(cudaDestroyTextureObject(tex));
        } else {
            std::printf("TEX tex1Dfetch   : linear textures of %d texels at most, x has %d\n", max_w, n);
        }
    }

    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q == cudaDriverEntryPointSuccess && fn) {
        auto enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        run_gather4<32, 8, 8>(enc, x, n, idx, count, out, err, sms, e0, e1);
        run_gather4<32, 4, 8>(enc, x, n, idx, count, out, err, sms, e0, e1);
        run_gather4<16, 8, 8>(enc, x, n, idx, count, out, err, sms, e0, e1);
        // the two paths side by side: a share of the gathers through the tensor unit
        for (double f : {1.0, 0.85, 0.75})
            run_hybrid<16, 4, 4, 4>(enc, x, n, idx, count, f, out, err, sms, e0, e1);
    }

    // host <-> device copies of x's 33.5 MB
    const size_t bytes = (size_t)n * 8;
    void *h_a, *h_b, *d_a, *m_a, *m_b;
    CK(cudaHostAlloc(&h_a, bytes, cudaHostAllocMapped));
    CK(cudaHostAlloc(&h_b, bytes, cudaHostAllocMapped));
    CK(cudaMalloc(&d_a, bytes));
    std::memset(h_a, 1, bytes);
    std::memset(h_b, 2, bytes);
    CK(cudaHostGetDevicePointer(&m_a, h_a, 0));
    CK(cudaHostGetDevicePointer(&m_b, h_b, 0));
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    auto copy_rate = [&](auto fn_, const char* name) {
        std::vector<float> t;
        for (int rep = 0; rep < 8; ++rep) {
            CK(cudaEventRecord(e0, st));
            fn_();
            CK(cudaEventRecord(e1, st));
            CK(cudaEventSynchronize(e1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (rep) t.push_back(ms);
        }
        std::printf("%-38s: %6.1f GB/s\n", name, bytes / (median_ms(t) * 1e-3) / 1e9);
    };
    copy_rate([&] { CK(cudaMemcpyAsync(d_a, h_a, bytes, cudaMemcpyHostToDevice, st)); },
              "cudaMemcpyAsync host -> device");
    copy_rate([&] { CK(cudaMemcpyAsync(h_b, d_a, bytes, cudaMemcpyDeviceToHost, st)); },
              "cudaMemcpyAsync device -> host");
    copy_rate([&] { k_copy<<<sms * 4, 512, 0, st>>>((const int4*)m_a, (int4*)d_a, bytes / 16); },
              "copy kernel, mapped host -> device");
    copy_rate([&] { k_copy<<<sms * 4, 512, 0, st>>>((const int4*)d_a, (int4*)m_b, bytes / 16); },
              "copy kernel, device -> mapped host");
    // pageable (malloc'd) host memory: cudaMemcpy stages it through pinned buffers; where the
    // device reads the host's page tables (Grace), a copy kernel reaches it directly
    int pageable = 0, host_tables = 0;
    CK(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, 0));
    CK(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, 0));
    void* p_a = std::malloc(bytes);
    void* p_b = std::malloc(bytes);
    if (p_a && p_b) {
        std::memset(p_a, 3, bytes);
        std::memset(p_b, 4, bytes);
        copy_rate([&] { CK(cudaMemcpyAsync(d_a, p_a, bytes, cudaMemcpyHostToDevice, st)); },
                  "cudaMemcpyAsync pageable -> device");
        copy_rate([&] { CK(cudaMemcpyAsync(p_b, d_a, bytes, cudaMemcpyDeviceToHost, st)); },
                  "cudaMemcpyAsync device -> pageable");
        if (pageable == 1 && host_tables == 1) {
            copy_rate([&] { k_copy<<<sms * 4, 512, 0, st>>>((const int4*)p_a, (int4*)d_a, bytes / 16); },
                      "copy kernel, pageable -> device");
            copy_rate([&] { k_copy<<<sms * 4, 512, 0, st>>>((const int4*)d_a, (int4*)p_b, bytes / 16); },
                      "copy kernel, device -> pageable");
        } else {
            std::printf("no pageable memory access through the host's page tables\n");
        }
    }
    std::free(p_a);
    std::free(p_b);
    CK(cudaFreeHost(h_a));
    CK(cudaFreeHost(h_b));
    CK(cudaFree(d_a));
    CK(cudaFree(x));
    CK(cudaFree(idx));
    CK(cudaFree(out));
    CK(cudaFree(err));
    return 0;
}
