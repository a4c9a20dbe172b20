// tile_kernel_tma.cuh -- the tile kernel with its val / col_idx stream staged in shared
// memory by 2D tensor (TMA) copies.
//
// Same algorithm and output as k_tiles (tile_kernel.cuh); what changes is how a tile reaches
// the lanes:
//  * val and col_idx are each viewed as a 2D tensor of 128-byte rows; a tile of 32*S
//    non-zeros is a whole number of rows, so one cp.async.bulk.tensor.2d per array moves the
//    tile into a slot of a per-warp ring of NSTAGE slots, completing on the slot's mbarrier.
//    The stream runs NSTAGE-1 tiles ahead of the multiply-adds without holding registers;
//  * the copies use the 128-byte swizzle (16-byte chunk j of row r lands at chunk j ^ (r & 7)),
//    which makes the lanes' 16-byte reads of their contiguous runs (64, 128 or 256 bytes
//    apart) bank-conflict free for runs of up to 128 bytes;
//  * x is gathered one chunk of 8 non-zeros ahead of the fused multiply-adds, across tile
//    boundaries (the next tile's slot is waited for during the current tile's last chunk);
//  * the row of a row head is read from the slot->row map built by tile_rows;
//  * the matrix's last tile, when partial, is staged by guarded loads into the same layout.
// Every mbarrier wait is bounded; a timeout sets ERR_WAIT_TIMEOUT, the warp waits (again
// bounded) for the copies it still has in flight and stops.
#pragma once
#include <cuda.h>

#include <atomic>

#include "tile_kernel.cuh"

namespace spmv {

// The two tensor maps of one launch (val and col_idx as rows of 128 bytes).
struct StreamMaps {
    CUtensorMap val;
    CUtensorMap col;
};

// Host: encode a map over `bytes` bytes at `base` as floor(bytes / 128) rows of 32 u32 words,
// box of `box_rows` rows, 128-byte swizzle (tensor_map.cu).  False if the driver rejects it
// (e.g. a base address that is not 16-byte aligned) or there is no full row.
bool encode_stream_map(const void* base, long long bytes, int box_rows, CUtensorMap* map);

template <typename VS>
__device__ __forceinline__ VS zero_value() { return VS(0.0f); }
template <>
__device__ __forceinline__ __nv_bfloat16 zero_value<__nv_bfloat16>() { return __float2bfloat16(0.0f); }

template <class P, int S, int NSTAGE>
struct TmaLayout {
    using VS = typename P::VS;
    static constexpr int TILE = 32 * S;
    static constexpr int VBYTES = TILE * (int)sizeof(VS);  // one tile of values
    static constexpr int CBYTES = TILE * 4;                // one tile of column indices
    static constexpr int VROWS = VBYTES / 128;             // box heights of the two copies
    static constexpr int CROWS = CBYTES / 128;
    static constexpr int VREG = (VBYTES + 1023) / 1024 * 1024;  // swizzle atoms are 1 KB aligned
    static constexpr int CREG = (CBYTES + 1023) / 1024 * 1024;
    static constexpr int SLOT = VREG + CREG;
    static constexpr int ROWOF = TILE * 4;
    static constexpr int RAW = NSTAGE * SLOT + ROWOF + 128 + NSTAGE * 8;
    static constexpr int WARP_BYTES = (RAW + 1023) / 1024 * 1024;
    static_assert(VBYTES % 128 == 0 && CBYTES % 128 == 0, "a tile is whole 128-byte rows");
    static_assert(VROWS <= 256 && CROWS <= 256, "TMA box height");
};

// 128-byte swizzle of a byte offset inside a 1 KB-aligned region
__device__ __forceinline__ uint32_t swz128(uint32_t o) { return o ^ (((o >> 7) & 7u) << 4); }

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar, uint64_t pol) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        ".L2::cache_hint [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}

// 8 values of one chunk: `off` is the logical byte offset of the chunk in the slot's values
__device__ __forceinline__ void swz_vals8(const unsigned char* base, uint32_t off,
                                          double (&v)[8], const double*) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const double2 d = *reinterpret_cast<const double2*>(base + swz128(off + 16 * i));
        v[2 * i] = d.x;
        v[2 * i + 1] = d.y;
    }
}
__device__ __forceinline__ void swz_vals8(const unsigned char* base, uint32_t off, float (&v)[8],
                                          const float*) {
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const float4 q = *reinterpret_cast<const float4*>(base + swz128(off + 16 * i));
        v[4 * i] = q.x;
        v[4 * i + 1] = q.y;
        v[4 * i + 2] = q.z;
        v[4 * i + 3] = q.w;
    }
}
__device__ __forceinline__ void swz_vals8(const unsigned char* base, uint32_t off, float (&v)[8],
                                          const __nv_bfloat16*) {
    const uint4 q = *reinterpret_cast<const uint4*>(base + swz128(off));
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[2 * i] = __uint_as_float(w[i] << 16);
        v[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
    }
}
__device__ __forceinline__ void swz_cols8(const unsigned char* base, uint32_t off, int (&c)[8]) {
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int4 q = *reinterpret_cast<const int4*>(base + swz128(off + 16 * i));
        c[4 * i] = q.x;
        c[4 * i + 1] = q.y;
        c[4 * i + 2] = q.z;
        c[4 * i + 3] = q.w;
    }
}

// x entries of one 8-slot chunk: through L1, or from L2 only (XL2, the plan's choice for
// columns without locality)
template <bool XL2, typename XT>
__device__ __forceinline__ void gather8(const XT* __restrict__ x, const int (&c)[8], uint64_t pol,
                                        XT (&xv)[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) xv[i] = c[i] >= 0 ? ld_x_sel<XL2>(x + c[i], pol) : XT(0);
}

template <class P, int S, int WARPS, int NSTAGE, bool OH, bool XL2>
__global__ void __launch_bounds__(WARPS * 32, 1)
    k_tiles_tma(TileArgs<P> a, const __grid_constant__ StreamMaps maps, int tpw, int nworkers,
                int ntiles) {
    using L = TmaLayout<P, S, NSTAGE>;
    using VS = typename P::VS;
    using Acc = typename P::Acc;
    using Carry = typename P::Carry;
    using VC = typename P::VC;
    using XT = typename P::XT;
    using YT = typename P::YT;
    constexpr int TILE = 32 * S;
    constexpr int NC = S / 8;
    constexpr uint32_t VRUN = S * sizeof(VS);  // bytes of one lane's values in a tile
    constexpr uint32_t CRUN = S * 4;
    extern __shared__ unsigned char smem_raw[];

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int worker = blockIdx.x * WARPS + warp;
    if (worker >= nworkers) return;
    // the launch reserves 1 KB more than the layout so that the base can be 1 KB aligned
    unsigned char* const smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    unsigned char* const wb = smem + warp * L::WARP_BYTES;
    int* const rowof = reinterpret_cast<int*>(wb + NSTAGE * L::SLOT);
    uint32_t* const words = reinterpret_cast<uint32_t*>(wb + NSTAGE * L::SLOT + L::ROWOF);
    uint64_t* const bars = reinterpret_cast<uint64_t*>(wb + NSTAGE * L::SLOT + L::ROWOF + 128);
    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
        fence_barrier_init();
    }
    __syncwarp();

    const int t_begin = worker * tpw;
    const int t_end = min(t_begin + tpw, ntiles);
    const uint64_t pol_s = policy_evict_first();
    const uint64_t pol_x = policy_evict_last();
    constexpr bool one_head = OH && sizeof(Acc) <= 8;  // the one-head chunk form
    auto is_full = [&](int t) { return (long long)(t + 1) * TILE <= a.nnz; };
    auto vslot = [&](int t) { return wb + ((t - t_begin) % NSTAGE) * L::SLOT; };

    // tensor copies of tile t's values and columns into its slot (full tiles only)
    int issued = t_begin;  // tiles [t_begin, issued) have been issued (or are staged by hand)
    auto issue_next = [&]() {
        const int t = issued;
        if (t >= t_end) return;
        ++issued;
        if (!is_full(t) || lane != 0) return;
        const int s = (t - t_begin) % NSTAGE;
        unsigned char* sl = wb + s * L::SLOT;
        mbar_arrive_expect_tx(&bars[s], (uint32_t)(L::VBYTES + L::CBYTES));
        tma_load_2d(sl, &maps.val, 0, t * L::VROWS, &bars[s], pol_s);
        tma_load_2d(sl + L::VREG, &maps.col, 0, t * L::CROWS, &bars[s], pol_s);
    };
    // make tile t's slot readable: wait for its copies, or stage the partial last tile
    auto ready = [&](int t) -> bool {
        if (is_full(t)) {
            const int s = (t - t_begin) % NSTAGE;
            const uint32_t parity = (uint32_t)((t - t_begin) / NSTAGE) & 1u;
            return mbar_wait_bounded(&bars[s], parity);
        }
        unsigned char* sl = vslot(t);
        const int e0 = t * TILE;
#pragma unroll 4
        for (int k = 0; k < S; ++k) {
            const int e = e0 + lane * S + k;
            const bool in = e < a.nnz;
            *reinterpret_cast<VS*>(sl + swz128(lane * VRUN + k * sizeof(VS))) =
                in ? a.val[e] : zero_value<VS>();
            *reinterpret_cast<int*>(sl + L::VREG + swz128(lane * CRUN + k * 4)) = in ? a.col[e] : -1;
        }
        __syncwarp();
        return true;
    };
    auto gather_chunk = [&](int t, int c, XT (&xv)[8]) {
        int cc[8];
        swz_cols8(vslot(t) + L::VREG, lane * CRUN + c * 32, cc);
        gather8<XL2>(a.x, cc, pol_x, xv);
    };

#pragma unroll
    for (int i = 0; i < NSTAGE - 1; ++i) issue_next();
    int t_fail = -1;  // tile whose wait timed out
    XT xa[8];
    if (!ready(t_begin)) {
        t_fail = t_begin;
    } else {
        gather_chunk(t_begin, 0, xa);
    }

    uint32_t tp0 = __ldg(a.tile_ptr + t_begin);
    uint32_t tp1 = __ldg(a.tile_ptr + t_begin + 1);
    RowBatch rb = prefetch_rows(a.row_ptr, a.m, (int)(tp0 & ROW_MASK));

    int carry_row = -1;
    bool carry_owned = false;
    Carry carry = P::carry_zero();
    Acc dc = P::zero();
    bool dc_active = false;
    bool rec_written = false;
    auto flush = [&](int row, Carry v, bool owned) {
        if (lane == 0) {
            if (owned) {
                store_row(a.y, a.m, row, P::out_carry(v), a.err);
            } else {
                a.rec_row[worker] = row;
                a.rec_val[worker] = P::rec_from(v);
            }
        }
        if (!owned) rec_written = true;
    };

    for (int t = t_begin; t < t_end && t_fail < 0; ++t) {
        issue_next();  // tile t+NSTAGE-1 into the slot that tile t-1 has released
        const int lo = (int)(tp0 & ROW_MASK);
        const int hi = (int)(tp1 & ROW_MASK);
        uint32_t tp2 = 0u;
        RowBatch rbn{0, 0, 0, 0};
        if (t + 1 < t_end) {  // meta of the next tile
            tp2 = __ldg(a.tile_ptr + t + 2);
            rbn = prefetch_rows(a.row_ptr, a.m, hi);
        }
        const uint32_t w = tile_rows<S, YT>(a.row_ptr, a.m, t * TILE, lo, hi, rb, words, rowof, a.y);
        const bool first_head = ((__shfl_sync(SPMV_FULL_MASK, w, 0) >> 31) & 1u) != 0u;
        const uint32_t fmask = __ballot_sync(SPMV_FULL_MASK, w != 0u);

        if (first_head) {
            if (carry_row >= 0) {
                Carry tot = carry;
                if (dc_active) tot = P::carry_add(tot, warp_sum_acc<P>(dc));
                flush(carry_row, tot, carry_owned);
            }
            carry_row = -1;
            carry = P::carry_zero();
            dc = P::zero();
            dc_active = false;
        } else if (carry_row < 0) {
            carry_row = lo;
            carry_owned = false;
            carry = P::carry_zero();
        }
        if (fmask != 0u && dc_active) {
            carry = P::carry_add(carry, warp_sum_acc<P>(dc));
            dc = P::zero();
            dc_active = false;
        }

        const unsigned char* vsl = vslot(t);
        Acc run = fmask ? P::zero() : dc;
        if (fmask != 0u && !first_head && lane == 0) run = P::carry_to_acc(carry);
        Acc head = P::zero();
        int cur_row = -1;  // row of this lane's open segment
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            XT xb[8];
            if (c + 1 < NC) {
                gather_chunk(t, c + 1, xb);
            } else if (t + 1 < t_end) {  // the next tile's first chunk
                if (ready(t + 1))
                    gather_chunk(t + 1, 0, xb);
                else
                    t_fail = t + 1;
            }
            VC v[8];
            swz_vals8(vsl, lane * VRUN + c * 8 * sizeof(VS), v, static_cast<const VS*>(nullptr));
            if (fmask == 0u) {
#pragma unroll
                for (int k = 0; k < 8; ++k) run = P::fma(v[k], xa[k], run);
            } else {
                const uint32_t cb = (w >> (32 - (c + 1) * 8)) & 0xFFu;
                chunk_segments<P, S, 8>(one_head, cb, c * 8, v, xa, run, head, cur_row, rowof,
                                        lane, a);
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) xa[k] = xb[k];
        }
        fence_proxy_async();  // this lane's reads of the slot come before the TMA that reuses it
        __syncwarp();

        tp0 = tp1;
        tp1 = tp2;
        rb = rbn;
        if (fmask == 0u) {
            dc = run;
            dc_active = true;
            continue;
        }
        const bool has = cur_row >= 0;
        if (!has) head = run;
        const Acc T = head_run_scan<P>(head, has, fmask, lane);
        Acc A = sh_down(T, 1);
        if (lane == 31) A = P::zero();
        const Acc T0 = sh_idx(T, 0);
        const int last = 31 - __clz(fmask);
        Acc fin = P::zero();
        if (has) {
            fin = P::add(run, A);
            if (lane != last) store_row(a.y, a.m, cur_row, P::out_acc(fin), a.err);
        }
        if (!first_head) flush(carry_row, P::carry_from(T0), carry_owned);
        carry_row = __shfl_sync(SPMV_FULL_MASK, cur_row, last);
        carry = P::carry_from(sh_idx(fin, last));
        carry_owned = true;
    }

    if (t_fail >= 0) {
        // the copies of tiles [t_fail, issued) may still be in flight; each must land (bounded
        // wait) before the warp's shared memory is released
        if (lane == 0) {
            atomicOr(a.err, ERR_WAIT_TIMEOUT);
            if (!rec_written) a.rec_row[worker] = -1;
        }
        for (int t = t_fail; t < issued; ++t) {
            if (!is_full(t)) continue;
            const int s = (t - t_begin) % NSTAGE;
            mbar_wait_bounded(&bars[s], (uint32_t)((t - t_begin) / NSTAGE) & 1u);
        }
        return;
    }
    if (carry_row >= 0) {
        Carry tot = carry;
        if (dc_active) tot = P::carry_add(tot, warp_sum_acc<P>(dc));
        flush(carry_row, tot, carry_owned);
    }
    if (!rec_written && lane == 0) a.rec_row[worker] = -1;
}

template <class P, int S, int WARPS, int NSTAGE, bool OH, bool XL2>
cudaError_t launch_tma_kernel(const TileArgs<P>& a, const StreamMaps& maps, int tpw, int nworkers,
                              int ntiles, int bytes, cudaStream_t st) {
    // the shared-memory opt-in is a per-device function attribute: set it once per device
    // (setting it twice from racing host threads is harmless; the flag word is atomic)
    static std::atomic<unsigned long long> attr_set{0ull};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_set.load(std::memory_order_acquire) & bit)) {
        e = cudaFuncSetAttribute(k_tiles_tma<P, S, WARPS, NSTAGE, OH, XL2>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit, std::memory_order_release);
    }
    const int blocks = (nworkers + WARPS - 1) / WARPS;
    k_tiles_tma<P, S, WARPS, NSTAGE, OH, XL2><<<blocks, WARPS * 32, bytes, st>>>(a, maps, tpw,
                                                                                nworkers, ntiles);
    return cudaSuccess;
}

template <class P, int S, int WARPS, int NSTAGE>
cudaError_t launch_tiles_tma_t(const TileArgs<P>& a, int tpw, int nworkers, int ntiles,
                               cudaStream_t st) {
    using L = TmaLayout<P, S, NSTAGE>;
    const int bytes = WARPS * L::WARP_BYTES + 1024;
    if (bytes > 227 * 1024) return cudaErrorInvalidValue;
    if (nworkers > 0 && (a.phase & 1)) {
        StreamMaps maps;
        const long long vbytes = (long long)a.nnz * (long long)sizeof(typename P::VS);
        if (a.nnz < 32 * S ||
            !encode_stream_map(a.val, vbytes, L::VROWS, &maps.val) ||
            !encode_stream_map(a.col, (long long)a.nnz * 4, L::CROWS, &maps.col)) {
            // no full tile, or a stream the tensor unit cannot address (not 16-byte aligned):
            // the direct-load kernel with the same tile size
            TileConfig c{S, tpw, WARPS, 0};
            return launch_tiles<P>(a, c, st);
        }
        cudaError_t e;
        if constexpr (sizeof(typename P::Acc) <= 8) {  // scalar accumulators: either form
            // chunk form and x gather path, both fixed by the plan
            if (a.one_head && a.x_l2)
                e = launch_tma_kernel<P, S, WARPS, NSTAGE, true, true>(a, maps, tpw, nworkers,
                                                                       ntiles, bytes, st);
            else if (a.one_head)
                e = launch_tma_kernel<P, S, WARPS, NSTAGE, true, false>(a, maps, tpw, nworkers,
                                                                        ntiles, bytes, st);
            else if (a.x_l2)
                e = launch_tma_kernel<P, S, WARPS, NSTAGE, false, true>(a, maps, tpw, nworkers,
                                                                        ntiles, bytes, st);
            else
                e = launch_tma_kernel<P, S, WARPS, NSTAGE, false, false>(a, maps, tpw, nworkers,
                                                                         ntiles, bytes, st);
        } else {
            e = launch_tma_kernel<P, S, WARPS, NSTAGE, false, false>(a, maps, tpw, nworkers,
                                                                     ntiles, bytes, st);
        }
        if (e != cudaSuccess) return e;
    }
    if (a.phase & 2) {
        const cudaError_t e = launch_calibrate(a, nworkers, st);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

template <class P>
int tma_smem_bytes(const TileConfig& c) {
    if (c.stages == 0) return 0;
    int per_warp = 0;
    switch (c.seg * 10 + c.stages) {
        case 82: per_warp = TmaLayout<P, 8, 2>::WARP_BYTES; break;
        case 83: per_warp = TmaLayout<P, 8, 3>::WARP_BYTES; break;
        case 84: per_warp = TmaLayout<P, 8, 4>::WARP_BYTES; break;
        case 162: per_warp = TmaLayout<P, 16, 2>::WARP_BYTES; break;
        case 163: per_warp = TmaLayout<P, 16, 3>::WARP_BYTES; break;
        case 164: per_warp = TmaLayout<P, 16, 4>::WARP_BYTES; break;
        case 322: per_warp = TmaLayout<P, 32, 2>::WARP_BYTES; break;
        case 323: per_warp = TmaLayout<P, 32, 3>::WARP_BYTES; break;
        case 324: per_warp = TmaLayout<P, 32, 4>::WARP_BYTES; break;
        default: return -1;
    }
    return per_warp * c.warps_per_cta + 1024;
}

// Direct-load kernel (stages == 0) or TMA-staged kernel (stages 2, 3 or 4).
template <class P>
cudaError_t launch_tiles_any(const TileArgs<P>& a, const TileConfig& cfg, cudaStream_t st) {
    if (cfg.stages == 0) return launch_tiles<P>(a, cfg, st);
    const int nt = num_tiles(a.nnz, 32 * cfg.seg);
    const int tpw = cfg.tiles_per_worker;
    const int nw = (nt + tpw - 1) / tpw;
    const bool w8 = cfg.warps_per_cta == 8;
#define SPMV_TMA_STAGES(SEG, W)                                                                    \
    switch (cfg.stages) {                                                                          \
        case 2: return launch_tiles_tma_t<P, SEG, W, 2>(a, tpw, nw, nt, st);                       \
        case 3: return launch_tiles_tma_t<P, SEG, W, 3>(a, tpw, nw, nt, st);                       \
        case 4: return launch_tiles_tma_t<P, SEG, W, 4>(a, tpw, nw, nt, st);                       \
        default: return cudaErrorInvalidValue;                                                     \
    }
#define SPMV_TMA_CASE(SEG)                                                                         \
    case SEG:                                                                                      \
        if (w8) {                                                                                  \
            SPMV_TMA_STAGES(SEG, 8)                                                                \
        }                                                                                          \
        SPMV_TMA_STAGES(SEG, 4)
    switch (cfg.seg) {
        SPMV_TMA_CASE(8)
        SPMV_TMA_CASE(16)
        SPMV_TMA_CASE(32)
        default:
            return cudaErrorInvalidValue;
    }
#undef SPMV_TMA_CASE
#undef SPMV_TMA_STAGES
}

}  // namespace spmv
