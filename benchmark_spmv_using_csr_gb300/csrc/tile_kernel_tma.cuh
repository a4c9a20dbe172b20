// tile_kernel_tma.cuh -- the tile kernel with its val / col_idx stream staged in shared
// memory by bulk (TMA) copies.
//
// Same algorithm and output as k_tiles (tile_kernel.cuh); what changes is how a tile reaches
// the lanes:
//  * every lane issues two cp.async.bulk copies per tile (its S values and its S column
//    indices) into its own padded run of a per-warp ring of NSTAGE tile slots, completing
//    on the slot's mbarrier.  The stream therefore runs NSTAGE-1 tiles ahead without holding
//    any registers, and the padding (16 bytes per run) makes the 16-byte shared-memory reads
//    of the lane-contiguous runs bank-conflict free;
//  * x is gathered one chunk of 8 non-zeros ahead of the fused multiply-adds;
//  * the row of a row head is read from a slot->row map built while the bit flags are
//    generated (tile_rows below), so dirty tiles (empty rows) need no compaction step;
//  * tile_ptr and the first 32 row_ptr entries of the next tile's span are prefetched one
//    tile ahead.
// Every mbarrier wait is bounded; a timeout sets ERR_WAIT_TIMEOUT, the warp drains the copies
// it still has in flight (again bounded) and stops.
#pragma once
#include "tile_kernel.cuh"

namespace spmv {

template <typename VS>
__device__ __forceinline__ VS zero_value() { return VS(0.0f); }
template <>
__device__ __forceinline__ __nv_bfloat16 zero_value<__nv_bfloat16>() { return __float2bfloat16(0.0f); }

template <class P, int S, int NSTAGE>
struct TmaLayout {
    using VS = typename P::VS;
    static constexpr int TILE = 32 * S;
    static constexpr int VSTR = S * (int)sizeof(VS) + 16;  // bytes per lane run of values
    static constexpr int CSTR = S * 4 + 16;                // bytes per lane run of columns
    static constexpr int SLOT = 32 * VSTR + 32 * CSTR;
    static constexpr int ROWOF = TILE * 4;
    static constexpr int RAW = NSTAGE * SLOT + ROWOF + 128 + NSTAGE * 8;
    static constexpr int WARP_BYTES = (RAW + 127) / 128 * 128;
    static_assert(VSTR % 16 == 0 && CSTR % 16 == 0 && SLOT % 16 == 0, "TMA alignment");
    static_assert(S * (int)sizeof(VS) % 16 == 0 && S * 4 % 16 == 0, "bulk copy size");
};

// 8 values / 8 columns of chunk c from this lane's runs in shared memory (16-byte reads)
__device__ __forceinline__ void smem_vals8(const unsigned char* run, int c, double (&v)[8]) {
    const double2* p = reinterpret_cast<const double2*>(run + c * 64);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const double2 d = p[i];
        v[2 * i] = d.x;
        v[2 * i + 1] = d.y;
    }
}
__device__ __forceinline__ void smem_vals8(const unsigned char* run, int c, float (&v)[8],
                                           const float*) {
    const float4* p = reinterpret_cast<const float4*>(run + c * 32);
    const float4 a = p[0], b = p[1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void smem_vals8(const unsigned char* run, int c, float (&v)[8],
                                           const __nv_bfloat16*) {
    const uint4 q = *reinterpret_cast<const uint4*>(run + c * 16);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[2 * i] = __uint_as_float(w[i] << 16);
        v[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
    }
}
template <typename VS>
__device__ __forceinline__ void smem_vals(const unsigned char* run, int c, double (&v)[8]) {
    smem_vals8(run, c, v);
}
template <typename VS>
__device__ __forceinline__ void smem_vals(const unsigned char* run, int c, float (&v)[8]) {
    smem_vals8(run, c, v, static_cast<const VS*>(nullptr));
}
__device__ __forceinline__ void smem_cols8(const unsigned char* run, int c, int (&cc)[8]) {
    const int4* p = reinterpret_cast<const int4*>(run + c * 32);
    const int4 a = p[0], b = p[1];
    cc[0] = a.x; cc[1] = a.y; cc[2] = a.z; cc[3] = a.w;
    cc[4] = b.x; cc[5] = b.y; cc[6] = b.z; cc[7] = b.w;
}

template <typename XT>
__device__ __forceinline__ void gather8(const XT* __restrict__ x, const int (&c)[8], uint64_t pol,
                                        XT (&xv)[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) xv[i] = c[i] >= 0 ? ld_x(x + c[i], pol) : XT(0);
}

template <class P, int S, int WARPS, int NSTAGE>
__global__ void __launch_bounds__(WARPS * 32, 1)
    k_tiles_tma(TileArgs<P> a, int tpw, int nworkers, int ntiles) {
    using L = TmaLayout<P, S, NSTAGE>;
    using VS = typename P::VS;
    using Acc = typename P::Acc;
    using Carry = typename P::Carry;
    using VC = typename P::VC;
    using XT = typename P::XT;
    using YT = typename P::YT;
    constexpr int TILE = 32 * S;
    constexpr int NC = S / 8;
    extern __shared__ __align__(128) unsigned char smem[];

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int worker = blockIdx.x * WARPS + warp;
    if (worker >= nworkers) return;
    unsigned char* const wb = smem + warp * L::WARP_BYTES;
    int* const rowof = reinterpret_cast<int*>(wb + NSTAGE * L::SLOT);
    uint32_t* const words = reinterpret_cast<uint32_t*>(wb + NSTAGE * L::SLOT + L::ROWOF);
    uint64_t* const bars = reinterpret_cast<uint64_t*>(wb + NSTAGE * L::SLOT + L::ROWOF + 128);
    if (lane == 0) {
#pragma unroll
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 32);
        fence_barrier_init();
    }
    __syncwarp();

    const int t_begin = worker * tpw;
    const int t_end = min(t_begin + tpw, ntiles);
    const uint64_t pol_s = policy_evict_first();
    const uint64_t pol_x = policy_evict_last();
    auto is_full = [&](int t) { return (long long)(t + 1) * TILE <= a.nnz; };

    // bulk copies of tile t's runs into its slot (full tiles only)
    int issued = t_begin;  // tiles [t_begin, issued) have been issued (or staged later)
    auto issue_next = [&]() {
        const int t = issued;
        if (t >= t_end) return;
        ++issued;
        if (!is_full(t)) return;
        const int s = (t - t_begin) % NSTAGE;
        unsigned char* sl = wb + s * L::SLOT;
        const int e = t * TILE + lane * S;
        mbar_arrive_expect_tx(&bars[s], (uint32_t)(S * sizeof(VS) + S * 4));
        bulk_g2s(sl + lane * L::VSTR, a.val + e, (uint32_t)(S * sizeof(VS)), &bars[s], pol_s);
        bulk_g2s(sl + 32 * L::VSTR + lane * L::CSTR, a.col + e, (uint32_t)(S * 4), &bars[s], pol_s);
    };
#pragma unroll
    for (int i = 0; i < NSTAGE - 1; ++i) issue_next();
    uint32_t parity = 0u;
    int t_fail = -1;  // tile whose wait timed out

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

    for (int t = t_begin; t < t_end; ++t) {
        issue_next();  // tile t+NSTAGE-1 into the slot that tile t-1 has released
        const int lo = (int)(tp0 & ROW_MASK);
        const int hi = (int)(tp1 & ROW_MASK);
        uint32_t tp2 = 0u;
        RowBatch rbn{0, 0, 0, 0};
        if (t + 1 < t_end) {  // meta of the next tile
            tp2 = __ldg(a.tile_ptr + t + 2);
            rbn = prefetch_rows(a.row_ptr, a.m, hi);
        }
        const int e0 = t * TILE;
        const uint32_t w = tile_rows<S, YT>(a.row_ptr, a.m, e0, lo, hi, rb, words, rowof, a.y);
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

        // the tile's data in its slot
        const int s = (t - t_begin) % NSTAGE;
        unsigned char* sl = wb + s * L::SLOT;
        unsigned char* vrun = sl + lane * L::VSTR;
        unsigned char* crun = sl + 32 * L::VSTR + lane * L::CSTR;
        if (is_full(t)) {
            if (!mbar_wait_bounded(&bars[s], (parity >> s) & 1u)) {
                t_fail = t;
                if (lane == 0) atomicOr(a.err, ERR_WAIT_TIMEOUT);
                break;
            }
            parity ^= 1u << s;
        } else {
            // the matrix's last, partial tile: staged with guarded loads, zero padded
#pragma unroll 4
            for (int k = 0; k < S; ++k) {
                const int e = e0 + lane * S + k;
                const bool in = e < a.nnz;
                reinterpret_cast<VS*>(vrun)[k] = in ? a.val[e] : zero_value<VS>();
                reinterpret_cast<int*>(crun)[k] = in ? a.col[e] : -1;
            }
            __syncwarp();
        }

        Acc run = fmask ? P::zero() : dc;
        if (fmask != 0u && !first_head && lane == 0) run = P::carry_to_acc(carry);
        Acc head = P::zero();
        int cur_row = -1;  // row of this lane's open segment
        {
            int cc[8];
            XT xa[8];
            smem_cols8(crun, 0, cc);
            gather8(a.x, cc, pol_x, xa);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                XT xb[8];
                if (c + 1 < NC) {
                    smem_cols8(crun, c + 1, cc);
                    gather8(a.x, cc, pol_x, xb);
                }
                VC v[8];
                smem_vals<VS>(vrun, c, v);
                if (fmask == 0u) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) run = P::fma(v[k], xa[k], run);
                } else {
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const int kk = c * 8 + k;
                        if ((w >> (31 - kk)) & 1u) {
                            if (cur_row >= 0)
                                store_row(a.y, a.m, cur_row, P::out_acc(run), a.err);
                            else
                                head = run;
                            cur_row = rowof[lane * S + kk];
                            run = P::zero();
                        }
                        run = P::fma(v[k], xa[k], run);
                    }
                }
                if (c + 1 < NC) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) xa[k] = xb[k];
                }
            }
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
        Acc T = head;
        const int D = longest_zero_run(fmask);
        if (D <= 5) {
            bool stop = has;
            for (int d = 1; d <= D; ++d) {
                const Acc hv = sh_down(head, d);
                if (!stop && lane + d < 32) {
                    T = P::add(T, hv);
                    stop = ((fmask >> (lane + d)) & 1u) != 0u;
                }
            }
        } else {
            int stop = has ? 1 : 0;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const Acc tv = sh_down(T, d);
                const int sv = __shfl_down_sync(SPMV_FULL_MASK, stop, d);
                if (!stop && lane + d < 32) {
                    T = P::add(T, tv);
                    stop = sv;
                }
            }
        }
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
        // drain: the copies of tiles [t_fail, issued) are still in flight; each must land
        // (bounded wait) before the warp's shared memory is released
        for (int t = t_fail; t < issued; ++t) {
            if (!is_full(t)) continue;
            const int s = (t - t_begin) % NSTAGE;
            mbar_wait_bounded(&bars[s], (parity >> s) & 1u);
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

template <class P, int S, int WARPS, int NSTAGE>
cudaError_t launch_tiles_tma_t(const TileArgs<P>& a, int tpw, int nworkers, int ntiles,
                               cudaStream_t st) {
    using L = TmaLayout<P, S, NSTAGE>;
    const int bytes = WARPS * L::WARP_BYTES;
    if (bytes > 227 * 1024) return cudaErrorInvalidValue;
    if (nworkers > 0 && (a.phase & 1)) {
        // the shared-memory opt-in is a per-device function attribute: set it once per device
        static unsigned long long attr_set = 0ull;
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(attr_set & bit)) {
            e = cudaFuncSetAttribute(k_tiles_tma<P, S, WARPS, NSTAGE>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (e != cudaSuccess) return e;
            attr_set |= bit;
        }
        const int blocks = (nworkers + WARPS - 1) / WARPS;
        k_tiles_tma<P, S, WARPS, NSTAGE><<<blocks, WARPS * 32, bytes, st>>>(a, tpw, nworkers, ntiles);
    }
    if (a.phase & 2) {
        int cb = (nworkers + 255) / 256;
        if (cb < 1) cb = 1;
        if (cb > 152 * 8) cb = 152 * 8;
        k_calibrate<P><<<cb, 256, 0, st>>>(a.rec_row, a.rec_val, nworkers, a.y, a.tile_ptr, a.m,
                                           a.err);
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
        case 162: per_warp = TmaLayout<P, 16, 2>::WARP_BYTES; break;
        case 163: per_warp = TmaLayout<P, 16, 3>::WARP_BYTES; break;
        case 322: per_warp = TmaLayout<P, 32, 2>::WARP_BYTES; break;
        case 323: per_warp = TmaLayout<P, 32, 3>::WARP_BYTES; break;
        default: return -1;
    }
    return per_warp * c.warps_per_cta;
}

// Direct-load kernel (stages == 0) or TMA-staged kernel (stages 2 or 3).
template <class P>
cudaError_t launch_tiles_any(const TileArgs<P>& a, const TileConfig& cfg, cudaStream_t st) {
    if (cfg.stages == 0) return launch_tiles<P>(a, cfg, st);
    const int nt = num_tiles(a.nnz, 32 * cfg.seg);
    const int tpw = cfg.tiles_per_worker;
    const int nw = (nt + tpw - 1) / tpw;
    const bool w8 = cfg.warps_per_cta == 8;
    const bool s3 = cfg.stages == 3;
#define SPMV_TMA_CASE(SEG)                                                                         \
    case SEG:                                                                                      \
        if (w8) return s3 ? launch_tiles_tma_t<P, SEG, 8, 3>(a, tpw, nw, nt, st)                   \
                          : launch_tiles_tma_t<P, SEG, 8, 2>(a, tpw, nw, nt, st);                  \
        return s3 ? launch_tiles_tma_t<P, SEG, 4, 3>(a, tpw, nw, nt, st)                           \
                  : launch_tiles_tma_t<P, SEG, 4, 2>(a, tpw, nw, nt, st);
    switch (cfg.seg) {
        SPMV_TMA_CASE(8)
        SPMV_TMA_CASE(16)
        SPMV_TMA_CASE(32)
        default:
            return cudaErrorInvalidValue;
    }
#undef SPMV_TMA_CASE
}

}  // namespace spmv
