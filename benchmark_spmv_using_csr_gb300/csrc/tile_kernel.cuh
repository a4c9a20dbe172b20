// tile_kernel.cuh -- the speculative segmented-sum tile kernel, generic over the arithmetic.
//
// Restates spmv_cuda/kernels_cuda.h:7-269 + the host calibration of
// spmv_cuda/bhsparse_spmv_cuda.h:166-222 for sm_103a:
//
//  * the per-tile binary search moves to a one-off tile_ptr with dirty bits
//    (partition.cu), read here with two loads per tile;
//  * bit flags come from tile_flags() (tile.cuh), the same code the parity kernel runs;
//  * each lane streams its own S consecutive non-zeros with 256-bit loads (evict-first in
//    L2) and gathers x through the read-only path (evict-last in L2), then runs its
//    segmented sum with one accumulate step per non-zero.  On GB300 the FP64 pipe issues
//    about 2 lane-FMAs per clock per SM, so the FP64 form spends exactly one FMA per
//    non-zero and amortises every other FP64 add over 32*S non-zeros;
//  * head-less lane partials are combined across lanes with a segmented suffix sum (a
//    linear chain when the longest run of head-less lanes is short, a 5-step log scan
//    otherwise), replacing the serial shared-memory walk of kernels_cuda.h:218-230;
//  * rows are written at their true index: in a dirty tile the k-th row head maps to the
//    k-th non-empty row of the span (listed by tile_flags), so there is no compacted y and
//    no host fix-up;
//  * a tile without any row head keeps its partial per lane across tiles and folds it only
//    when the row ends (one butterfly per long row instead of one per tile);
//  * a worker (one warp) walks tiles_per_worker consecutive tiles with its carry in
//    registers.  The row it starts inside of (the reference's synchronizer entry,
//    kernels_cuda.h:243-247) is the only value it cannot write itself; it goes to a
//    per-worker carry record that k_calibrate adds in worker order after the main kernel
//    (replacing the host loop of bhsparse_spmv_cuda.h:170-173).  Every other row is
//    written exactly once, by the worker in which it starts, so y needs no zeroing and
//    repeated calls give the same y.
//
// The arithmetic policy P fixes the storage types and the accumulate / carry arithmetic:
// plain FP64 and FP32 (Acc = Carry = value type, one FMA per non-zero) and the mixed forms
// (FP32 or BF16 values, FP32 x and y, compensated float-float Acc, FP64 Carry).
#pragma once
#include "tile.cuh"

namespace spmv {

template <class P>
struct TileArgs {
    const int* __restrict__ row_ptr;
    const int* __restrict__ col;
    const typename P::VS* __restrict__ val;
    const typename P::XT* __restrict__ x;
    typename P::YT* __restrict__ y;
    const uint32_t* __restrict__ tile_ptr;
    int* __restrict__ rec_row;
    typename P::Carry* __restrict__ rec_val;
    uint32_t* err;
    int m, n, nnz;
    int phase;  // bit 0: tile kernel, bit 1: calibration kernel
};

// ---- shuffles for the accumulator types ----
__device__ __forceinline__ double sh_down(double v, int d) { return __shfl_down_sync(SPMV_FULL_MASK, v, d); }
__device__ __forceinline__ float sh_down(float v, int d) { return __shfl_down_sync(SPMV_FULL_MASK, v, d); }
__device__ __forceinline__ float2 sh_down(float2 v, int d) {
    return make_float2(__shfl_down_sync(SPMV_FULL_MASK, v.x, d), __shfl_down_sync(SPMV_FULL_MASK, v.y, d));
}
__device__ __forceinline__ double sh_idx(double v, int s) { return __shfl_sync(SPMV_FULL_MASK, v, s); }
__device__ __forceinline__ float sh_idx(float v, int s) { return __shfl_sync(SPMV_FULL_MASK, v, s); }
__device__ __forceinline__ float2 sh_idx(float2 v, int s) {
    return make_float2(__shfl_sync(SPMV_FULL_MASK, v.x, s), __shfl_sync(SPMV_FULL_MASK, v.y, s));
}
__device__ __forceinline__ double sh_xor(double v, int d) { return __shfl_xor_sync(SPMV_FULL_MASK, v, d); }
__device__ __forceinline__ float sh_xor(float v, int d) { return __shfl_xor_sync(SPMV_FULL_MASK, v, d); }
__device__ __forceinline__ float2 sh_xor(float2 v, int d) {
    return make_float2(__shfl_xor_sync(SPMV_FULL_MASK, v.x, d), __shfl_xor_sync(SPMV_FULL_MASK, v.y, d));
}

// ---- streamed loads of 8 consecutive non-zeros of one lane ----
__device__ __forceinline__ void load8_full(const double* val, const int* col, int e, uint64_t pol,
                                           double (&v)[8], int (&c)[8]) {
    double a[4], b[4];
    uint32_t cc[8];
    ld_stream_f64x4(val + e, pol, a);
    ld_stream_f64x4(val + e + 4, pol, b);
    ld_stream_b32x8(col + e, pol, cc);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[i] = a[i];
        v[i + 4] = b[i];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) c[i] = (int)cc[i];
}
__device__ __forceinline__ void load8_full(const float* val, const int* col, int e, uint64_t pol,
                                           float (&v)[8], int (&c)[8]) {
    uint32_t vv[8], cc[8];
    ld_stream_b32x8(val + e, pol, vv);
    ld_stream_b32x8(col + e, pol, cc);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        v[i] = __uint_as_float(vv[i]);
        c[i] = (int)cc[i];
    }
}
__device__ __forceinline__ void load8_full(const __nv_bfloat16* val, const int* col, int e,
                                           uint64_t pol, float (&v)[8], int (&c)[8]) {
    uint32_t vv[4], cc[8];
    ld_stream_b32x4(val + e, pol, vv);
    ld_stream_b32x8(col + e, pol, cc);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[2 * i] = __uint_as_float(vv[i] << 16);          // low half = element 2i
        v[2 * i + 1] = __uint_as_float(vv[i] & 0xffff0000u);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) c[i] = (int)cc[i];
}
__device__ __forceinline__ double to_compute(double v) { return v; }
__device__ __forceinline__ float to_compute(float v) { return v; }
__device__ __forceinline__ float to_compute(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename VS, typename VC>
__device__ __forceinline__ void load8_tail(const VS* val, const int* col, int e, int nnz,
                                           VC (&v)[8], int (&c)[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        if (e + i < nnz) {
            v[i] = to_compute(val[e + i]);
            c[i] = col[e + i];
        } else {
            v[i] = VC(0);
            c[i] = -1;  // padding slot: contributes 0, x is not read
        }
    }
}

template <class P, int S>
__device__ __forceinline__ void load_chunk(const TileArgs<P>& a, int t, int c, int lane,
                                           uint64_t pol, typename P::VC (&v)[8], int (&cc)[8]) {
    constexpr int TILE = 32 * S;
    const int e = t * TILE + lane * S + c * 8;
    if ((long long)(t + 1) * TILE <= a.nnz)
        load8_full(a.val, a.col, e, pol, v, cc);
    else
        load8_tail(a.val, a.col, e, a.nnz, v, cc);
}

template <typename XT>
__device__ __forceinline__ void gather8(const XT* __restrict__ x, const int (&c)[8], uint64_t pol,
                                        XT (&xv)[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) xv[i] = c[i] >= 0 ? ld_x(x + c[i], pol) : XT(0);
}

// Row of the q-th non-empty row of the span (checked: a bad index is recorded in the error
// word and yields -1, whose store is then skipped).
__device__ __forceinline__ int span_row(bool dirty, const int* list, int lo, int q, int cap,
                                        uint32_t* err) {
    if (!dirty) return lo + q;
    if ((unsigned)q < (unsigned)cap) return list[q];
    atomicOr(err, ERR_LIST_OVERFLOW);
    return -1;
}
template <typename YT>
__device__ __forceinline__ void store_row(YT* y, int m, int row, YT v, uint32_t* err) {
    if ((unsigned)row < (unsigned)m)
        y[row] = v;
    else
        atomicOr(err, ERR_BAD_TILE);
}

template <class P>
__device__ __forceinline__ typename P::Acc warp_sum_acc(typename P::Acc v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = P::add(v, sh_xor(v, d));
    return v;
}

template <class P, int S, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
    k_tiles(TileArgs<P> a, int tpw, int nworkers, int ntiles) {
    using Acc = typename P::Acc;
    using Carry = typename P::Carry;
    using VC = typename P::VC;
    using XT = typename P::XT;
    using YT = typename P::YT;
    constexpr int TILE = 32 * S;
    constexpr int NC = S / 8;
    constexpr int LIST = TILE + 1;  // non-empty rows of one tile span: at most TILE + 1
    __shared__ uint32_t s_words[WARPS][32];
    __shared__ int s_list[WARPS][LIST];

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int worker = blockIdx.x * WARPS + warp;
    if (worker >= nworkers) return;
    const int t_begin = worker * tpw;
    const int t_end = min(t_begin + tpw, ntiles);
    const uint64_t pol_s = policy_evict_first();
    const uint64_t pol_x = policy_evict_last();
    int* const list = s_list[warp];

    int carry_row = -1;  // row of the segment left open by the previous tile (-1: none)
    bool carry_owned = false;
    Carry carry = P::carry_zero();
    Acc dc = P::zero();  // per-lane partials of carry_row from tiles without a row head
    bool dc_active = false;
    bool rec_written = false;

    auto flush = [&](int row, Carry v, bool owned) {
        if (lane == 0) {
            if (owned) {
                store_row(a.y, a.m, row, P::out_carry(v), a.err);
            } else {
                a.rec_row[worker] = row;
                a.rec_val[worker] = v;
            }
        }
        if (!owned) rec_written = true;
    };

    VC cv[8], nv[8];
    XT xv[8];
    int cc[8], nc[8];
    load_chunk<P, S>(a, t_begin, 0, lane, pol_s, cv, cc);

    for (int t = t_begin; t < t_end; ++t) {
        const uint32_t tp0 = __ldg(a.tile_ptr + t);
        const uint32_t tp1 = __ldg(a.tile_ptr + t + 1);
        const int lo = (int)(tp0 & ROW_MASK);
        const int hi = (int)(tp1 & ROW_MASK);
        const bool dirty = (tp0 & DIRTY_BIT) != 0u;
        const int e0 = t * TILE;
        const uint32_t w = tile_flags<S, YT>(a.row_ptr, a.m, e0, lo, hi, dirty, s_words[warp],
                                             list, LIST, a.y, a.err);
        const bool first_head = ((shfl_idx(w, 0) >> 31) & 1u) != 0u;
        const int nf = __popc(w);
        const uint32_t fmask = __ballot_sync(SPMV_FULL_MASK, nf > 0);

        if (first_head) {
            // the open row ended exactly at this tile's start
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
            // first tile of this worker starts inside row lo, which began in an earlier worker
            carry_row = lo;
            carry_owned = false;
            carry = P::carry_zero();
        }

        if (fmask == 0u) {
            // no row head anywhere in the tile: every slot continues carry_row
            Acc r = dc;
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                if (c + 1 < NC)
                    load_chunk<P, S>(a, t, c + 1, lane, pol_s, nv, nc);
                else if (t + 1 < t_end)
                    load_chunk<P, S>(a, t + 1, 0, lane, pol_s, nv, nc);
                gather8(a.x, cc, pol_x, xv);
#pragma unroll
                for (int k = 0; k < 8; ++k) r = P::fma(cv[k], xv[k], r);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    cv[k] = nv[k];
                    cc[k] = nc[k];
                }
            }
            dc = r;
            dc_active = true;
            continue;
        }
        if (dc_active) {
            carry = P::carry_add(carry, warp_sum_acc<P>(dc));
            dc = P::zero();
            dc_active = false;
        }

        // ordinal (among the span's non-empty rows) of this lane's first row head
        const int qbase = warp_exclusive_scan(nf) + (first_head ? 0 : 1);
        Acc run = P::zero(), head = P::zero();
        int fidx = 0;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            if (c + 1 < NC)
                load_chunk<P, S>(a, t, c + 1, lane, pol_s, nv, nc);
            else if (t + 1 < t_end)
                load_chunk<P, S>(a, t + 1, 0, lane, pol_s, nv, nc);
            gather8(a.x, cc, pol_x, xv);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const bool f = ((w >> (31 - (c * 8 + k))) & 1u) != 0u;
                if (f) {
                    if (fidx > 0) {  // a row that starts and ends inside this lane
                        const int row = span_row(dirty, list, lo, qbase + fidx - 1, LIST, a.err);
                        store_row(a.y, a.m, row, P::out_acc(run), a.err);
                    } else {
                        head = run;  // slots before the lane's first row head
                    }
                    ++fidx;
                    run = P::zero();
                }
                run = P::fma(cv[k], xv[k], run);
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                cv[k] = nv[k];
                cc[k] = nc[k];
            }
        }

        const bool has = fidx > 0;
        if (!has) head = run;
        // T_l = head_l + (has_l ? 0 : T_{l+1}): the head-less run that starts at lane l
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
        int frow = 0;
        if (has) {
            fin = P::add(run, A);
            frow = span_row(dirty, list, lo, qbase + fidx - 1, LIST, a.err);
            if (lane != last) store_row(a.y, a.m, frow, P::out_acc(fin), a.err);
        }
        if (!first_head) flush(carry_row, P::carry_add(carry, T0), carry_owned);  // open row ends here
        carry_row = __shfl_sync(SPMV_FULL_MASK, frow, last);
        if (carry_row < 0) carry_row = -1;  // a failed lookup was recorded; nothing to carry
        carry = P::carry_from(sh_idx(fin, last));
        carry_owned = true;
    }

    if (carry_row >= 0) {
        Carry tot = carry;
        if (dc_active) tot = P::carry_add(tot, warp_sum_acc<P>(dc));
        flush(carry_row, tot, carry_owned);
    }
    if (!rec_written && lane == 0) a.rec_row[worker] = -1;
}

// Carry records -> y, in worker order (deterministic): the first record of each run of equal
// rows sums the run and adds it to the owner's value.  Also zeroes the leading empty rows,
// which lie in no tile span (the reference never writes them).
template <class P>
__global__ void k_calibrate(const int* __restrict__ rec_row,
                            const typename P::Carry* __restrict__ rec_val, int nworkers,
                            typename P::YT* __restrict__ y, const uint32_t* __restrict__ tile_ptr,
                            int m, uint32_t* err) {
    using Carry = typename P::Carry;
    const int stride = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int w = tid; w < nworkers; w += stride) {
        const int r = rec_row[w];
        if (r < 0) continue;
        if (w > 0 && rec_row[w - 1] == r) continue;
        Carry s = rec_val[w];
        for (int v = w + 1; v < nworkers && rec_row[v] == r; ++v) s = s + rec_val[v];
        if (r >= m) {
            atomicOr(err, ERR_BAD_TILE);
            continue;
        }
        y[r] = P::out_carry(P::carry_of_y(y[r]) + s);
    }
    const int lead = min((int)(tile_ptr[0] & ROW_MASK), m);
    for (int r = tid; r < lead; r += stride) y[r] = typename P::YT(0);
}

template <class P, int S, int WARPS>
cudaError_t launch_tiles_t(const TileArgs<P>& a, int tpw, int nworkers, int ntiles,
                           cudaStream_t st) {
    if (nworkers > 0 && (a.phase & 1)) {
        const int blocks = (nworkers + WARPS - 1) / WARPS;
        k_tiles<P, S, WARPS><<<blocks, WARPS * 32, 0, st>>>(a, tpw, nworkers, ntiles);
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
cudaError_t launch_tiles(const TileArgs<P>& a, const TileConfig& cfg, cudaStream_t st) {
    const int nt = num_tiles(a.nnz, 32 * cfg.seg);
    const int tpw = cfg.tiles_per_worker;
    const int nw = (nt + tpw - 1) / tpw;
    const bool w8 = cfg.warps_per_cta == 8;
    switch (cfg.seg) {
        case 8:
            return w8 ? launch_tiles_t<P, 8, 8>(a, tpw, nw, nt, st) : launch_tiles_t<P, 8, 4>(a, tpw, nw, nt, st);
        case 16:
            return w8 ? launch_tiles_t<P, 16, 8>(a, tpw, nw, nt, st) : launch_tiles_t<P, 16, 4>(a, tpw, nw, nt, st);
        case 32:
            return w8 ? launch_tiles_t<P, 32, 8>(a, tpw, nw, nt, st) : launch_tiles_t<P, 32, 4>(a, tpw, nw, nt, st);
        default:
            return cudaErrorInvalidValue;
    }
}

}  // namespace spmv
