// tile_kernel.cuh -- the speculative segmented-sum tile kernel, generic over the arithmetic.
//
// Restates spmv_cuda/kernels_cuda.h:7-269 + the host calibration of
// spmv_cuda/bhsparse_spmv_cuda.h:166-222 for sm_103a:
//
//  * the per-tile binary search moves to a one-off tile_ptr with dirty bits
//    (partition.cu), read here with two loads per tile;
//  * bit flags and the slot -> row map come from tile_rows() (tile.cuh), the same code the
//    parity kernel runs; the plain FP64 kernels build them one tile ahead, overlapped with
//    the current tile's work;
//  * each lane streams its own S consecutive non-zeros with 256-bit loads and gathers x
//    through the read-only path, then runs its segmented sum with one accumulate step per
//    non-zero: a branch per slot, or, when no lane has two row heads in a chunk (long rows),
//    selects and one store per chunk.  On GB300 the FP64 pipe issues about 2 lane-FMAs per
//    clock per SM, so the FP64 form spends exactly one FMA per non-zero and amortises every
//    other FP64 add over 32*S non-zeros;
//  * head-less lane partials are combined across lanes with a segmented suffix sum (a
//    linear chain when the longest run of head-less lanes is short, a 5-step log scan
//    otherwise), replacing the serial shared-memory walk of kernels_cuda.h:218-230;
//  * rows are written at their true index: in a dirty tile the k-th row head maps to the
//    k-th non-empty row of the span (listed by tile_rows), so there is no compacted y and
//    no host fix-up;
//  * a tile without any row head keeps its partial per lane across tiles and folds it only
//    when the row ends (one butterfly per long row instead of one per tile);
//  * a worker is tiles_per_worker consecutive tiles, walked by one warp with its carry in
//    registers; a matrix larger than one wave of workers runs a persistent kernel whose warps
//    take workers from a global ticket, a smaller one a warp per worker.  The row it starts inside of (the reference's synchronizer entry,
//    kernels_cuda.h:243-247) is the only value it cannot write itself; it goes to a
//    per-worker carry record that k_calibrate adds in worker order after the main kernel
//    (replacing the host loop of bhsparse_spmv_cuda.h:170-173).  Every other row is
//    written exactly once, by the worker in which it starts, so y needs no zeroing and
//    repeated calls give the same y.
//
// The arithmetic policy P fixes the storage types and the accumulate / carry arithmetic:
// plain FP64 and FP32 (accumulator, carry and record all in the value type, one FMA per
// non-zero) and the mixed forms (FP32 or BF16 values, FP32 x and y, compensated float-float
// accumulator and within-worker carry, FP64 carry records and calibration).
//
// Policy interface: Acc (per-lane accumulator): zero, fma, add; Carry (a worker's open row):
// carry_zero, carry_add(Carry, Acc), carry_from(Acc), carry_to_acc, out_carry -> YT; Rec (a carry record
// between workers): rec_from(Carry), rec_add, rec_of_y(YT), out_rec -> YT; out_acc(Acc) -> YT.
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
    typename P::Rec* __restrict__ rec_val;
    uint32_t* err;
    int m, n, nnz;
    int phase;  // bit 0: tile kernel, bit 1: calibration kernel
    // launcher choice, made at plan time: the kernel specialised for the one-head chunk form
    // (few rows shorter than a chunk, so that most chunks take it)
    bool one_head = false;
    // launcher choice, made at plan time: x gathers from L2 only (columns without locality)
    bool x_l2 = false;
    // the persistent kernel's work queue: [0] the next worker, [1] warps done; zero before a
    // launch, and zero again after it (the last warp to finish resets both)
    int* ticket = nullptr;
    // the tile kernel's grid: -1 by the rule below (launch_tile_kernel), 0 static (a warp per
    // worker), 1 persistent where the variant has a persistent kernel
    int grid_mode = -1;
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

__device__ __forceinline__ double to_compute(double v) { return v; }
__device__ __forceinline__ float to_compute(float v) { return v; }
__device__ __forceinline__ float to_compute(__nv_bfloat16 v) { return __bfloat162float(v); }

// Non-zeros per lane handled per pipeline step (a "chunk"): 4 for S = 8 (two steps per tile,
// fewer live registers), 8 otherwise.
template <int S, typename XT>
__host__ __device__ constexpr int chunk_width() {
    // x entries wider than 8 bytes (several right-hand sides) use 4-wide chunks, and 8 right-
    // hand sides (32-byte entries) 2-wide ones: 160 instead of 190 registers, 12 instead of 8
    // resident warps per SM, +19 % on the batched workload at k = 8
    return sizeof(XT) > 16 ? 2 : (S == 8 || sizeof(XT) > 8) ? 4 : 8;
}

// one x entry: through L1 (read-only path), or from L2 only (XL2)
template <bool XL2, typename XT>
__device__ __forceinline__ XT ld_x_sel(const XT* p, uint64_t pol) {
    if constexpr (XL2)
        return ld_x_l2(p);
    else
        return ld_x(p, pol);
}
template <bool XL2, int CW, typename XT>
__device__ __forceinline__ void gather_cw(const XT* __restrict__ x, const int (&c)[CW], uint64_t pol,
                                          XT (&xv)[CW]) {
#pragma unroll
    for (int i = 0; i < CW; ++i) xv[i] = c[i] >= 0 ? ld_x_sel<XL2>(x + c[i], pol) : XT(0);
}
// x entries of a chunk of a full tile, which has no padding slot (column -1) to test
template <bool XL2, int CW, typename XT>
__device__ __forceinline__ void gather_cw_full(const XT* __restrict__ x, const int (&c)[CW],
                                               uint64_t pol, XT (&xv)[CW]) {
#pragma unroll
    for (int i = 0; i < CW; ++i) xv[i] = ld_x_sel<XL2>(x + c[i], pol);
}

template <typename YT>
__device__ __forceinline__ void store_row(YT* y, int m, int row, YT v, uint32_t* err) {
    if ((unsigned)row < (unsigned)m)
        y[row] = v;
    else
        atomicOr(err, ERR_BAD_TILE);
}

// Loops over the lanes of a warp that run once per tile or less: fully unrolled for scalar
// accumulators, kept rolled for the batched form's wide ones (2 or more right-hand sides), whose
// unrolled copies would crowd the multiply-add loop out of the instruction cache.
template <class P>
constexpr int cold_unroll() {
    return sizeof(typename P::Acc) >= 16 ? 1 : 5;
}

template <class P>
__device__ __forceinline__ typename P::Acc warp_sum_acc(typename P::Acc v) {
    constexpr int U = cold_unroll<P>();
#pragma unroll U
    for (int d = 16; d > 0; d >>= 1) v = P::add(v, sh_xor(v, d));
    return v;
}

// Column indices / values of chunk c (CW non-zeros) of tile t for this lane: one vector load
// each on full tiles, guarded scalar loads on the matrix's last, partial tile (column -1 and
// value 0 mark padding slots, which contribute nothing and read no x).
template <class P, int S, int CW>
__device__ __forceinline__ void load_cols(const TileArgs<P>& a, int t, int c, int lane,
                                          uint64_t pol, int (&cc)[CW]) {
    constexpr int TILE = 32 * S;
    const int e = t * TILE + lane * S + c * CW;
    if ((long long)(t + 1) * TILE <= a.nnz) {
        uint32_t u[CW];
        ld_stream_u32s(a.col + e, pol, u);
#pragma unroll
        for (int i = 0; i < CW; ++i) cc[i] = (int)u[i];
    } else {
#pragma unroll
        for (int i = 0; i < CW; ++i) cc[i] = e + i < a.nnz ? a.col[e + i] : -1;
    }
}
// S = 8: a lane's 8 column indices of tile t (one 32-byte sector) in one load, split into the
// tile's two 4-slot chunks.  Two 16-byte loads a chunk apart read the sector twice when the x
// gathers in between evict it from L1.
template <class P>
__device__ __forceinline__ void load_cols_tile8(const TileArgs<P>& a, int t, int lane, uint64_t pol,
                                                int (&c0)[4], int (&c1)[4]) {
    const int e = t * 256 + lane * 8;
    if ((long long)(t + 1) * 256 <= a.nnz) {
        uint32_t u[8];
        ld_stream_b32x8(a.col + e, pol, u);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            c0[i] = (int)u[i];
            c1[i] = (int)u[4 + i];
        }
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            c0[i] = e + i < a.nnz ? a.col[e + i] : -1;
            c1[i] = e + 4 + i < a.nnz ? a.col[e + 4 + i] : -1;
        }
    }
}
template <int CW>
__device__ __forceinline__ void load_vals_full(const double* val, int e, uint64_t pol,
                                               double (&v)[CW]) {
#pragma unroll
    for (int h = 0; h < CW / 4; ++h) {
        double p[4];
        ld_stream_f64x4(val + e + 4 * h, pol, p);
#pragma unroll
        for (int i = 0; i < 4; ++i) v[4 * h + i] = p[i];
    }
}
template <int CW>
__device__ __forceinline__ void load_vals_full(const float* val, int e, uint64_t pol,
                                               float (&v)[CW]) {
    uint32_t u[CW];
    ld_stream_u32s(val + e, pol, u);
#pragma unroll
    for (int i = 0; i < CW; ++i) v[i] = __uint_as_float(u[i]);
}
// S = 8, 4-byte values: a lane's 8 values of tile t (one 32-byte sector) in one load, split into
// the tile's two 4-slot chunks
template <class P>
__device__ __forceinline__ void load_vals_tile8(const TileArgs<P>& a, int t, int lane, uint64_t pol,
                                                typename P::VC (&v0)[4], typename P::VC (&v1)[4]) {
    const int e = t * 256 + lane * 8;
    if ((long long)(t + 1) * 256 <= a.nnz) {
        uint32_t u[8];
        ld_stream_b32x8(a.val + e, pol, u);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            v0[i] = __uint_as_float(u[i]);
            v1[i] = __uint_as_float(u[4 + i]);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            v0[i] = e + i < a.nnz ? to_compute(a.val[e + i]) : typename P::VC(0);
            v1[i] = e + 4 + i < a.nnz ? to_compute(a.val[e + 4 + i]) : typename P::VC(0);
        }
    }
}
template <int CW>
__device__ __forceinline__ void load_vals_full(const __nv_bfloat16* val, int e, uint64_t pol,
                                               float (&v)[CW]) {
    uint32_t u[CW / 2];
    ld_stream_u32s(val + e, pol, u);
#pragma unroll
    for (int i = 0; i < CW / 2; ++i) {
        v[2 * i] = __uint_as_float(u[i] << 16);  // the low half holds element 2i
        v[2 * i + 1] = __uint_as_float(u[i] & 0xffff0000u);
    }
}
template <class P, int S, int CW>
__device__ __forceinline__ void load_vals(const TileArgs<P>& a, int t, int c, int lane,
                                          uint64_t pol, typename P::VC (&v)[CW]) {
    constexpr int TILE = 32 * S;
    const int e = t * TILE + lane * S + c * CW;
    if ((long long)(t + 1) * TILE <= a.nnz) {
        load_vals_full(a.val, e, pol, v);
    } else {
#pragma unroll
        for (int i = 0; i < CW; ++i)
            v[i] = e + i < a.nnz ? to_compute(a.val[e + i]) : typename P::VC(0);
    }
}

// T_l = head_l + (has_l ? 0 : T_{l+1}): the head-less run that starts at lane l (the slots
// before lane l's first row head plus, while lanes have no head, those of the lanes after it).
// fmask has bit l set when lane l has a row head.  A short chain of shuffles when the longest
// run of head-less lanes is at most 5, else a 5-step segmented scan.
template <class P>
__device__ __forceinline__ typename P::Acc head_run_scan(typename P::Acc head, bool has,
                                                         uint32_t fmask, int lane) {
    using Acc = typename P::Acc;
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
        constexpr int U = cold_unroll<P>();
#pragma unroll U
        for (int d = 1; d < 32; d <<= 1) {
            const Acc tv = sh_down(T, d);
            const int sv = __shfl_down_sync(SPMV_FULL_MASK, stop, d);
            if (!stop && lane + d < 32) {
                T = P::add(T, tv);
                stop = sv;
            }
        }
    }
    return T;
}

// The segmented multiply-accumulate of one chunk of CW slots of this lane.  cb = the lane's row-
// head bits for the chunk (its first slot, lane slot kk0, in bit CW-1).  At a head the running
// sum `run` closes a segment: stored to cur_row when the lane already had a head, else kept as
// `head` (the slots before the lane's first head); cur_row becomes the head's row.
//
// When no lane of the warp has two heads in the chunk (rows of CW non-zeros or more, which the
// plan's one-head word says is the common case) the slots run branch-free: the head closes the
// segment by selects and the closed segment is stored once per chunk.  The per-slot branch of
// the general form runs its body whenever any lane of the warp has a head in that slot, which
// on such matrices is most slots.
template <class P, int S, int CW, typename VC, typename XT>
__device__ __forceinline__ void chunk_segments(bool one_head, uint32_t cb, int kk0,
                                               const VC (&v)[CW], const XT (&x)[CW],
                                               typename P::Acc& run, typename P::Acc& head,
                                               int& cur_row, const int* rowof, int lane,
                                               const TileArgs<P>& a) {
    using Acc = typename P::Acc;
    if (one_head && __all_sync(SPMV_FULL_MASK, (cb & (cb - 1u)) == 0u)) {
        const int h = cb != 0u ? __clz(cb) - (32 - CW) : CW;  // head slot, CW: none
        Acc done = run;
#pragma unroll
        for (int k = 0; k < CW; ++k) {
            const bool at = k == h;
            done = at ? run : done;
            run = at ? P::zero() : run;
            run = P::fma(v[k], x[k], run);
        }
        if (cb != 0u) {
            if (cur_row >= 0)
                store_row(a.y, a.m, cur_row, P::out_acc(done), a.err);
            else
                head = done;
            cur_row = rowof[lane * S + kk0 + h];
        }
    } else {
#pragma unroll
        for (int k = 0; k < CW; ++k) {
            if ((cb >> (CW - 1 - k)) & 1u) {
                if (cur_row >= 0)
                    store_row(a.y, a.m, cur_row, P::out_acc(run), a.err);  // complete in lane
                else
                    head = run;  // slots before the lane's first row head
                cur_row = rowof[lane * S + kk0 + k];
                run = P::zero();
            }
            run = P::fma(v[k], x[k], run);
        }
    }
}

// The tile kernel.  One warp = one worker over tiles [t_begin, t_end).  The stream runs as a
// software pipeline over the worker's chunks of CW non-zeros per lane: while chunk g is
// multiplied, the values of chunk g+1 and the column indices of chunk g+2 are in flight and the
// x gathers of chunk g+1 are issued; the bit flags' row_ptr entries and tile_ptr are fetched
// one tile ahead.
template <class P, int S, bool OH = false, bool MID = false, bool XL2 = false>
__device__ __forceinline__ void tile_worker(const TileArgs<P>& a, int worker, int tpw, int ntiles,
                                            uint32_t* const s_words_w, int* const rowof) {
    using Acc = typename P::Acc;
    using Carry = typename P::Carry;
    using VC = typename P::VC;
    using XT = typename P::XT;
    using YT = typename P::YT;
    constexpr int TILE = 32 * S;
    constexpr int CW = chunk_width<S, typename P::XT>();
    constexpr int NC = S / CW;
    // the one-head chunk form (scalar accumulators only; wide ones keep the per-slot loop)
    constexpr bool one_head = OH && sizeof(Acc) <= 8;
    const int lane = threadIdx.x & 31;
    const int t_begin = worker * tpw;
    const int t_end = min(t_begin + tpw, ntiles);
    const uint64_t pol_s = policy_evict_first();
    const uint64_t pol_x = policy_evict_last();

    uint32_t tp0 = __ldg(a.tile_ptr + t_begin);
    uint32_t tp1 = __ldg(a.tile_ptr + t_begin + 1);
    RowBatch rb = prefetch_rows(a.row_ptr, a.m, (int)(tp0 & ROW_MASK));

    // pipeline registers: A = chunk g (values, x) and g+1 (columns); B = the next ones
    int colA[CW], colB[CW];
    VC valA[CW], valB[CW];
    XT xA[CW], xB[CW];
    // S = 8 with 4-byte values (FP32 storage): a tile's values per lane are one sector, loaded
    // whole like the column indices; valC holds the tile's second chunk until it is due
    constexpr bool whole_val_sector = S == 8 && CW == 4 && sizeof(typename P::VS) == 4;
    VC valC[CW] = {};
    {
        int col0[CW];
        load_cols<P, S, CW>(a, t_begin, 0, lane, pol_s, col0);
        if constexpr (whole_val_sector)
            load_vals_tile8(a, t_begin, lane, pol_s, valA, valC);
        else
            load_vals<P, S, CW>(a, t_begin, 0, lane, pol_s, valA);
        gather_cw<XL2>(a.x, col0, pol_x, xA);
        const int t1 = t_begin + (NC > 1 ? 0 : 1);
        const int c1 = NC > 1 ? 1 : 0;
        if (t1 < t_end) load_cols<P, S, CW>(a, t1, c1, lane, pol_s, colA);
    }

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
                a.rec_val[worker] = P::rec_from(v);
            }
        }
        if (!owned) rec_written = true;
    };

    // Plain FP64: the first tile's flag words and slot -> row map are built here, every later
    // tile's during the tile before it (after its chunk loop, the last reader of the map), so
    // that the segmented scan and the stores of that tile overlap the shared-memory atomics:
    // +3 % on both benchmark matrices.  The FP32 and mixed forms build each tile's words at its
    // start (building them early cost them 2-6 %).
    constexpr bool early_flags = std::is_same<VC, double>::value && sizeof(Acc) == 8;
    // MID (the caller gave two map buffers): the next tile's words are built half-way through
    // this tile's chunk loop, into the other buffer, overlapping the FMA chain as well
    constexpr bool mid_flags = MID && early_flags;
    // S = 8 (4-slot chunks): a tile's column indices per lane are one sector, loaded whole (+2 %
    // on the power-law matrix in every form; the FP64 kernels that build flags half-way lost
    // 7 % with it and keep two 16-byte loads)
    constexpr bool whole_col_sector = S == 8 && CW == 4 && !mid_flags;
    // the next tile's second column chunk, loaded with its first (copied on a worker's last tile
    // without a load, but then never used; initialising it costs the S = 8 FP64 kernel a spill)
    int colC[CW];
    int* rowof_cur = rowof;
    int* rowof_nxt = rowof + (mid_flags ? TILE : 0);
    uint32_t w_next = 0u;
    if constexpr (early_flags)
        w_next = tile_rows<S, YT>(a.row_ptr, a.m, t_begin * TILE, (int)(tp0 & ROW_MASK),
                                  (int)(tp1 & ROW_MASK), rb, s_words_w, rowof_cur, a.y);
    for (int t = t_begin; t < t_end; ++t) {
        const int lo = (int)(tp0 & ROW_MASK);
        const int hi = (int)(tp1 & ROW_MASK);
        uint32_t tp2 = 0u;
        RowBatch rbn{0, 0, 0, 0};
        if (t + 1 < t_end) {  // the next tile's meta, one tile ahead
            tp2 = __ldg(a.tile_ptr + t + 2);
            rbn = prefetch_rows(a.row_ptr, a.m, hi);
        }
        uint32_t w;
        if constexpr (early_flags)
            w = w_next;
        else
            w = tile_rows<S, YT>(a.row_ptr, a.m, t * TILE, lo, hi, rb, s_words_w, rowof_cur, a.y);
        const bool first_head = ((__shfl_sync(SPMV_FULL_MASK, w, 0) >> 31) & 1u) != 0u;
        const uint32_t fmask = __ballot_sync(SPMV_FULL_MASK, w != 0u);

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
        if (fmask != 0u && dc_active) {
            carry = P::carry_add(carry, warp_sum_acc<P>(dc));
            dc = P::zero();
            dc_active = false;
        }

        // A tile with a row head that does not start with one continues carry_row in its first
        // slots: lane 0's running sum starts from the carry, so the tile's head-less run T0
        // already holds the whole row (one FP64 add per tile less than adding it afterwards).
        Acc run = fmask ? P::zero() : dc;
        if (fmask != 0u && !first_head && lane == 0) run = P::carry_to_acc(carry);
        Acc head = P::zero();
        int cur_row = -1;  // row of this lane's open segment
        // the chunk loop is unrolled fully, except for wide accumulators (8 right-hand sides):
        // unrolled by 2 there, to keep the loop in the instruction cache
        constexpr int UNR = sizeof(Acc) > 16 ? 2 : NC;
#pragma unroll UNR
        for (int c = 0; c < NC; ++c) {
            // issue: columns of chunk g+2, values and x of chunk g+1
            const int t1 = t + (c + 1) / NC, c1 = (c + 1) % NC;
            const int t2 = t + (c + 2) / NC, c2 = (c + 2) % NC;
            if constexpr (whole_col_sector) {
                if (c == 0) {  // the next tile's columns, both chunks
                    if (t + 1 < t_end) load_cols_tile8(a, t + 1, lane, pol_s, colB, colC);
                } else {
#pragma unroll
                    for (int k = 0; k < CW; ++k) colB[k] = colC[k];
                }
            } else {
                if (t2 < t_end) load_cols<P, S, CW>(a, t2, c2, lane, pol_s, colB);
            }
            if (t1 < t_end) {
                if constexpr (whole_val_sector) {
                    if (c == 0) {  // the tile's second chunk, loaded with its first
#pragma unroll
                        for (int k = 0; k < CW; ++k) valB[k] = valC[k];
                    } else {  // the next tile's values, both chunks
                        load_vals_tile8(a, t1, lane, pol_s, valB, valC);
                    }
                } else {
                    load_vals<P, S, CW>(a, t1, c1, lane, pol_s, valB);
                }
                // the one-head kernels gather a full tile's x without the padding test (1 %
                // on the 27-point stencil; the per-slot kernels measured no gain from it)
                if (one_head && (long long)(t1 + 1) * TILE <= a.nnz)
                    gather_cw_full<XL2>(a.x, colA, pol_x, xB);
                else
                    gather_cw<XL2>(a.x, colA, pol_x, xB);
            }
            // multiply chunk g (its row-head bits: slot c*CW in bit CW-1)
            const uint32_t cb = (w >> (32 - (c + 1) * CW)) & ((1u << CW) - 1u);
            chunk_segments<P, S, CW>(one_head, cb, c * CW, valA, xA, run, head, cur_row,
                                     rowof_cur, lane, a);
            if constexpr (mid_flags) {
                if (c == NC / 2 - 1 && t + 1 < t_end)
                    w_next = tile_rows<S, YT>(a.row_ptr, a.m, (t + 1) * TILE, hi,
                                              (int)(tp2 & ROW_MASK), rbn, s_words_w, rowof_nxt,
                                              a.y);
            }
#pragma unroll
            for (int k = 0; k < CW; ++k) {
                colA[k] = colB[k];
                valA[k] = valB[k];
                xA[k] = xB[k];
            }
        }
        __syncwarp();  // rowof / s_words are rebuilt next
        if constexpr (mid_flags) {
            int* const t_ = rowof_cur;
            rowof_cur = rowof_nxt;
            rowof_nxt = t_;
        } else if constexpr (early_flags) {
            if (t + 1 < t_end)
                w_next = tile_rows<S, YT>(a.row_ptr, a.m, (t + 1) * TILE, hi,
                                          (int)(tp2 & ROW_MASK), rbn, s_words_w, rowof_cur, a.y);
        } else {
            rb = rbn;
        }

        tp0 = tp1;
        tp1 = tp2;
        if (fmask == 0u) {  // no row head: the whole tile continues carry_row
            dc = run;
            dc_active = true;
            continue;
        }
        const bool has = cur_row >= 0;
        if (!has) head = run;
        // T_l = head_l + (has_l ? 0 : T_{l+1}): the head-less run that starts at lane l
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
        if (!first_head) flush(carry_row, P::carry_from(T0), carry_owned);  // open row ends here
        carry_row = __shfl_sync(SPMV_FULL_MASK, cur_row, last);
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

// Resident warps per SM asked of the register allocator by the static-grid kernel k_tiles (the
// launch bound is that many warps divided by the warps of a CTA), measured per arithmetic policy
// on the 27-point stencil and the power-law matrix at 16 to 32 warps (4-warp CTAs):
//  * S = 8: 24 (80 registers) for plain FP64 (28 and 32 warps spill: 11 % and 22 % slower on the
//    power-law matrix), 32 (64 registers) for FP32 and the mixed forms' per-slot kernels (-1.4 %
//    FP32, -2.8 % mixed FP32, -1.5 % BF16 values on the power-law matrix against 24); the mixed
//    one-head kernels, which would spill at 64 registers, keep 24;
//  * plain FP64 at S = 16 and 32: 16 (128 registers).  Left alone the S = 32 kernel takes 136
//    registers and 12 warps; at 128 it does not spill and runs 13 % faster on the stencil, while
//    20 or 24 warps spill and run 1.5-2.4x slower;
//  * plain FP32: 24 at S = 16 (-5.4 % on the stencil, -1.5 % on the power-law matrix against
//    16) and 20 at S = 32 (-5.2 % on the stencil);
//  * the mixed forms: 20 (mixed FP32 -3.8 % at S = 32 and -10.5 % at S = 16 on the stencil,
//    -2.1 % at S = 16 on the power-law matrix; BF16 values -12 % at S = 16).
template <class P, int S, bool OH>
constexpr int resident_warps() {
    if constexpr (std::is_same<typename P::VC, double>::value)
        return S == 8 ? 24 : 16;
    else if constexpr (S == 8)
        return OH && !std::is_same<typename P::Acc, float>::value ? 24 : 32;
    else if constexpr (std::is_same<typename P::Acc, float>::value)
        return S == 16 ? 24 : 20;
    else
        return 20;
}

// Plain FP64 with the one-head form (long rows) keeps two slot -> row maps per warp where they
// fit in 40 KB (all but S = 32 at 8 warps), so that the next tile's map is built half-way through
// this tile's chunk loop: +1.4 % on the 27-point stencil at (32, 4, 4).  The per-slot form builds
// it after the loop: half-way cost the power-law matrix 5-9 %.
template <class P, int S, int WARPS, bool OH>
constexpr bool two_maps() {
    return OH && std::is_same<typename P::VC, double>::value && sizeof(typename P::Acc) == 8 &&
           WARPS * 2 * 32 * S * 4 <= 40 * 1024;
}

// One warp = one worker, worker = global warp index (static schedule).
template <class P, int S, int WARPS, bool OH, bool XL2>
__global__ void __launch_bounds__(WARPS * 32, (resident_warps<P, S, OH>() / WARPS))
    k_tiles(TileArgs<P> a, int tpw, int nworkers, int ntiles) {
    constexpr bool MID = two_maps<P, S, WARPS, OH>();
    __shared__ uint32_t s_words[WARPS][32];
    __shared__ int s_rowof[WARPS][(MID ? 2 : 1) * 32 * S];
    // the calibration kernel may be scheduled now; it waits for this grid's completion itself
    asm volatile("griddepcontrol.launch_dependents;");
    const int warp = threadIdx.x >> 5;
    const int worker = blockIdx.x * WARPS + warp;
    if (worker >= nworkers) return;
    tile_worker<P, S, OH, MID, XL2>(a, worker, tpw, ntiles, s_words[warp], s_rowof[warp]);
}

// Persistent tile kernels: a grid of at most the GPU's resident capacity in which each warp takes
// the next worker (tiles_per_worker consecutive tiles) from a global ticket until none is left, so
// that a warp that drew cheap tiles takes more of them; the static grid keeps each CTA's slot until
// its slowest warp is done.  After its last draw a warp counts itself done, and the grid's last
// warp puts the ticket back to zero, ready for the next launch on the stream (no reset launch or
// graph node is needed; one plan or batch runs one SpMV at a time).  The loop stays this simple on
// purpose: drawing the next worker at the start of the current one (to hide the atomic's round
// trip) or a branch for grids of one wave raised the register count from 80 to 90-96 at S = 16 and
// cost more than either saved.
template <class P, int S, bool OH, bool MID, bool XL2>
__device__ __forceinline__ void persistent_workers(const TileArgs<P>& a, int tpw, int nworkers,
                                                   int ntiles, uint32_t* s_words_w, int* rowof) {
    const int lane = threadIdx.x & 31;
    int* const ticket = a.ticket;
    for (;;) {
        int w = 0;
        if (lane == 0) w = atomicAdd(ticket, 1);
        w = __shfl_sync(SPMV_FULL_MASK, w, 0);
        if (w >= nworkers) break;
        if (w < 0) {  // cannot happen with the ticket at zero before the launch
            if (lane == 0) atomicOr(a.err, ERR_QUEUE);
            break;
        }
        tile_worker<P, S, OH, MID, XL2>(a, w, tpw, ntiles, s_words_w, rowof);
        __syncwarp();
    }
    if (lane == 0) {
        __threadfence();  // this warp's last draw comes before its count
        const int warps = (int)(gridDim.x * (blockDim.x >> 5));
        if (atomicAdd(ticket + 1, 1) == warps - 1) {  // every warp has drawn for the last time
            atomicExch(ticket, 0);
            atomicExch(ticket + 1, 0);
        }
    }
}


// No register target: without a minimum-blocks launch bound the register allocator gives the
// persistent kernels 62-90 registers (116-122 for plain FP64 at S = 16 and 32).
template <class P, int S, int WARPS, bool OH, bool XL2>
__global__ void __launch_bounds__(WARPS * 32)
    k_tiles_persistent(TileArgs<P> a, int tpw, int nworkers, int ntiles) {
    constexpr bool MID = two_maps<P, S, WARPS, OH>();
    __shared__ uint32_t s_words[WARPS][32];
    __shared__ int s_rowof[WARPS][(MID ? 2 : 1) * 32 * S];
    // the calibration kernel may be scheduled now; it waits for this grid's completion itself
    asm volatile("griddepcontrol.launch_dependents;");
    const int warp = threadIdx.x >> 5;
    persistent_workers<P, S, OH, MID, XL2>(a, tpw, nworkers, ntiles, s_words[warp],
                                           s_rowof[warp]);
}

// The same with 16 resident warps per SM asked of the register allocator (128 registers), for
// the accumulators of 4 and 8 right-hand sides: +1 % and +5 % on the batched workload (8
// right-hand sides take 148 registers and 12 warps uncapped, a 48-byte spill capped).  One and
// two right-hand sides keep the uncapped kernel: any explicit minimum changed their code and
// cost one right-hand side 3-14 %.
template <class P, int S, int WARPS, bool OH, bool XL2>
__global__ void __launch_bounds__(WARPS * 32, 16 / WARPS)
    k_tiles_persistent_capped(TileArgs<P> a, int tpw, int nworkers, int ntiles) {
    __shared__ uint32_t s_words[WARPS][32];
    __shared__ int s_rowof[WARPS][32 * S];
    asm volatile("griddepcontrol.launch_dependents;");
    const int warp = threadIdx.x >> 5;
    persistent_workers<P, S, OH, false, XL2>(a, tpw, nworkers, ntiles, s_words[warp],
                                             s_rowof[warp]);
}

// CTAs per SM of a kernel, from the occupancy calculator (at least 1)
template <class K>
int ctas_per_sm(K kernel, int threads) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, 0) != cudaSuccess) b = 0;
    return b > 0 ? b : 1;
}

// The tile kernel launch.  The persistent kernel on the GPU's resident capacity, except
//  * when one wave of the static grid (a warp per worker) holds every worker: a small matrix,
//    where the ticket's atomics would cost 2-4 us of a 10-20 us SpMV;
//  * for plain FP64 in the one-head form (long rows), which is bound by GB300's FP64 pipe: the
//    ticket's round trip between a warp's workers leaves the pipe idle, and the static grid was
//    1.5 % faster at the best schedules on the 27-point stencil (3.8 % at (32, 4, 4)).
// Measured on one box against the static grid everywhere, at the best of 32 schedules on 154
// matrices of the tuner's dataset: 4.2 % (FP64), 1.2 % (FP32), 2.4 % (mixed FP32) and 1.8 %
// (mixed BF16) faster on average above 50 us and on a par below 20 us; the power-law matrix
// 2.5 % (FP64), the 27-point stencil 4.6 % (FP32) and 10 % (mixed FP32) faster.
template <class P, int S, int WARPS, bool OH, bool XL2>
void launch_tile_kernel(const TileArgs<P>& a, int tpw, int nworkers, int ntiles, cudaStream_t st) {
    static const int static_per_sm = ctas_per_sm(k_tiles<P, S, WARPS, OH, XL2>, WARPS * 32);
    const long long blocks = ((long long)nworkers + WARPS - 1) / WARPS;
    const int sms = device_sm_count();
    constexpr bool fp64_pipe_bound = OH && std::is_same<typename P::VC, double>::value;
    if constexpr (!fp64_pipe_bound) {
        const bool persistent = a.grid_mode >= 0 ? a.grid_mode == 1
                                                 : blocks > (long long)sms * static_per_sm;
        if (persistent) {
            static const int persistent_per_sm =
                ctas_per_sm(k_tiles_persistent<P, S, WARPS, OH, XL2>, WARPS * 32);
            const long long cap = (long long)sms * persistent_per_sm;
            k_tiles_persistent<P, S, WARPS, OH, XL2>
                <<<(int)(blocks < cap ? blocks : cap), WARPS * 32, 0, st>>>(a, tpw, nworkers,
                                                                           ntiles);
            return;
        }
    }
    k_tiles<P, S, WARPS, OH, XL2><<<(int)blocks, WARPS * 32, 0, st>>>(a, tpw, nworkers, ntiles);
}

// Exchange of any carry-record type between lanes (as 32-bit words).
template <class R>
__device__ __forceinline__ R rec_shfl_xor(const R& v, int d) {
    static_assert(sizeof(R) % 4 == 0, "records are whole 32-bit words");
    constexpr int W = (int)(sizeof(R) / 4);
    uint32_t w[W];
    memcpy(w, &v, sizeof(R));
#pragma unroll
    for (int i = 0; i < W; ++i) w[i] = __shfl_xor_sync(SPMV_FULL_MASK, w[i], d);
    R r;
    memcpy(&r, w, sizeof(R));
    return r;
}

// Carry records -> y.  One warp per 32 consecutive records.  A record whose row has no other
// record (the common case) is added by its own lane.  A row with several records (a row that
// spans several workers) forms a contiguous run; the warp that holds the run's first record sums
// it cooperatively: lanes take records 32 apart, then a butterfly reduction, so a run of L
// records costs ceil(L/32) rounds instead of L dependent loads, in an order fixed by L alone
// (deterministic).  Also zeroes the leading empty rows, which lie in no tile span (the
// reference never writes them).
template <class P>
__global__ void k_calibrate(const int* __restrict__ rec_row,
                            const typename P::Rec* __restrict__ rec_val, int nworkers,
                            typename P::YT* __restrict__ y, const uint32_t* __restrict__ tile_ptr,
                            int m, uint32_t* err) {
    using Rec = typename P::Rec;
    using YT = typename P::YT;
    // launched as a programmatic dependent of the tile kernel: wait until that grid has
    // completed and its records and y are visible (returns at once for an ordinary launch)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (int base = gw * 32; base < nworkers; base += nwarps * 32) {  // warp-uniform
        const int w = base + lane;
        const int r = w < nworkers ? rec_row[w] : -1;
        const int rprev = (w > 0 && w < nworkers) ? rec_row[w - 1] : -1;
        const int rnext = w + 1 < nworkers ? rec_row[w + 1] : -1;
        const bool head = r >= 0 && rprev != r;
        const bool single = head && rnext != r;
        if (single) {
            if (r < m)
                y[r] = P::out_rec(P::rec_add(P::rec_of_y(y[r]), rec_val[w]));
            else
                atomicOr(err, ERR_BAD_TILE);
        }
        unsigned runs = __ballot_sync(SPMV_FULL_MASK, head && !single);
        while (runs) {
            const int src = __ffs(runs) - 1;
            runs &= runs - 1;
            const int w0 = base + src;
            const int row = __shfl_sync(SPMV_FULL_MASK, r, src);
            Rec acc = P::rec_of_y(YT(0));
            for (int v = w0 + lane;; v += 32) {
                const bool in = v < nworkers && rec_row[v] == row;
                if (in) acc = P::rec_add(acc, rec_val[v]);
                if (__ballot_sync(SPMV_FULL_MASK, in) != SPMV_FULL_MASK) break;  // the run ended
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) acc = P::rec_add(acc, rec_shfl_xor(acc, d));
            if (lane == 0) {
                if (row < m)
                    y[row] = P::out_rec(P::rec_add(P::rec_of_y(y[row]), acc));
                else
                    atomicOr(err, ERR_BAD_TILE);
            }
        }
    }
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int lead = min((int)(tile_ptr[0] & ROW_MASK), m);
    for (long long r = tid; r < lead; r += stride) y[r] = YT(0);
}

// The calibration launch, as a programmatic dependent of the tile kernel launched just before
// on the same stream: it is scheduled while the tile kernel drains and waits for it on the
// device (griddepcontrol.wait), which hides the launch gap between the two.
template <class P>
cudaError_t launch_calibrate(const TileArgs<P>& a, int nworkers, cudaStream_t st) {
    const int cb = grid_for(nworkers, 256, 8);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cb);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = (a.phase & 1) ? 1 : 0;  // a dependent only when the tile kernel precedes it
    return cudaLaunchKernelEx(&cfg, k_calibrate<P>, a.rec_row, a.rec_val, nworkers, a.y,
                              a.tile_ptr, a.m, a.err);
}

template <class P, int S, int WARPS>
cudaError_t launch_tiles_t(const TileArgs<P>& a, int tpw, int nworkers, int ntiles,
                           cudaStream_t st) {
    if (nworkers > 0 && (a.phase & 1)) {
        if (!a.ticket) return cudaErrorInvalidValue;
        if constexpr (sizeof(typename P::Acc) <= 8) {  // scalar accumulators: either form
            // chunk form x gather path, both fixed by the plan
            if (a.one_head && a.x_l2)
                launch_tile_kernel<P, S, WARPS, true, true>(a, tpw, nworkers, ntiles, st);
            else if (a.one_head)
                launch_tile_kernel<P, S, WARPS, true, false>(a, tpw, nworkers, ntiles, st);
            else if (a.x_l2)
                launch_tile_kernel<P, S, WARPS, false, true>(a, tpw, nworkers, ntiles, st);
            else
                launch_tile_kernel<P, S, WARPS, false, false>(a, tpw, nworkers, ntiles, st);
        } else {
            launch_tile_kernel<P, S, WARPS, false, false>(a, tpw, nworkers, ntiles, st);
        }
    }
    if (a.phase & 2) {
        const cudaError_t e = launch_calibrate(a, nworkers, st);
        if (e != cudaSuccess) return e;
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
