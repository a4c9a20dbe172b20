// policies_mixed.cuh -- arithmetic policy of the mixed-precision forms: values stored in FP32 or
// BF16, x and y in FP32, products and the in-tile segmented sum in compensated FP32 (TwoProduct
// by FMA + TwoSum, a float-float accumulator), carries between tiles and the calibration of rows
// that span several tiles or workers in FP64.  No counterpart in the reference, which only has
// the USE_DOUBLE switch (spmv_cuda/common.h:27-31).  Shared by spmv_mixed.cu (FP32 storage) and
// spmv_mixed_bf16.cu (BF16 storage), one translation unit per storage type.
#pragma once
#include "internal.h"
#include "tile_kernel_tma.cuh"

namespace spmv {

// Error-free transforms with explicitly rounded intrinsics, so that nvcc cannot contract
// or reassociate them (Knuth TwoSum; TwoProduct through the exact FMA residual).
__device__ __forceinline__ float2 ff_add_product(float v, float x, float2 a) {
    const float p = __fmul_rn(v, x);
    const float ep = __fmaf_rn(v, x, -p);
    const float s = __fadd_rn(a.x, p);
    const float bb = __fsub_rn(s, a.x);
    const float es = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    return make_float2(s, __fadd_rn(a.y, __fadd_rn(es, ep)));
}
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float bb = __fsub_rn(s, a.x);
    const float es = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
    return make_float2(s, __fadd_rn(__fadd_rn(a.y, b.y), es));
}

// The carry of a worker's open row stays a float-float pair (compensated, about 48 significant
// bits) from tile to tile -- converting to FP64 on every tile would cost two conversions and
// two adds on GB300's narrow FP64 pipe per tile -- and becomes FP64 when the row is handed to
// another worker (the carry record) and in the calibration that adds those records.
template <typename VSTORE>
struct PolMixed {
    using VS = VSTORE;
    using VC = float;
    using XT = float;
    using YT = float;
    using Acc = float2;
    using Carry = float2;
    using Rec = double;
    __device__ static float2 zero() { return make_float2(0.f, 0.f); }
    __device__ static float2 carry_zero() { return make_float2(0.f, 0.f); }
    __device__ static float2 fma(float v, float x, float2 a) { return ff_add_product(v, x, a); }
    __device__ static float2 add(float2 a, float2 b) { return ff_add(a, b); }
    __device__ static float2 carry_from(float2 a) { return a; }
    __device__ static float2 carry_to_acc(float2 c) { return c; }
    __device__ static float2 carry_add(float2 c, float2 a) { return ff_add(c, a); }
    __device__ static float out_acc(float2 a) { return __fadd_rn(a.x, a.y); }
    __device__ static float out_carry(float2 c) { return __fadd_rn(c.x, c.y); }
    __device__ static double rec_from(float2 c) { return (double)c.x + (double)c.y; }
    __device__ static double rec_add(double a, double b) { return a + b; }
    __device__ static double rec_of_y(float y) { return (double)y; }
    __device__ static float out_rec(double r) { return __double2float_rn(r); }
};

template <typename VSTORE>
cudaError_t launch_mixed_t(const MixedLaunch& l, const TileConfig& cfg, cudaStream_t st) {
    TileArgs<PolMixed<VSTORE>> a;
    a.row_ptr = l.row_ptr;
    a.col = l.col;
    a.val = static_cast<const VSTORE*>(l.val);
    a.x = l.x;
    a.y = l.y;
    a.tile_ptr = l.tile_ptr;
    a.rec_row = l.rec_row;
    a.rec_val = l.rec_val;
    a.err = l.err;
    a.m = l.m;
    a.n = l.n;
    a.nnz = l.nnz;
    a.phase = l.phase;
    a.one_head = l.one_head;
    a.x_l2 = l.x_l2;
    a.ticket = l.ticket;
    a.grid_mode = l.grid_mode;
    return launch_tiles_any(a, cfg, st);
}

}  // namespace spmv
