// policies_plain.cuh -- arithmetic policies of the plain forms (the reference's USE_DOUBLE=1 /
// USE_DOUBLE=0 builds, spmv_cuda/common.h:27-31): values, x, y, accumulation and carries all in
// the value type, one fused multiply-add per non-zero.  Shared by spmv_plain_f64.cu and
// spmv_plain_f32.cu, one translation unit per value type so that the build runs them in
// parallel.
#pragma once
#include "internal.h"
#include "tile_kernel_tma.cuh"

namespace spmv {

struct PolF64 {
    using VS = double;
    using VC = double;
    using XT = double;
    using YT = double;
    using Acc = double;
    using Carry = double;
    __device__ static double zero() { return 0.0; }
    __device__ static double carry_zero() { return 0.0; }
    __device__ static double fma(double v, double x, double a) { return ::fma(v, x, a); }
    __device__ static double add(double a, double b) { return a + b; }
    __device__ static double carry_add(double c, double a) { return c + a; }
    __device__ static double carry_from(double a) { return a; }
    __device__ static double carry_to_acc(double c) { return c; }
    __device__ static double out_acc(double a) { return a; }
    __device__ static double out_carry(double c) { return c; }
    using Rec = double;
    __device__ static double rec_from(double c) { return c; }
    __device__ static double rec_add(double a, double b) { return a + b; }
    __device__ static double rec_of_y(double y) { return y; }
    __device__ static double out_rec(double r) { return r; }
};

struct PolF32 {
    using VS = float;
    using VC = float;
    using XT = float;
    using YT = float;
    using Acc = float;
    using Carry = float;
    __device__ static float zero() { return 0.0f; }
    __device__ static float carry_zero() { return 0.0f; }
    __device__ static float fma(float v, float x, float a) { return fmaf(v, x, a); }
    __device__ static float add(float a, float b) { return a + b; }
    __device__ static float carry_add(float c, float a) { return c + a; }
    __device__ static float carry_from(float a) { return a; }
    __device__ static float carry_to_acc(float c) { return c; }
    __device__ static float out_acc(float a) { return a; }
    __device__ static float out_carry(float c) { return c; }
    using Rec = float;
    __device__ static float rec_from(float c) { return c; }
    __device__ static float rec_add(float a, float b) { return a + b; }
    __device__ static float rec_of_y(float y) { return y; }
    __device__ static float out_rec(float r) { return r; }
};

template <class P>
inline cudaError_t launch_plain_any(const PlainLaunch& l, const TileConfig& cfg, cudaStream_t st) {
    TileArgs<P> a;
    a.row_ptr = l.row_ptr;
    a.col = l.col;
    a.val = static_cast<const typename P::VS*>(l.val);
    a.x = static_cast<const typename P::XT*>(l.x);
    a.y = static_cast<typename P::YT*>(l.y);
    a.tile_ptr = l.tile_ptr;
    a.rec_row = l.rec_row;
    a.rec_val = static_cast<typename P::Rec*>(l.rec_val);
    a.err = l.err;
    a.m = l.m;
    a.n = l.n;
    a.nnz = l.nnz;
    a.phase = l.phase;
    a.one_head = l.one_head;
    a.x_l2 = l.x_l2;
    a.ticket = l.ticket;
    a.grid_mode = l.grid_mode;
    return launch_tiles_any<P>(a, cfg, st);
}

}  // namespace spmv
