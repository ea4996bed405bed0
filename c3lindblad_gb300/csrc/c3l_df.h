// Double-float arithmetic on the FP32 pipe, shared by the Krylov and tensor
// kernels.  GB300's FP64 pipe is narrow (about 1/58 of the FP32 rate), so
// FP64-accurate sums of products are formed from FP32 (hi, lo) pairs.
#pragma once

#include <cuda_runtime.h>

// Double-float arithmetic on the FP32 pipe (a value is an unevaluated sum hi + lo
// of two floats).  two_sum is Knuth's error-free addition, the product split
// p + e = a_hi b_hi uses one FMA (Dekker's product with a fused multiply-add);
// the cross terms a_hi b_lo + a_lo b_hi are added to the error term and
// a_lo b_lo (2^-48 relative) is dropped.  The _rn intrinsics keep the compiler
// from contracting the additions into FMAs, which would break the
// transformations.
static __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// (S, C) += (ahi + alo)(bhi + blo)
static __device__ __forceinline__ void df_mac(float& S, float& C, float ahi, float alo, float bhi, float blo) {
    const float p = __fmul_rn(ahi, bhi);
    float e = fmaf(ahi, bhi, -p);
    e = fmaf(ahi, blo, fmaf(alo, bhi, e));
    float s, t;
    two_sum(S, p, s, t);
    S = s;
    C = __fadd_rn(C, __fadd_rn(t, e));
}
// (S, C) += (S2, C2)
static __device__ __forceinline__ void df_add(float& S, float& C, float S2, float C2) {
    float s, t;
    two_sum(S, S2, s, t);
    S = s;
    C = __fadd_rn(C, __fadd_rn(C2, t));
}
// double-float sum over the warp, valid in lane 0
static __device__ __forceinline__ void df_warp_sum(float& S, float& C) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float S2 = __shfl_down_sync(0xffffffffu, S, o);
        const float C2 = __shfl_down_sync(0xffffffffu, C, o);
        df_add(S, C, S2, C2);
    }
}
// FP32 (hi, lo) pair of a double
static __device__ __forceinline__ void split_d(double x, float& hi, float& lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

