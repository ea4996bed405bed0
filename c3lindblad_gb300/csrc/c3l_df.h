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
// The same pair from the bits of x, with no FP64 instruction (the conversions
// above run on the narrow FP64 pipe): hi keeps the sign, the exponent and the
// top 23 fraction bits (x truncated to 24 significant bits), lo = x - hi is
// the low 29 fraction bits times 2^(e - 52), rounded once to FP32, so
// |hi + lo - x| <= 2^-48 |x|.  Exponents outside [-100, 100] (and zeros,
// subnormals, infinities, NaN) take the FP64 route.
static __device__ __forceinline__ void split_d_bits(double x, float& hi, float& lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int top = (unsigned int)(b >> 32);
    const int e = (int)((top >> 20) & 0x7FFu) - 1023;
    if (e < -100 || e > 100) {
        split_d(x, hi, lo);
        return;
    }
    const unsigned int sign = top & 0x80000000u;
    const unsigned long long m = b & 0x000FFFFFFFFFFFFFull;
    hi = __uint_as_float(sign | ((unsigned int)(e + 127) << 23) | (unsigned int)(m >> 29));
    const float r = __uint2float_rn((unsigned int)(m & 0x1FFFFFFFull));
    // r 2^(e - 52) = (r 2^-64) 2^(e + 12): both factors normal floats for |e| <= 100
    const float l = __fmul_rn(__fmul_rn(r, 0x1p-64f), __uint_as_float((unsigned int)(e + 139) << 23));
    lo = sign ? -l : l;
}

