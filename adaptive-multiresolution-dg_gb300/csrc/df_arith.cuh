// FP32-pair (double-float) arithmetic of the mixed-mode stage updates (hi + lo with |lo| <=
// ulp(hi) / 2): the error-free transformations two-sum (Knuth) and the FMA-based exact product,
// combined as in the double-double algorithms of Hida, Li and Bailey.  Shared by the linear and the
// batched stage kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"

namespace amdg {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& ph, float& pl) {
    const float p = __fmul_rn(ah, bh);
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
    fast_two_sum(p, e, ph, pl);
}
__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float& sh, float& sl) {
    float s, e;
    two_sum(ah, bh, s, e);
    e = __fadd_rn(e, __fadd_rn(al, bl));
    fast_two_sum(s, e, sh, sl);
}
// out = a*un + b*(us + dt*rhs) on (hi, lo) pairs; rhs is only FP32-accurate, so dt*rhs is one FP32 product
__device__ __forceinline__ void df_stage_update(const DFState& df, int64_t i, float rhs) {
    const float p = __fmul_rn(df.dt, rhs);
    float th, tl;
    two_sum(df.us_hi[i], p, th, tl);
    tl = __fadd_rn(tl, df.us_lo[i]);
    fast_two_sum(th, tl, th, tl);
    float x1h, x1l, x2h, x2l, vh, vl;
    df_mul(df.ah, df.al, df.un_hi[i], df.un_lo[i], x1h, x1l);
    df_mul(df.bh, df.bl, th, tl, x2h, x2l);
    df_add(x1h, x1l, x2h, x2l, vh, vl);
    df.out_hi[i] = vh;
    df.out_lo[i] = vl;
}

}  // namespace amdg
