// bella_df.cuh -- double-float ("FP32 pair") arithmetic for the Krylov path.
//
// GB300 executes FP64 at 1/64 of its FP32 rate (measured 1.01 vs 64.2
// TFLOP/s), which makes the FP64 stencil FP64-pipe bound at ~14 % of HBM
// bandwidth.  A value is kept as hi + lo with |lo| <= ulp(hi)/2 (about 48
// significant bits, ~1e-14 relative) and operated on with error-free
// transformations on the FP32 pipe:
//   two-sum (Knuth), fast-two-sum (Dekker), two-product via fmaf,
// following Dekker (1971) / Knuth TAOCP vol. 2 and the double-double
// algorithms of Hida, Li & Bailey (2001).  Every operation uses the _rn
// intrinsics so the compiler cannot contract or reassociate them.
#pragma once
#include <cuda_runtime.h>

namespace bella {

struct __align__(8) dfloat {
    float hi, lo;
    __host__ __device__ __forceinline__ dfloat() {}
    __host__ __device__ __forceinline__ dfloat(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ dfloat(int v) : hi((float)v), lo(0.f) {}
    __device__ __forceinline__ dfloat(double d) {
        hi = __double2float_rn(d);
        lo = __double2float_rn(d - (double)hi);
    }
    __device__ __forceinline__ double to_double() const { return (double)hi + (double)lo; }
};

// s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// accurate double-float sum (relative error ~2^-47 even under cancellation)
__device__ __forceinline__ dfloat df_add(dfloat a, dfloat b) {
    float s, e, t, f;
    two_sum(a.hi, b.hi, s, e);
    two_sum(a.lo, b.lo, t, f);
    e = __fadd_rn(e, t);
    fast_two_sum(s, e, s, e);
    e = __fadd_rn(e, f);
    fast_two_sum(s, e, s, e);
    return dfloat(s, e);
}

__device__ __forceinline__ dfloat df_neg(dfloat a) { return dfloat(-a.hi, -a.lo); }

__device__ __forceinline__ dfloat df_mul(dfloat a, dfloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    float s;
    fast_two_sum(p, e, s, e);
    return dfloat(s, e);
}

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) { return df_add(a, b); }
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) { return df_mul(a, b); }
__device__ __forceinline__ dfloat &operator+=(dfloat &a, dfloat b) { a = df_add(a, b); return a; }

// x / 2, exact in every type (scaling by a power of two)
template <typename T> __device__ __forceinline__ T half_of(T a) { return (T)0.5 * a; }
template <> __device__ __forceinline__ dfloat half_of<dfloat>(dfloat a) { return dfloat(a.hi * 0.5f, a.lo * 0.5f); }

// Inner-product accumulator: each product a*b of two double-floats is formed
// to ~2^-48 relative (exact hi*hi via fmaf plus the cross terms) and summed
// into a compensated FP32 pair; converted to FP64 once per thread.
struct DFAcc {
    float hi, lo;
    __device__ __forceinline__ void zero() { hi = 0.f; lo = 0.f; }
    __device__ __forceinline__ void add_prod(dfloat a, dfloat b) {
        const float p = __fmul_rn(a.hi, b.hi);
        float e = __fmaf_rn(a.hi, b.hi, -p);
        e = __fmaf_rn(a.hi, b.lo, e);
        e = __fmaf_rn(a.lo, b.hi, e);
        float s, err;
        two_sum(hi, p, s, err);
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(err, e));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

}  // namespace bella
