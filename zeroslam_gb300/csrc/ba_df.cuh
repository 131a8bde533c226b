// Double-float arithmetic: a value held as an unevaluated sum hi + lo of two
// FP32 numbers (|lo| <= ulp(hi) / 2), about 48 significant bits, built from
// error-free transformations:
//   two_sum       Knuth, The Art of Computer Programming vol. 2, 4.2.2
//   fast_two_sum  Dekker, "A floating-point technique for extending the
//                 available precision", Numer. Math. 18 (1971)
//   two_prod      the FMA form of Dekker's exact product
// and compensated dot products in the manner of Ogita, Rump and Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005), Dot2,
// extended to double-float operands. On GB300 the FP32 pipe is 64 times the
// FP64 pipe, so the mixed form's FP64-accurate Schur operator runs in these
// instead of in FP64.
//
// Error bounds used by the callers: df_add(x, y) and the dot products err by
// at most a few eps^2 (|x| + |y|) (eps = 2^-24), i.e. absolutely, relative to
// the operands, not to a result that cancels. That is the accuracy the
// operator needs: its cancellation (pose motion against landmark motion,
// ~1e-4 relative in the weakest directions) leaves ~1e-10 relative.
//
// The transformations must not be contracted or reassociated: on the device
// they use the _rn intrinsics; host code (tests) must be compiled without
// -ffast-math.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define ZS_DF_HD __host__ __device__ __forceinline__
#else
#define ZS_DF_HD inline
#endif

namespace zs {

struct df {
    float hi, lo;
};

ZS_DF_HD float df_radd(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
ZS_DF_HD float df_rsub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
ZS_DF_HD float df_rmul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
ZS_DF_HD float df_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

// s + e == a + b exactly.
ZS_DF_HD float two_sum(float a, float b, float& e) {
    const float s = df_radd(a, b);
    const float bp = df_rsub(s, a);
    e = df_radd(df_rsub(a, df_rsub(s, bp)), df_rsub(b, bp));
    return s;
}
// s + e == a + b exactly when |a| >= |b| or a == 0.
ZS_DF_HD float fast_two_sum(float a, float b, float& e) {
    const float s = df_radd(a, b);
    e = df_rsub(b, df_rsub(s, a));
    return s;
}
// p + e == a * b exactly.
ZS_DF_HD float two_prod(float a, float b, float& e) {
    const float p = df_rmul(a, b);
    e = df_fma(a, b, -p);
    return p;
}

ZS_DF_HD df df_make(float hi, float lo) {
    df r;
    r.hi = fast_two_sum(hi, lo, r.lo);
    return r;
}
ZS_DF_HD df df_zero() { return df{0.f, 0.f}; }
ZS_DF_HD df df_neg(df x) { return df{-x.hi, -x.lo}; }

ZS_DF_HD df df_add(df x, df y) {
    float e;
    const float s = two_sum(x.hi, y.hi, e);
    e = df_radd(e, df_radd(x.lo, y.lo));
    return df_make(s, e);
}
ZS_DF_HD df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

// x * b for a float b.
ZS_DF_HD df df_mul_f(df x, float b) {
    float e;
    const float p = two_prod(x.hi, b, e);
    e = df_fma(x.lo, b, e);
    return df_make(p, e);
}
// x * y.
ZS_DF_HD df df_mul(df x, df y) {
    float e;
    const float p = two_prod(x.hi, y.hi, e);
    e = df_fma(x.hi, y.lo, df_fma(x.lo, y.hi, e));
    return df_make(p, e);
}

// Compensated accumulator for sum_k a_k x_k (a_k float, x_k double-float):
// the leading products are exact (two_prod), their running sum is exact
// (two_sum), and all error terms and the x_k.lo products meet in c.
struct df_dot {
    float s = 0.f, c = 0.f;
    ZS_DF_HD void add(float a, df x) {
        float pe, se;
        const float p = two_prod(a, x.hi, pe);
        s = two_sum(s, p, se);
        c = df_radd(c, df_radd(df_radd(pe, se), df_rmul(a, x.lo)));
    }
    ZS_DF_HD void add_df(df x) {
        float se;
        s = two_sum(s, x.hi, se);
        c = df_radd(c, df_radd(se, x.lo));
    }
    ZS_DF_HD df result() const { return df_make(s, c); }
};

ZS_DF_HD df df_from_double(double d) {
    const float hi = (float)d;
    return df{hi, (float)(d - (double)hi)};
}
ZS_DF_HD double df_to_double(df x) { return (double)x.hi + (double)x.lo; }

}  // namespace zs
