// Host checks of the double-float arithmetic in zeroslam_gb300/csrc/ba_df.cuh:
// the error-free transformations are exact, and sums, products and
// compensated dot products (including ones that cancel to 1e-5 of their terms)
// stay within a few eps^2 of their operands, against long double references.
// Prints OK or the first failure.
#include <cmath>
#include <cstdio>
#include <random>

#include "ba_df.cuh"

using zs::df;
typedef long double ld;

static int fail(const char* what, int i, ld got, ld want, ld bound) {
    std::printf("FAIL %s case %d: got %.21Lg want %.21Lg bound %.3Lg\n", what, i, got, want, bound);
    return 1;
}

static ld val(df x) { return (ld)x.hi + (ld)x.lo; }

int main() {
    const ld eps = std::ldexp((ld)1, -24);
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> mant(-1.0, 1.0);
    std::uniform_int_distribution<int> ex(-20, 20);
    auto rf = [&]() { return (float)std::ldexp(mant(rng), ex(rng)); };
    auto rdf = [&]() {
        const double d = std::ldexp(mant(rng), ex(rng)) * (1.0 + 1e-9 * mant(rng));
        return zs::df_from_double(d);
    };
    for (int i = 0; i < 200000; ++i) {
        const float a = rf(), b = rf();
        float e;
        const float s = zs::two_sum(a, b, e);
        if ((ld)s + (ld)e != (ld)a + (ld)b) return fail("two_sum", i, (ld)s + e, (ld)a + b, 0);
        const float p = zs::two_prod(a, b, e);
        if ((ld)p + (ld)e != (ld)a * (ld)b) return fail("two_prod", i, (ld)p + e, (ld)a * b, 0);
        const float big = std::fabs(a) >= std::fabs(b) ? a : b, small = std::fabs(a) >= std::fabs(b) ? b : a;
        const float f = zs::fast_two_sum(big, small, e);
        if ((ld)f + (ld)e != (ld)big + (ld)small) return fail("fast_two_sum", i, (ld)f + e, (ld)big + small, 0);

        const df x = rdf(), y = rdf();
        const ld bx = std::fabs(val(x)), by = std::fabs(val(y));
        ld want = val(x) + val(y), bound = 4 * eps * eps * (bx + by);
        if (std::fabs(val(zs::df_add(x, y)) - want) > bound) return fail("df_add", i, val(zs::df_add(x, y)), want, bound);
        want = val(x) * val(y);
        bound = 4 * eps * eps * bx * by;
        if (std::fabs(val(zs::df_mul(x, y)) - want) > bound) return fail("df_mul", i, val(zs::df_mul(x, y)), want, bound);
        want = val(x) * (ld)a;
        bound = 4 * eps * eps * bx * std::fabs((ld)a);
        if (std::fabs(val(zs::df_mul_f(x, a)) - want) > bound)
            return fail("df_mul_f", i, val(zs::df_mul_f(x, a)), want, bound);
        const double d = std::ldexp(mant(rng), ex(rng));
        if (std::fabs((ld)zs::df_to_double(zs::df_from_double(d)) - (ld)d) > 2 * eps * eps * std::fabs((ld)d))
            return fail("df_from_double", i, zs::df_to_double(zs::df_from_double(d)), d, 0);
    }
    // compensated dot products of 2..12 terms, half of them built to cancel:
    // sum a_k x_k + c ~ 1e-5 of sum |a_k x_k|
    for (int i = 0; i < 100000; ++i) {
        const int n = 2 + i % 11;
        float a[12];
        df x[12];
        ld want = 0, mag = 0;
        zs::df_dot dot;
        for (int k = 0; k < n; ++k) {
            a[k] = rf();
            x[k] = rdf();
            dot.add(a[k], x[k]);
            want += (ld)a[k] * val(x[k]);
            mag += std::fabs((ld)a[k] * val(x[k]));
        }
        if (i % 2) {  // add a double-float that cancels the sum down to ~1e-5
            const df cx = zs::df_from_double((double)(-want * (1 + 1e-5L)));
            dot.add_df(cx);
            want += val(cx);
            mag += std::fabs(val(cx));
        }
        const ld bound = 2 * (n + 2) * eps * eps * mag;
        const ld got = val(dot.result());
        if (std::fabs(got - want) > bound) return fail("df_dot", i, got, want, bound);
    }
    std::printf("OK\n");
    return 0;
}
