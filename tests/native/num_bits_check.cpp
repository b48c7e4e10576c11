// Host check of the double helpers of fractalshades_gb300/csrc/fsg_num.cuh
// that replace FP64 operations by tests on the bit patterns: each must give
// the bits of the double operation it stands for, for every finite, zero,
// subnormal, infinite and NaN operand.  The header is compiled for the host
// with the device intrinsics it uses defined by memcpy.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>
static inline long long __double_as_longlong(double d) { long long x; memcpy(&x, &d, 8); return x; }
static inline double __longlong_as_double(long long x) { double d; memcpy(&d, &x, 8); return d; }
static inline int __float_as_int(float f) { int x; memcpy(&x, &f, 4); return x; }
static inline float __int_as_float(int x) { float f; memcpy(&f, &x, 4); return f; }
using std::max;
using std::min;
#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif
#include "../../fractalshades_gb300/csrc/fsg_num.cuh"

static unsigned long long bits(double d) { unsigned long long x; memcpy(&x, &d, 8); return x; }
static bool same(double a, double b) { return (std::isnan(a) && std::isnan(b)) || bits(a) == bits(b); }
// the promoted complex product as the reference computes it (each operation
// rounded once: volatile temporaries, built without contraction)
static double2 promoted_product(double s, double2 b) {
    volatile double p = s * b.x, q = 0. * b.y, r = s * b.y, t = 0. * b.x;
    return make_double2(p - q, r + t);
}

int main(int argc, char **argv) {
    const long cases = argc > 1 ? atol(argv[1]) : 2000000;
    const std::vector<double> special = {
        0., -0., 1., -1., 2., -2., 0.5, 3., -3., 1e-300, -1e-300, 1e-310, -1e-310,
        2.225073858507201e-308, -2.225073858507201e-308, 8.98846567431158e307, -8.98846567431158e307,
        4.9e-324, -4.9e-324, 2.2250738585072014e-308, 1e308, -1e308, 1.7976931348623157e308,
        INFINITY, -INFINITY, NAN, -NAN};
    std::mt19937_64 g(7);
    auto draw = [&]() {
        if (g() % 8 == 0) return special[g() % special.size()];
        const double m = std::ldexp((double)(g() >> 11) * 0x1p-53, (int)(g() % 2200) - 1100);
        return (g() & 1) ? -m : m;
    };
    long bad = 0;
    for (long i = 0; i < cases; i++) {
        const double s = draw(), x = draw(), y = draw(), t = draw();
        const double2 f = rmul(s, make_double2(x, y)), r = promoted_product(s, make_double2(x, y));
        if (!same(f.x, r.x) || !same(f.y, r.y)) {
            if (bad++ < 5) printf("rmul(%a, %a, %a)\n", s, x, y);
        }
        volatile double two_x = x * 2.;
        if (!same(d_twice(x), two_x)) { if (bad++ < 5) printf("d_twice(%a)\n", x); }
        const double2 f2 = rmul2(make_double2(x, y)), r2 = promoted_product(2., make_double2(x, y));
        if (!same(f2.x, r2.x) || !same(f2.y, r2.y)) {
            if (bad++ < 5) printf("rmul2(%a, %a)\n", x, y);
        }
        volatile double xx = x * x, yy = y * y, xy = x * y, yx = y * x;
        const double2 sq2 = csq(make_double2(x, y));
        if (!same(sq2.x, xx - yy) || !same(sq2.y, xy + yx)) { if (bad++ < 5) printf("csq(%a, %a)\n", x, y); }
        const int k = (int)(g() % 2300) - 1150;
        volatile double pk = pow2d(k);
        const double2 fp = rmul_p2(k, make_double2(x, y)), rp = promoted_product(pk, make_double2(x, y));
        if (!same(fp.x, rp.x) || !same(fp.y, rp.y)) { if (bad++ < 5) printf("rmul_p2(%d, %a, %a)\n", k, x, y); }
        // |z| < r without the hypot: where abs_cmp decides, hypot's answer
        // (radii drawn at random and within a few units of |z|)
        {
            const double h = std::hypot(x, y);
            const AbsScaled as = abs_scaled(make_double2(x, y));
            const double near = std::isfinite(h) ? h * (1. + std::ldexp((double)((long)(g() % 2001) - 1000), -52 + (int)(g() % 12))) : t;
            for (double r : {t, std::fabs(t), near, std::nextafter(h, INFINITY), std::nextafter(h, 0.), h}) {
                const int c = abs_cmp(as, r);
                if (c >= 0 && c != (h < r ? 1 : 0)) {
                    if (bad++ < 5) printf("abs_cmp(%a, %a; %a) = %d\n", x, y, r, c);
                }
            }
        }
        if (d_ge0(x) != (x >= 0.) || d_le0(x) != (x <= 0.) || d_lt0(x) != (x < 0.)) {
            if (bad++ < 5) printf("sign tests(%a)\n", x);
        }
        if (!same(d_abs(x), std::fabs(x))) { if (bad++ < 5) printf("d_abs(%a)\n", x); }
        if (d_is0(x) != (x == 0.)) { if (bad++ < 5) printf("d_is0(%a)\n", x); }
        if (d_nonfinite(x) != !std::isfinite(x)) { if (bad++ < 5) printf("d_nonfinite(%a)\n", x); }
        if (d_abs_le(x, y) != (std::fabs(x) <= std::fabs(y))) {
            if (bad++ < 5) printf("d_abs_le(%a, %a)\n", x, y);
        }
        volatile double sq = x * x + y * y, tt = t * t;
        if (d_sq_gt(sq, tt) != (sq > tt)) { if (bad++ < 5) printf("d_sq_gt(%a, %a)\n", (double)sq, (double)tt); }
        if (d_sq_lt(sq, tt) != (sq < tt)) { if (bad++ < 5) printf("d_sq_lt(%a, %a)\n", (double)sq, (double)tt); }
        const double nan = (g() & 1) ? NAN : -NAN;
        if (d_sq_gt(nan, tt) || d_sq_lt(nan, tt) || d_sq_gt(sq, nan) || d_sq_lt(sq, nan)) {
            if (bad++ < 5) printf("NaN compare\n");
        }
        // Xrange sum of squares against a square, through the co-exponent
        xf a; a.m = sq; a.e = (int)(g() % 400) - 200;
        double o0, o1; int e;
        xr_coexp_r(a.m, a.e, tt, 0, o0, o1, e);
        if (xf_sq_lt_s(a, tt) != (o0 < o1)) { if (bad++ < 5) printf("xf_sq_lt_s\n"); }
    }
    printf("%ld cases, %ld mismatches\n", cases, bad);
    return bad != 0;
}
