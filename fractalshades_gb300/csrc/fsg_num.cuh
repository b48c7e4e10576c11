// fsg_num.cuh -- device arithmetic for the escape-time kernels.
//
//   * complex double helpers with the operation order of numba / CPython
//     complex128 ((a+bi)(c+di) = (ac-bd) + (ad+bc)i, a float is promoted to
//     complex(x, 0) before a complex product);
//   * xc: the "Xrange" extended-exponent complex of the reference
//     (numpy_utils/numba_xr.py): complex128 mantissa + int32 exponent shared by
//     both parts, lazy renormalisation when the unbiased exponent of a part
//     leaves [-100, 100];
//   * fe: the FP32-mantissa / int32-exponent complex used by the fast kernels,
//     normalised so that max(|x|, |y|) is in [1, 2) (zero carries FE_ZERO_E).
//
// The translation units that must reproduce the reference's rounding are
// compiled with -fmad=false, so every double operation below rounds once.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define FSG_DEV __device__ __forceinline__

// ---------------------------------------------------------------------------
// double tests on the bit patterns.  GB300 issues a double compare to the
// FP64 pipe, where it costs what a multiply costs (a warp instruction holds
// the pipe for about 64 cycles); the forms below read the bits on the
// integer pipes and decide exactly as the double compare does, NaN included.
// ---------------------------------------------------------------------------
#define FSG_D_INF_BITS 0x7ff0000000000000ULL
FSG_DEV unsigned long long dbits(double m) { return (unsigned long long)__double_as_longlong(m); }
// m == 0. (+0 or -0)
FSG_DEV bool d_is0(double m) { return (dbits(m) << 1) == 0ULL; }
// inf or NaN
FSG_DEV bool d_nonfinite(double m) { return (dbits(m) & FSG_D_INF_BITS) == FSG_D_INF_BITS; }
// |a| <= |b| (false when either is NaN)
FSG_DEV bool d_abs_le(double a, double b) {
    const unsigned long long x = dbits(a) << 1, y = dbits(b) << 1;
    return x <= y && y <= (FSG_D_INF_BITS << 1);
}
// s > t and s < t for s >= +0 or NaN (a sum of squares, never -0) and t a
// square (never -0): non-negative doubles order as their bit patterns read as
// signed integers, and a NaN on either side (of either sign) decides false
FSG_DEV bool d_sq_gt(double s, double t) {
    const long long a = __double_as_longlong(s), b = __double_as_longlong(t);
    return a > b && (unsigned long long)a <= FSG_D_INF_BITS
           && (dbits(t) << 1) <= (FSG_D_INF_BITS << 1);
}
FSG_DEV bool d_sq_lt(double s, double t) {
    const long long a = __double_as_longlong(s), b = __double_as_longlong(t);
    return a < b && (unsigned long long)a <= FSG_D_INF_BITS
           && (dbits(t) << 1) <= (FSG_D_INF_BITS << 1);
}
// x >= 0., x <= 0., x < 0. and fabs(x) on the bits (either zero is >= 0
// and <= 0, a NaN is neither)
FSG_DEV bool d_ge0(double x) { return dbits(x) <= FSG_D_INF_BITS || dbits(x) == 0x8000000000000000ULL; }
FSG_DEV bool d_le0(double x) {
    return dbits(x) == 0ULL || ((dbits(x) >> 63) && (dbits(x) << 1) <= (FSG_D_INF_BITS << 1));
}
FSG_DEV bool d_lt0(double x) {
    const unsigned long long b = dbits(x);
    return (b >> 63) && (b << 1) != 0ULL && (b << 1) <= (FSG_D_INF_BITS << 1);
}
FSG_DEV double d_abs(double x) { return __longlong_as_double((long long)(dbits(x) & 0x7fffffffffffffffULL)); }
// a zero of the given sign
FSG_DEV double d_zero(bool neg) { return __longlong_as_double(neg ? (long long)0x8000000000000000ULL : 0LL); }

// |z| < r as hypot(z.x, z.y) < r decides it, without the hypot.  abs_scaled
// takes |z|^2 on z's own power of two: the larger part scaled into [1, 2) on
// its exponent bits, the other alike (dropped below 2^-1022 of it), s =
// a^2 + b^2 in [1, 8) within 2^-51 of the true value.  abs_cmp scales r the
// same way and compares r^2 with s: outside a margin of 256 units in the last
// place (at least 2^-45 of the value, far beyond the roundings of s, of r^2
// and of any hypot within a few units in the last place) the answer is
// hypot's; inside it, and for zero, subnormal, infinite or NaN parts of z or
// r, abs_cmp returns -1 and the caller computes hypot.
struct AbsScaled { double s; int k; bool ok, zero; };
FSG_DEV AbsScaled abs_scaled(double2 z) {
    const unsigned long long MAG = 0x7fffffffffffffffULL, FRAC = 0x000fffffffffffffULL;
    const unsigned long long ux = dbits(z.x) & MAG, uy = dbits(z.y) & MAG;
    const unsigned long long um = ux > uy ? ux : uy, un = ux > uy ? uy : ux;
    const int em = (int)(um >> 52), en = (int)(un >> 52);
    AbsScaled r;
    r.zero = um == 0ULL;
    r.ok = em >= 1 && em <= 2046 && (un == 0ULL || (en >= 1 && en <= 2046));
    r.s = 0.;
    r.k = 0;
    if (r.ok) {
        r.k = em - 1023;
        const double a = __longlong_as_double((long long)((um & FRAC) | (1023ULL << 52)));
        const int eb = en - r.k;
        const double b = (un == 0ULL || eb < 1)
            ? 0. : __longlong_as_double((long long)((un & FRAC) | ((unsigned long long)eb << 52)));
        r.s = a * a + b * b;
    }
    return r;
}
// 1: hypot(z) < r, 0: not, -1: open (compute hypot)
FSG_DEV int abs_cmp(const AbsScaled &a, double r) {
    const unsigned long long FRAC = 0x000fffffffffffffULL;
    const unsigned long long ur = dbits(r);
    const int er = (int)(ur >> 52) & 0x7ff;
    if ((ur << 1) == 0ULL) return 0;                      // hypot < 0: never
    if (a.zero) return d_sq_gt(r, 0.) ? 1 : 0;            // hypot(0) = 0 < r
    if (!a.ok || (ur >> 63) != 0ULL || er < 1 || er > 2046) return -1;
    const int e2 = er - a.k;
    if (e2 < 1) return 0;                                 // r below 2^-1022 |z|
    if (e2 > 2046) return 1;                              // r above 2^1023 |z|
    const double rs = __longlong_as_double((long long)((ur & FRAC) | ((unsigned long long)e2 << 52)));
    const unsigned long long sb = dbits(a.s), rb = dbits(rs * rs);
    if (sb + 256ULL < rb) return 1;
    if (sb > rb + 256ULL) return 0;
    return -1;
}

// ---------------------------------------------------------------------------
// complex128
// ---------------------------------------------------------------------------
FSG_DEV double2 cx(double re, double im) { return make_double2(re, im); }
FSG_DEV double2 cadd(double2 a, double2 b) { return cx(a.x + b.x, a.y + b.y); }
FSG_DEV double2 cmul(double2 a, double2 b) {
    return cx(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// float * complex: the float promoted to complex(s, 0.) first, so the product
// is (s x - 0 y) + (s y + 0 x) i.  For finite s, x, y the products with 0 are
// zeros whose only effect is the sign of a zero result (-0 - +0 = -0,
// -0 + -0 = -0, any other sum of two zeros +0): two multiplies and the sign
// rule give the same bits as the four multiplies and two additions.  Inf or
// NaN operands take the full product, out of line: inlined, the compiler
// evaluates both forms and selects, and the FP64 pipe pays for both.
static __device__ __noinline__ double2 rmul_full(double s, double2 b) { return cmul(cx(s, 0.), b); }
FSG_DEV double2 rmul(double s, double2 b) {
    if (d_nonfinite(s) || d_nonfinite(b.x) || d_nonfinite(b.y)) return rmul_full(s, b);
    double re = s * b.x, im = s * b.y;
    if (d_is0(re)) re = d_zero((dbits(re) >> 63) && !(dbits(b.y) >> 63));
    if (d_is0(im)) im = d_zero((dbits(im) >> 63) && (dbits(b.x) >> 63));
    return cx(re, im);
}
// 2 x, exact, on the bits: one more in the exponent field of a normal x, the
// magnitude shifted up for a zero or subnormal x (a carry into the exponent
// field gives the normal result); x * 2. out of line where 2 x overflows, and
// for inf and NaN
static __device__ __noinline__ double d_twice_full(double x) { return x * 2.; }
FSG_DEV double d_twice(double x) {
    const unsigned long long b = dbits(x), e = b & FSG_D_INF_BITS;
    const unsigned long long sign = b & 0x8000000000000000ULL;
    if (e == 0ULL) return __longlong_as_double((long long)(sign | ((b ^ sign) << 1)));
    if (e < (2046ULL << 52)) return __longlong_as_double((long long)(b + (1ULL << 52)));
    return d_twice_full(x);
}
// rmul(2., b): the same bits, the two products taken by d_twice
FSG_DEV double2 rmul2(double2 b) {
    if (d_nonfinite(b.x) || d_nonfinite(b.y)) return rmul_full(2., b);
    double re = d_twice(b.x), im = d_twice(b.y);
    if (d_is0(re)) re = d_zero((dbits(re) >> 63) && !(dbits(b.y) >> 63));
    if (d_is0(im)) im = d_zero((dbits(im) >> 63) && (dbits(b.x) >> 63));
    return cx(re, im);
}
FSG_DEV double2 caddr(double2 a, double s) { return cx(a.x + s, a.y + 0.); }
// cmul(a, a) without contraction (the translation units built with
// -fmad=false): a.x a.y + a.y a.x adds one rounded product to itself, which
// is twice that product exactly
FSG_DEV double2 csq(double2 a) { return cx(a.x * a.x - a.y * a.y, d_twice(a.x * a.y)); }

// ---------------------------------------------------------------------------
// Xrange complex (reference semantics, numba_xr.py)
// ---------------------------------------------------------------------------
struct xc { double re, im; int e; };
struct xf { double m; int e; };

FSG_DEV xc xc_make(double re, double im, int e) { xc r; r.re = re; r.im = im; r.e = e; return r; }
FSG_DEV xc xc_zero() { return xc_make(0., 0., 0); }

// numba_xr.py _frexp: rewrite the biased exponent to 1023, m in [1, 2)
FSG_DEV double xr_frexp(double m, int &e) {
    unsigned long long b = (unsigned long long)__double_as_longlong(m);
    e = (int)((b >> 52) & 0x7ff) - 0x3ff;
    return __longlong_as_double((long long)((b & 0x8000000000000000ULL) + (0x3ffULL << 52)
                                            + (b & 0xfffffffffffffULL)));
}
FSG_DEV double xr_norm_real(double m, int exp, int &eo) {
    if (d_is0(m)) { eo = 0; return m; }
    int ne; double nm = xr_frexp(m, ne);
    eo = exp + ne; return nm;
}
// numba_xr.py _exp2_shift: add to the biased exponent, clamped at 0
FSG_DEV double xr_exp2_shift(double m, long long shift) {
    unsigned long long b = (unsigned long long)__double_as_longlong(m);
    long long ex = (long long)((b >> 52) & 0x7ff) + shift;
    if (ex < 0) ex = 0;
    return __longlong_as_double((long long)((b & 0x8000000000000000ULL)
                                            + ((unsigned long long)ex << 52)
                                            + (b & 0xfffffffffffffULL)));
}
FSG_DEV bool xr_need_renorm_r(double m) {
    long long d = (long long)(((unsigned long long)__double_as_longlong(m) >> 52) & 0x7ff) - 1023;
    return (d < 0 ? -d : d) > 100;
}
FSG_DEV bool xr_need_renorm_c(double2 m) { return xr_need_renorm_r(m.x) || xr_need_renorm_r(m.y); }

FSG_DEV void xr_coexp_r(double m0, int e0, double m1, int e1, double &o0, double &o1, int &eo) {
    long long d = (long long)e0 - (long long)e1;
    if (d_is0(m0)) { eo = e1; }
    else if (d_is0(m1)) { eo = e0; }
    else if (e1 > e0) { m0 = xr_exp2_shift(m0, d); eo = e1; }
    else if (e0 > e1) { m1 = xr_exp2_shift(m1, -d); eo = e0; }
    else { eo = e0; }
    o0 = m0; o1 = m1;
}
FSG_DEV void xr_coexp_c(double2 m0, int e0, double2 m1, int e1, double2 &o0, double2 &o1, int &eo) {
    long long d = (long long)e0 - (long long)e1;
    if (d_is0(m0.x) && d_is0(m0.y)) { eo = e1; }
    else if (d_is0(m1.x) && d_is0(m1.y)) { eo = e0; }
    else if (e1 > e0) { m0 = cx(xr_exp2_shift(m0.x, d), xr_exp2_shift(m0.y, d)); eo = e1; }
    else if (e0 > e1) { m1 = cx(xr_exp2_shift(m1.x, -d), xr_exp2_shift(m1.y, -d)); eo = e0; }
    else { eo = e0; }
    o0 = m0; o1 = m1;
}
FSG_DEV xc xr_normalize_c(double2 m, int exp) {
    int ere, eim;
    double nre = xr_norm_real(m.x, exp, ere), nim = xr_norm_real(m.y, exp, eim);
    double cr, ci; int ce;
    xr_coexp_r(nre, ere, nim, eim, cr, ci, ce);
    return xc_make(cr, ci, ce);
}
FSG_DEV xc xr_from(double2 z) { return xr_normalize_c(z, 0); }
FSG_DEV double2 xm(xc a) { return cx(a.re, a.im); }
FSG_DEV xc xr_add(xc a, xc b) {
    double2 o0, o1; int e;
    xr_coexp_c(xm(a), a.e, xm(b), b.e, o0, o1, e);
    double2 s = cadd(o0, o1);
    return xc_make(s.x, s.y, e);
}
FSG_DEV xc xr_add_s(xc a, double2 z) {
    xc b = xr_need_renorm_c(z) ? xr_normalize_c(z, 0) : xc_make(z.x, z.y, 0);
    return xr_add(a, b);
}
FSG_DEV xc xr_mul(xc a, xc b) {
    double2 m = cmul(xm(a), xm(b));
    int e = (int)((unsigned)a.e + (unsigned)b.e);
    if (xr_need_renorm_c(m)) return xr_normalize_c(m, e);
    return xc_make(m.x, m.y, e);
}
FSG_DEV xc xr_mul_s(double2 s, xc b) {
    double2 m = cmul(s, xm(b));
    if (xr_need_renorm_c(m)) return xr_normalize_c(m, b.e);
    return xc_make(m.x, m.y, b.e);
}
FSG_DEV xc xr_mul_r(double s, xc b) {
    double2 m = rmul(s, xm(b));
    if (xr_need_renorm_c(m)) return xr_normalize_c(m, b.e);
    return xc_make(m.x, m.y, b.e);
}
// xr_mul_r(2., b)
FSG_DEV xc xr_mul_2(xc b) {
    double2 m = rmul2(xm(b));
    if (xr_need_renorm_c(m)) return xr_normalize_c(m, b.e);
    return xc_make(m.x, m.y, b.e);
}
FSG_DEV xc xf_mul_c(xf a, double2 z) {
    double2 m = rmul(a.m, z);
    if (xr_need_renorm_c(m)) return xr_normalize_c(m, a.e);
    return xc_make(m.x, m.y, a.e);
}
FSG_DEV xf xr_abs2(xc a) {
    xf r; r.m = a.re * a.re + a.im * a.im; r.e = (int)((unsigned)a.e + (unsigned)a.e); return r;
}
FSG_DEV bool xf_lt_s(xf a, double x) {
    double o0, o1; int e; xr_coexp_r(a.m, a.e, x, 0, o0, o1, e); return o0 < o1;
}
// xf_lt_s for a the Xrange sum of squares and x a square: the co-exponent
// mantissas are >= +0 and finite there and compare on their bits; any other
// pair (a NaN or infinite mantissa shifted into a finite one) takes the
// double compare, out of line
static __device__ __noinline__ bool d_lt_full(double a, double b) { return a < b; }
FSG_DEV bool xf_sq_lt_s(xf a, double x) {
    double o0, o1; int e; xr_coexp_r(a.m, a.e, x, 0, o0, o1, e);
    if (dbits(o0) < FSG_D_INF_BITS && dbits(o1) < FSG_D_INF_BITS)
        return (long long)dbits(o0) < (long long)dbits(o1);
    return d_lt_full(o0, o1);
}
FSG_DEV bool xf_le(xf a, xf b) {
    double o0, o1; int e; xr_coexp_r(a.m, a.e, b.m, b.e, o0, o1, e); return o0 <= o1;
}
// real Xrange records (numba_xr.py on float64 Xrange): add / sub through the
// co-exponent, lazy renormalisation of products, float * Xrange
FSG_DEV xf xf_make(double m, int e) { xf r; r.m = m; r.e = e; return r; }
FSG_DEV xf xr_from_r(double x) { int e; double m = xr_norm_real(x, 0, e); return xf_make(m, e); }
FSG_DEV xf xf_add(xf a, xf b) {
    double o0, o1; int e; xr_coexp_r(a.m, a.e, b.m, b.e, o0, o1, e); return xf_make(o0 + o1, e);
}
FSG_DEV xf xf_sub(xf a, xf b) {
    double o0, o1; int e; xr_coexp_r(a.m, a.e, b.m, b.e, o0, o1, e); return xf_make(o0 - o1, e);
}
// Xrange + float: the float as a record (normalised only out of +-2^100)
FSG_DEV xf xf_add_s(xf a, double x) {
    xf b = xr_need_renorm_r(x) ? xr_from_r(x) : xf_make(x, 0);
    return xf_add(a, b);
}
FSG_DEV xf xf_mul(xf a, xf b) {
    const double m = a.m * b.m;
    const int e = (int)((unsigned)a.e + (unsigned)b.e);
    if (xr_need_renorm_r(m)) { int eo; double nm = xr_norm_real(m, e, eo); return xf_make(nm, eo); }
    return xf_make(m, e);
}
FSG_DEV xf xf_mul_s(double s, xf b) {
    const double m = s * b.m;
    if (xr_need_renorm_r(m)) { int eo; double nm = xr_norm_real(m, b.e, eo); return xf_make(nm, eo); }
    return xf_make(m, b.e);
}
FSG_DEV bool xf_ge_s(xf a, double x) {
    double o0, o1; int e; xr_coexp_r(a.m, a.e, x, 0, o0, o1, e); return o0 >= o1;
}
FSG_DEV bool xf_le_s(xf a, double x) {
    double o0, o1; int e; xr_coexp_r(a.m, a.e, x, 0, o0, o1, e); return o0 <= o1;
}

// ldexp(1., e) for any int e (exact power of two, 0 below 2^-1074, inf above)
FSG_DEV double pow2d(int e) {
    if (e > 1023) return __longlong_as_double(0x7ff0000000000000LL);
    if (e >= -1022) return __longlong_as_double((long long)(e + 1023) << 52);
    if (e >= -1074) return __longlong_as_double(1LL << (e + 1074));
    return 0.;
}
// rmul(pow2d(k), b): where both parts are normal and stay normal the
// product is exact and only moves the exponent fields; anything else (a zero
// or subnormal part, a rounded or overflowing result, an inf or NaN, k out of
// the normal powers) takes the full product, out of line
FSG_DEV double2 rmul_p2(int k, double2 b) {
    const unsigned long long bx = dbits(b.x), by = dbits(b.y);
    const int ex = (int)((bx >> 52) & 0x7ff), ey = (int)((by >> 52) & 0x7ff);
    if (k >= -1022 && k <= 1023 && ex >= 1 && ex <= 2046 && ey >= 1 && ey <= 2046
        && ex + k >= 1 && ex + k <= 2046 && ey + k >= 1 && ey + k <= 2046) {
        const unsigned long long sh = (unsigned long long)(long long)k << 52;
        return cx(__longlong_as_double((long long)(bx + sh)), __longlong_as_double((long long)(by + sh)));
    }
    return rmul_full(pow2d(k), b);
}
FSG_DEV double2 xr_to_std(xc a) {
    int ere, eim;
    double nre = xr_norm_real(a.re, a.e, ere), nim = xr_norm_real(a.im, a.e, eim);
    double cr, ci; int ce;
    xr_coexp_r(nre, ere, nim, eim, cr, ci, ce);
    return rmul_p2(ce, cx(cr, ci));
}
// to_standard of a real Xrange record
FSG_DEV double ldexp_d(double m, int e);
FSG_DEV double xf_to_std(xf a) { return d_is0(a.m) ? 0. * a.m : ldexp_d(a.m, a.e); }

// ldexp(m, e) with one rounding (m is in [1, 2) or a small normal number)
FSG_DEV double ldexp_d(double m, int e) {
    if (e >= -1022 && e <= 1023) return m * pow2d(e);
    if (e > 1023) return (m * pow2d(e - 1023)) * pow2d(1023);
    // subnormal results: scale into range first so only the last product rounds
    if (e < -2200) return 0. * m;
    return (m * pow2d(e + 1000)) * pow2d(-1000);
}

// ---------------------------------------------------------------------------
// fe: FP32 mantissa + int32 exponent (the fast form)
// ---------------------------------------------------------------------------
#define FE_ZERO_E (-(1 << 29))
struct fe { float x, y; int e; };

FSG_DEV fe fe_make(float x, float y, int e) { fe r; r.x = x; r.y = y; r.e = e; return r; }
FSG_DEV fe fe_zero() { return fe_make(0.f, 0.f, FE_ZERO_E); }
// 2^k as a float for k <= 0 (0 below 2^-126)
FSG_DEV float exp2neg(int k) {
    k = max(k, -127);
    return __int_as_float((k + 127) << 23);
}
// exponent of max(|x|, |y|) (biased; 0 for zero / subnormal)
FSG_DEV int fe_bexp(float x, float y) {
    float a = fmaxf(fabsf(x), fabsf(y));
    return (__float_as_int(a) >> 23) & 0xff;
}
FSG_DEV fe fe_norm(fe a) {
    int b = fe_bexp(a.x, a.y);
    if (b == 0) return fe_zero();
    float s = __int_as_float((254 - b) << 23);   // 2^(127 - b)
    return fe_make(a.x * s, a.y * s, a.e + (b - 127));
}
FSG_DEV fe fe_add(fe a, fe b) {
    int d = a.e - b.e;
    if (d >= 0) {
        float s = exp2neg(-d);
        return fe_make(fmaf(b.x, s, a.x), fmaf(b.y, s, a.y), a.e);
    }
    float s = exp2neg(d);
    return fe_make(fmaf(a.x, s, b.x), fmaf(a.y, s, b.y), b.e);
}
FSG_DEV fe fe_mul(fe a, fe b) {
    return fe_make(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x, a.e + b.e);
}
FSG_DEV fe fe_scale2(fe a, int k) { return fe_make(a.x, a.y, a.e + k); }
// from a double complex (exact exponent, mantissa rounded to float)
FSG_DEV fe fe_from_d(double2 z) {
    double a = fmax(fabs(z.x), fabs(z.y));
    if (a == 0.) return fe_zero();
    int e;
    frexp(a, &e);              // a = f * 2^e, f in [0.5, 1)
    e -= 1;
    double s = pow2d(-e);
    if (e < -1022) s = pow2d(-e - 100) * pow2d(100);
    return fe_make((float)(z.x * s), (float)(z.y * s), e);
}
FSG_DEV fe fe_from_xc(xc v) {
    fe r = fe_from_d(xm(v));
    if (r.e != FE_ZERO_E) r.e += v.e;
    return r;
}
// value as a double complex (underflows to 0 like to_standard)
FSG_DEV double2 fe_to_d(fe a) {
    if (a.e == FE_ZERO_E || (a.x == 0.f && a.y == 0.f)) return cx(0., 0.);
    return cx(ldexp_d((double)a.x, a.e), ldexp_d((double)a.y, a.e));
}
// value as a float complex (flushes below 2^-126)
FSG_DEV float2 fe_to_f(fe a) {
    if (a.e > 0) {
        float s = __int_as_float((min(a.e, 127) + 127) << 23);
        return make_float2(a.x * s, a.y * s);
    }
    float s = exp2neg(a.e);
    return make_float2(a.x * s, a.y * s);
}
// |a|^2 < t (t a positive double threshold, a normalised or not)
FSG_DEV bool fe_abs2_lt(fe a, double t) {
    float m2 = a.x * a.x + a.y * a.y;
    if (m2 == 0.f) return 0. < t;
    // compare log2 magnitudes first, exact compare only when close
    double lhs = (double)m2 * 1.0;
    int e2 = 2 * a.e;
    if (e2 < -2000) return true;
    if (e2 > 2000) return false;
    return ldexp_d(lhs, e2) < t;
}
