// fsg_bs.cuh -- the Burning Ship family perturbation loop, templated on the
// real type of the deltas:
//   * double -- the reference's standard branch (instantiated in
//     fsg_perturb.cu, compiled without FMA contraction: one rounding per
//     operation in the order of the reference source);
//   * fr -- FP32 mantissa + int32 exponent (instantiated in fsg_perturb_bs32.cu):
//     no underflow at any depth and FP32-pipe arithmetic instead of GB300's
//     slow FP64 pipe; results within FP32 rounding of the double form.
// perturbation.py:1406-1811 (numba_cycles_perturb_BS, numba_iterate_BS,
// apply_BLA_BS, apply_BLA_deriv_BS) with the closures of
// models/burning_ship.py:19-60 (diffabs and its derivatives), 535-619
// (_p_iter_zn) and 622-859 (_p_iter_hessian).
#pragma once
#include "fsg_internal.cuh"

// Whether ref_BLA_get can admit any dz at start index w >> 3: radii never
// grow with the stage (combine_BLA, combine_BLA_BS: r <= r of the first child,
// perturbation.py:2023-2024, 2104-2105) and 0 < r is strict, so a stage-3
// radius of 0 -- at the orbit's critical point, where A = 2 Z = 0 -- rules
// every stage out, and |dz| need not be computed for the search.
__device__ __forceinline__ bool bla_possible(const RefDev &R, int w) {
    const int i3 = 2 * (w >> FSG_STG_COMPRESSED);
    return i3 < R.bla_len && d_sq_gt(__ldg(&R.rbla[i3]), 0.);
}

// perturbation.py:2116-2170 ref_BLA_get on dz itself: returns the step (0 if
// none) and the table index of the accepted entry.  The reference tests
// abs(dz) < r, a hypot, against each candidate radius; abs_cmp (fsg_num.cuh)
// gives the same answers from |dz|^2 on dz's own scale, and hypot(dz) is
// computed (out of line) only where that leaves one open.
// hypot(z) < r, with hypot(z) computed once per lookup (h < 0: not yet);
// out of line, compare included (inlined, the FP64 form ran 1.4 % slower)
static __device__ __noinline__ int bla_hypot_lt(double2 z, double r, double &h) {
    if (h < 0.) h = hypot(z.x, z.y);
    return h < r;
}
__device__ __forceinline__ int bla_lookup_z(const RefDev &R, double2 z, int w, int &ib) {
    const AbsScaled a = abs_scaled(z);
    double h = -1.;              // hypot(z), once needed
    int it = w >> FSG_STG_COMPRESSED;
    int stages = FSG_STG_COMPRESSED;
    for (int st = FSG_STG_COMPRESSED; st < R.stages; st++) {
        stages = st;
        if (it & 1) break;
        it >>= 1;
    }
    const int invalid_step = R.first_invalid - w;
    for (int stg = stages; stg >= FSG_STG_COMPRESSED; stg--) {
        const int step = 1 << stg;
        if (step >= invalid_step) continue;
        const int idx = 2 * (w >> FSG_STG_COMPRESSED) + ((1 << (stg - FSG_STG_COMPRESSED)) - 1);
        const double r = __ldg(&R.rbla[idx]);
        int lt = abs_cmp(a, r);
        if (lt < 0) lt = bla_hypot_lt(z, r, h);
        if (lt) { ib = idx; return step; }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// fr: a real m * 2^e with an FP32 mantissa, |m| in [1, 2), or m = 0 (e =
// FR_ZERO_E).  Every operation rounds the mantissa once (FP32) and keeps the
// exponent exact.
// ---------------------------------------------------------------------------
struct fr { float m; int e; };
#define FR_ZERO_E (-(1 << 29))

FSG_DEV fr fr_zero() { fr r; r.m = 0.f; r.e = FR_ZERO_E; return r; }
// normalise m * 2^e for finite m (0 and subnormal mantissas give 0): the
// biased exponent of m moves to e and m's own is set to 0 (bit operations)
FSG_DEV fr fr_norm(float m, int e) {
    const int bits = __float_as_int(m);
    const int b = (bits >> 23) & 0xff;
    fr r;
    r.m = __int_as_float((bits & 0x807fffff) | 0x3f800000);
    r.e = e + (b - 127);
    if (b == 0) r = fr_zero();
    return r;
}
FSG_DEV fr fr_from_d(double x) {
    const long long bits = __double_as_longlong(x);
    const int be = (int)((bits >> 52) & 0x7ff);
    if (be == 0) {
        if (x == 0.) return fr_zero();
        int e; double f = frexp(x, &e);            // subnormal double
        return fr_norm((float)(2. * f), e - 1);
    }
    // the mantissa in [1, 2) with the sign of x; its FP32 rounding may give 2
    const double m = __longlong_as_double((bits & 0x800fffffffffffffLL) | 0x3ff0000000000000LL);
    return fr_norm((float)m, be - 1023);
}
FSG_DEV double fr_to_d(fr a) { return a.m == 0.f ? 0. : ldexp_d((double)a.m, a.e); }
// 2^-d for d >= 0 (0 from d = 127 on)
FSG_DEV float fr_p2n(int d) { return __int_as_float((127 - min(d, 127)) << 23); }

// Branch-free: the operand of larger exponent (a zero has the smallest) takes
// the other scaled by 2^-d in one FMA.  From d = 61 on the scaled term is
// below half an ulp and the sum is the larger operand itself.
FSG_DEV fr operator+(fr a, fr b) {
    const bool ge = a.e >= b.e;
    const float mb = ge ? a.m : b.m, ms = ge ? b.m : a.m;
    const int eb = ge ? a.e : b.e, d = ge ? a.e - b.e : b.e - a.e;
    return fr_norm(fmaf(ms, fr_p2n(d), mb), eb);
}
FSG_DEV fr operator-(fr a) { a.m = -a.m; return a; }
FSG_DEV fr operator-(fr a, fr b) { return a + (-b); }
FSG_DEV fr operator*(fr a, fr b) {
    fr r; r.m = a.m * b.m; r.e = a.e + b.e;              // |m| in [1, 4) or 0
    if (fabsf(r.m) >= 2.f) { r.m *= 0.5f; r.e += 1; }
    if (r.m == 0.f) r = fr_zero();
    return r;
}
// product by a literal constant (the closures' 2. * x): FP32 only, exact for
// the powers of two the loop uses
FSG_DEV fr operator*(double s, fr b) {
    if (s == 2. || s == -2.) {
        if (b.m != 0.f) b.e += 1;
        if (s < 0.) b.m = -b.m;
        return b;
    }
    return fr_norm((float)s * b.m, b.e);
}
FSG_DEV fr &operator+=(fr &a, fr b) { a = a + b; return a; }

// xf: the reference's float64 Xrange record (numba_xr.py), the real type of
// the Xrange branch.  Constants are the unnormalised records {x, 0}, so that a
// constant times a record rounds as the reference's float * Xrange.
FSG_DEV xf operator+(xf a, xf b) { return xf_add(a, b); }
FSG_DEV xf operator-(xf a) { a.m = -a.m; return a; }
FSG_DEV xf operator-(xf a, xf b) { return xf_sub(a, b); }
FSG_DEV xf operator*(xf a, xf b) { return xf_mul(a, b); }
FSG_DEV xf operator*(double s, xf b) { return xf_mul_s(s, b); }
FSG_DEV xf &operator+=(xf &a, xf b) { a = a + b; return a; }

// the operations the loop needs, for every real type
FSG_DEV double to_d(double x) { return x; }
FSG_DEV double to_d(fr x) { return fr_to_d(x); }
FSG_DEV double to_d(xf x) { return xf_to_std(x); }
template <class T> FSG_DEV T from_d(double x);
template <> FSG_DEV double from_d<double>(double x) { return x; }
template <> FSG_DEV fr from_d<fr>(double x) { return fr_from_d(x); }
template <> FSG_DEV xf from_d<xf>(double x) { return xr_from_r(x); }      // to_Xrange_scalar
// a literal constant (0, +-1, +-2) of the loop's real type, without FP64
template <class T> FSG_DEV T cst(float x);
template <> FSG_DEV double cst<double>(float x) { return (double)x; }
template <> FSG_DEV fr cst<fr>(float x) { return fr_norm(x, 0); }
template <> FSG_DEV xf cst<xf>(float x) { return xf_make((double)x, 0); }
// m * 2^e from a mantissa and an exponent (the Xrange form of c)
template <class T> FSG_DEV T from_me(double m, int e);
template <> FSG_DEV double from_me<double>(double m, int e) { return ldexp_d(m, e); }
template <> FSG_DEV fr from_me<fr>(double m, int e) {
    fr r = fr_from_d(m);
    if (r.m != 0.f) r.e += e;
    return r;
}
template <> FSG_DEV xf from_me<xf>(double m, int e) { return xf_make(m, e); }
FSG_DEV bool ge0(double x) { return d_ge0(x); }
FSG_DEV bool ge0(fr x) { return x.m >= 0.f; }
FSG_DEV bool ge0(xf x) { return xf_ge_s(x, 0.); }
FSG_DEV bool le0(double x) { return d_le0(x); }
FSG_DEV bool le0(fr x) { return x.m <= 0.f; }
FSG_DEV bool le0(xf x) { return xf_le_s(x, 0.); }
FSG_DEV double absT(double x) { return d_abs(x); }
FSG_DEV fr absT(fr x) { x.m = fabsf(x.m); return x; }
FSG_DEV xf absT(xf x) { x.m = fabs(x.m); return x; }
// sgn with 0 mapped to +1 (burning_ship.py:12-17)
FSG_DEV double sgnT(double x) { return d_lt0(x) ? -1. : 1.; }
FSG_DEV fr sgnT(fr x) { fr r; r.m = x.m < 0.f ? -1.f : 1.f; r.e = 0; return r; }
FSG_DEV xf sgnT(xf x) { return xf_make(xf_lt_s(x, 0.) ? -1. : 1., 0); }
// |a| <= |b|
FSG_DEV bool abs_le(double a, double b) { return d_abs_le(a, b); }
FSG_DEV bool abs_le(xf a, xf b) { a.m = fabs(a.m); b.m = fabs(b.m); return xf_le(a, b); }
FSG_DEV bool abs_le(fr a, fr b) {
    if (a.m == 0.f) return true;
    if (b.m == 0.f) return false;
    return a.e != b.e ? a.e < b.e : fabsf(a.m) <= fabsf(b.m);
}

// |(x, y)| as s * 2^e, s in [1, 2 sqrt 2], in FP32 (z = false: (0, 0))
struct fr_mod { float s; int e; bool z; };
FSG_DEV fr_mod fr_modulus2(fr x, fr y, bool squared) {
    const int e = max(x.e, y.e);
    const float mx = x.m * fr_p2n(e - x.e), my = y.m * fr_p2n(e - y.e);
    const float q = fmaf(mx, mx, my * my);
    fr_mod r; r.s = squared ? q : sqrtf(q); r.e = squared ? 2 * e : e;
    r.z = x.m == 0.f && y.m == 0.f;
    return r;
}
// v * 2^d as a float, d in [-3, 0]
FSG_DEV float fr_scale_small(float v, int d) { return v * __int_as_float((127 + d) << 23); }

// The double-precision forms of the two comparisons below, for the rare
// near-ties: out of line so that the compiler does not evaluate them ahead
// of the branch on every call.
static __device__ __noinline__ bool fr_escaped_exact(fr X, fr Y, double M2) {
    const double Xd = fr_to_d(X), Yd = fr_to_d(Y);
    return Xd * Xd + Yd * Yd > M2;
}
static __device__ __noinline__ bool fr_below_exact(fr xn, fr yn, double r) {
    return hypot(fr_to_d(xn), fr_to_d(yn)) < r;
}

// The escape test |z|^2 > M2 of the loop (perturbation.py:1636-1639) with z in
// fr: decided in FP32 unless within 2^-18 of the bound, where the double form
// of the reference decides (so that the outcome is the FP64 one of the same
// fr values).
FSG_DEV bool fr_escaped(fr X, fr Y, fr M2f, double M2) {
    const fr_mod q = fr_modulus2(X, Y, true);           // s in [1, 8)
    if (q.z) return false;                              // M2 > 0
    const int d = q.e - M2f.e;
    if (d >= 1) return true;                            // >= 2 > M2 mantissa
    if (d <= -4) return false;                          // < 0.5
    const float t = fr_scale_small(q.s, d);
    if (fabsf(t - M2f.m) > M2f.m * 0x1p-18f) return t > M2f.m;
    return fr_escaped_exact(X, Y, M2);
}

// |dz| < r for a BLA radius r (double r, its fr copy rm * 2^re), the
// comparison of ref_BLA_get (perturbation.py:2116-2170) in FP32 unless within
// 2^-18 of r, where the double form decides.
FSG_DEV bool fr_below(const fr_mod &a, fr xn, fr yn, float rm, int re, double r) {
    if (rm == 0.f) return false;                        // r = 0
    if (a.z) return true;                               // 0 < r
    const int d = a.e - re;
    if (d >= 1) return false;                           // >= 2 > rm
    if (d <= -2) return true;                           // < 0.71 < rm
    const float t = fr_scale_small(a.s, d);
    if (fabsf(t - rm) > rm * 0x1p-18f) return t < rm;
    return fr_below_exact(xn, yn, r);
}

// ref_BLA_get in the loop's real type: double |dz| against the double radii,
// or the FP32 modulus against their fr copies
template <class T> struct BLAGet;
template <> struct BLAGet<double> {
    static FSG_DEV int get(const RefDev &R, double xn, double yn, int w, int &ib) {
        return bla_possible(R, w) ? bla_lookup_z(R, cx(xn, yn), w, ib) : 0;
    }
};
template <> struct BLAGet<fr> {
    static FSG_DEV int get(const RefDev &R, fr xn, fr yn, int w, int &ib) {
        if (!bla_possible(R, w)) return 0;
        int it = w >> FSG_STG_COMPRESSED;
        int stages = FSG_STG_COMPRESSED;
        for (int s = FSG_STG_COMPRESSED; s < R.stages; s++) {
            stages = s;
            if (it & 1) break;
            it >>= 1;
        }
        const fr_mod a = fr_modulus2(xn, yn, false);
        const int invalid_step = R.first_invalid - w;
        for (int stg = stages; stg >= FSG_STG_COMPRESSED; stg--) {
            const int step = 1 << stg;
            if (step >= invalid_step) continue;
            const int idx = 2 * (w >> FSG_STG_COMPRESSED) + ((1 << (stg - FSG_STG_COMPRESSED)) - 1);
            const int2 rf = __ldg(&R.bs_rf[idx]);
            if (fr_below(a, xn, yn, __int_as_float(rf.x), rf.y, __ldg(&R.rbla[idx]))) {
                ib = idx;
                return step;
            }
        }
        return 0;
    }
};

// v * 2^k (k = 0: v)
FSG_DEV double scale2(double v, int k) { return k == 0 ? v : ldexp_d(v, k); }
FSG_DEV fr scale2(fr v, int k) { if (v.m != 0.f) v.e += k; return v; }
FSG_DEV xf scale2(xf v, int k) { v.e += k; return v; }

// ref_BLA_get on the Xrange branch: the standard values of the deltas (0
// below the double range, perturbation.py:1520-1527)
template <> struct BLAGet<xf> {
    static FSG_DEV int get(const RefDev &R, xf xn, xf yn, int w, int &ib) {
        return bla_possible(R, w) ? bla_lookup_z(R, cx(xf_to_std(xn), xf_to_std(yn)), w, ib)
                                  : 0;
    }
};

// Reads of the reference's tables in the loop's real type: the double
// tables themselves, or their fr copies (orbit values from the Xrange side
// table where the orbit holds one)
template <class T> struct BSRef;
template <> struct BSRef<double> {
    static FSG_DEV void orbit(const RefDev &R, int w, double &X, double &Y) {
        double2 z = __ldg(&R.Zn[w]); X = z.x; Y = z.y;
    }
    static FSG_DEV void hess(const RefDev &R, int w, double &a, double &b, double &c, double &d) {
        a = __ldg(&R.dXa[w]); b = __ldg(&R.dXb[w]); c = __ldg(&R.dYa[w]); d = __ldg(&R.dYb[w]);
    }
    static FSG_DEV void bla(const RefDev &R, int ib, double M[8]) {
        const double *p = R.Mbla_bs + 8 * ib;
        for (int k = 0; k < 8; k++) M[k] = __ldg(p + k);
    }
};
template <> struct BSRef<fr> {
    static FSG_DEV fr lo(int4 v) { fr r; r.m = __int_as_float(v.x); r.e = v.y; return r; }
    static FSG_DEV fr hi(int4 v) { fr r; r.m = __int_as_float(v.z); r.e = v.w; return r; }
    static FSG_DEV void orbit(const RefDev &R, int w, fr &X, fr &Y) {
        int4 v = __ldg(&R.bs_Zf[w]); X = lo(v); Y = hi(v);
    }
    static FSG_DEV void hess(const RefDev &R, int w, fr &a, fr &b, fr &c, fr &d) {
        int4 p = __ldg(&R.bs_hf[2 * w]), q = __ldg(&R.bs_hf[2 * w + 1]);
        a = lo(p); b = hi(p); c = lo(q); d = hi(q);
    }
    static FSG_DEV void bla(const RefDev &R, int ib, fr M[8]) {
        for (int k = 0; k < 4; k++) {
            int4 v = __ldg(&R.bs_blaf[4 * ib + k]);
            M[2 * k] = lo(v); M[2 * k + 1] = hi(v);
        }
    }
};

// The Xrange branch: ensure_xr_BS (perturbation.py:2182-2193) -- the side
// table's value where the orbit holds one, else the standard value as a
// record; the Xrange Jacobian paths; the BLA coefficients as float64 (the
// reference multiplies them float * Xrange: unnormalised records {M, 0})
template <> struct BSRef<xf> {
    static FSG_DEV bool table(const RefDev &R, int w, xf &X, xf &Y) {
        const int s = (R.n_xr > 0 && w < R.len) ? __ldg(&R.xr_slot[w]) : -1;
        if (s < 0) return false;
        const double *m = (const double *)R.xr_m;
        X = xf_make(__ldg(&m[s]), __ldg(&R.xr_e[s]));
        Y = xf_make(__ldg(&m[R.n_xr + s]), __ldg(&R.xr_e[R.n_xr + s]));
        return true;
    }
    static FSG_DEV void orbit(const RefDev &R, int w, xf &X, xf &Y) {
        if (!table(R, w, X, Y)) {
            const double2 z = __ldg(&R.Zn[w]);
            X = xr_from_r(z.x); Y = xr_from_r(z.y);
        }
    }
    static FSG_DEV void hess(const RefDev &R, int w, xf &a, xf &b, xf &c, xf &d) {
        const int L = R.len + 1;
        a = xf_make(__ldg(&R.bs_xpm[w]), __ldg(&R.bs_xpe[w]));
        b = xf_make(__ldg(&R.bs_xpm[L + w]), __ldg(&R.bs_xpe[L + w]));
        c = xf_make(__ldg(&R.bs_xpm[2 * L + w]), __ldg(&R.bs_xpe[2 * L + w]));
        d = xf_make(__ldg(&R.bs_xpm[3 * L + w]), __ldg(&R.bs_xpe[3 * L + w]));
    }
    static FSG_DEV void bla(const RefDev &R, int ib, xf M[8]) {
        const double *p = R.Mbla_bs + 8 * ib;
        for (int k = 0; k < 8; k++) M[k] = xf_make(__ldg(p + k), 0);
    }
};

// burning_ship.py:19-60 diffabs(X, x) = |X + x| - |X| and its derivatives
// 2. * x and 1. * x of the closures in their real type: for a double, the
// doubling on the exponent bits and x itself (a NaN or inf takes the
// product, out of line) -- the same bits with no FP64 instruction
FSG_DEV double twice_t(double x) { return d_twice(x); }
FSG_DEV fr twice_t(fr x) { return 2. * x; }
FSG_DEV xf twice_t(xf x) { return 2. * x; }
static __device__ __noinline__ double d_one_full(double x) { return 1. * x; }
FSG_DEV double one_t(double x) { return d_nonfinite(x) ? d_one_full(x) : x; }
FSG_DEV fr one_t(fr x) { return 1. * x; }
FSG_DEV xf one_t(xf x) { return 1. * x; }
template <class T> FSG_DEV T diffabs(T X, T x) {
    if (ge0(X)) { if (ge0(X + x)) return one_t(x); else return -(twice_t(X) + x); }
    else { if (le0(X + x)) return -x; else return (twice_t(X) + x); }
}
template <class T> FSG_DEV T ddiffabsdX(T X, T x) {
    if (ge0(X)) { if (ge0(X + x)) return cst<T>(0.f); else return cst<T>(-2.f); }
    else { if (le0(X + x)) return cst<T>(0.f); else return cst<T>(2.f); }
}
template <class T> FSG_DEV T ddiffabsdx(T X, T x) {
    if (ge0(X)) { if (ge0(X + x)) return cst<T>(1.f); else return cst<T>(-1.f); }
    else { if (le0(X + x)) return cst<T>(-1.f); else return cst<T>(1.f); }
}

// burning_ship.py:535-619 _p_iter_zn
template <class T>
FSG_DEV void bs_zn(int flavor, T &xn, T &yn, T X, T Y, T a, T b) {
    T nx, ny;
    if (flavor == 1) {
        T ref_xyn = X * Y;
        nx = xn * (xn + twice_t(X)) - yn * (yn + twice_t(Y)) + a;
        ny = twice_t(diffabs(ref_xyn, xn * yn + xn * Y + yn * X)) - b;
    } else if (flavor == 2) {
        nx = xn * (xn + twice_t(X)) - yn * (yn + twice_t(Y)) + a;
        ny = twice_t(X * diffabs(Y, yn) + xn * absT(Y + yn)) - b;
    } else if (flavor == 3) {
        nx = xn * (xn + twice_t(X)) - Y * diffabs(Y, yn) - yn * absT(Y + yn) + a;
        ny = twice_t(X * yn + Y * xn + xn * yn) - b;
    } else if (flavor == 4) {
        T q = X * X - Y * Y;
        nx = diffabs(q, xn * (xn + twice_t(X)) - yn * (yn + twice_t(Y))) + a;
        ny = twice_t(X * yn + Y * xn + xn * yn) - b;
    } else {
        T ref_xyn = X * Y, q = X * X - Y * Y;
        nx = diffabs(q, xn * (xn + twice_t(X)) - yn * (yn + twice_t(Y))) + a;
        ny = twice_t(diffabs(ref_xyn, xn * yn + xn * Y + yn * X)) - b;
    }
    xn = nx; yn = ny;
}

// burning_ship.py:622-859 _p_iter_hessian, h = (dxnda, dxndb, dynda, dyndb)
template <class T>
FSG_DEV void bs_hess(int flavor, T h[4], T xn, T yn, T X, T Y, T Xa, T Xb, T Ya, T Yb) {
    T xa = h[0], xb = h[1], ya = h[2], yb = h[3];
    T nxa, nxb, nya, nyb;
    if (flavor == 1 || flavor == 5) {
        T opX = X * Y;
        T dXa = Xa * Y + X * Ya, dXb = Xb * Y + X * Yb;
        T opx = xn * yn + xn * Y + yn * X;
        T dxa = xa * yn + xn * ya + xa * Y + xn * Ya + ya * X + yn * Xa;
        T dxb = xb * yn + xn * yb + xb * Y + xn * Yb + yb * X + yn * Xb;
        T dX = ddiffabsdX(opX, opx), dx = ddiffabsdx(opX, opx);
        nya = twice_t(dX * dXa + dx * dxa);
        nyb = twice_t(dX * dXb + dx * dxb);
        if (flavor == 1) {
            nxa = twice_t((X + xn) * xa + Xa * xn) - twice_t((Y + yn) * ya + Ya * yn);
            nxb = twice_t((X + xn) * xb + Xb * xn) - twice_t((Y + yn) * yb + Yb * yn);
        } else {
            T opX2 = X * X - Y * Y;
            T dXa2 = twice_t(X * Xa - Y * Ya), dXb2 = twice_t(X * Xb - Y * Yb);
            T opx2 = xn * (xn + twice_t(X)) - yn * (yn + twice_t(Y));
            T dxa2 = xa * (xn + twice_t(X)) + xn * (xa + twice_t(Xa)) - ya * (yn + twice_t(Y)) - yn * (ya + twice_t(Ya));
            T dxb2 = xb * (xn + twice_t(X)) + xn * (xb + twice_t(Xb)) - yb * (yn + twice_t(Y)) - yn * (yb + twice_t(Yb));
            T dX2 = ddiffabsdX(opX2, opx2), dx2 = ddiffabsdx(opX2, opx2);
            nxa = dX2 * dXa2 + dx2 * dxa2;
            nxb = dX2 * dXb2 + dx2 * dxb2;
        }
    } else if (flavor == 2) {
        T da = diffabs(Y, yn), dX = ddiffabsdX(Y, yn), dx = ddiffabsdx(Y, yn);
        T Yy = Y + yn, ab = absT(Yy), sg = sgnT(Yy);
        nxa = twice_t(((X + xn) * xa + Xa * xn) - ((Y + yn) * ya + Ya * yn));
        nxb = twice_t(((X + xn) * xb + Xb * xn) - ((Y + yn) * yb + Yb * yn));
        nya = twice_t(Xa * da + X * (dX * Ya + dx * ya) + xa * ab + xn * sg * (Ya + ya));
        nyb = twice_t(Xb * da + X * (dX * Yb + dx * yb) + xb * ab + xn * sg * (Yb + yb));
    } else if (flavor == 3) {
        T da = diffabs(Y, yn), dX = ddiffabsdX(Y, yn), dx = ddiffabsdx(Y, yn);
        T Yy = Y + yn, ab = absT(Yy), sg = sgnT(Yy);
        nxa = xa * (xn + twice_t(X)) + xn * (xa + twice_t(Xa)) - Ya * da - Y * (Ya * dX + ya * dx)
              - ya * ab - yn * sg * (Ya + ya);
        nxb = xb * (xn + twice_t(X)) + xn * (xb + twice_t(Xb)) - Yb * da - Y * (Yb * dX + yb * dx)
              - yb * ab - yn * sg * (Yb + yb);
        nya = twice_t(Xa * yn + X * ya + Ya * xn + Y * xa + xa * yn + xn * ya);
        nyb = twice_t(Xb * yn + X * yb + Yb * xn + Y * xb + xb * yn + xn * yb);
    } else {
        T opX = X * X - Y * Y;
        T dXa = twice_t(X * Xa - Y * Ya), dXb = twice_t(X * Xb - Y * Yb);
        T opx = xn * (xn + twice_t(X)) - yn * (yn + twice_t(Y));
        T dxa = xa * (xn + twice_t(X)) + xn * (xa + twice_t(Xa)) - ya * (yn + twice_t(Y)) - yn * (ya + twice_t(Ya));
        T dxb = xb * (xn + twice_t(X)) + xn * (xb + twice_t(Xb)) - yb * (yn + twice_t(Y)) - yn * (yb + twice_t(Yb));
        T dX = ddiffabsdX(opX, opx), dx = ddiffabsdx(opX, opx);
        nxa = dX * dXa + dx * dxa;
        nxb = dX * dXb + dx * dxb;
        nya = twice_t(Xa * yn + X * ya + Ya * xn + Y * xa + xa * yn + xn * ya);
        nyb = twice_t(Xb * yn + X * yb + Yb * xn + Y * xb + xb * yn + xn * yb);
    }
    h[0] = nxa; h[1] = nxb; h[2] = nya; h[3] = nyb;
}

// ---------------------------------------------------------------------------
// Frame form of the fr loop.  The delta pair shares one exponent and the
// Hessian another:  (xn, yn) = (ux, uy) 2^E,  (dxnda, dxndb, dynda, dyndb) =
// h 2^F,  with (a, b) 2^-E kept as (cux, cuy).  A step then runs the closures'
// formulas (burning_ship.py:535-859) in plain FP32: the orbit values X, Y are
// floats (the fa table), products of two deltas carry the factor s = 2^E (0
// below 2^-127, where those terms are below FP32 resolution against the
// others), products with the reference Hessian R = Hm 2^g carry 2^(g + E - F)
// (with the delta) or 2^(g - F) (with the orbit).  A diffabs(P, d) is taken
// only when its branch is known: P = 0 (|d|, with the reference's derivative
// convention sgn(0) = +1), or |d| < |P| / 2 (sgn(P) d); otherwise, and at
// orbit points that are both 0 or outside [2^-60, 2^40], the step runs in fr.
// The rounding is FP32's as in fr (one rounding per operation, FMAs where the
// compiler contracts), so the two forms agree to FP32 rounding.
// ---------------------------------------------------------------------------
struct BSFrame {
    float ux, uy; int E;          // deltas
    float s;                      // 2^E, 0 below 2^-127
    float cux, cuy;               // (a, b) 2^-E
    float h[4]; int F;            // Hessian, F = FR_ZERO_E when h = 0
    float am, bm; int ae, be;     // (a, b) = (am 2^ae, bm 2^be)
};

// 2^k for k clamped to [-127, 127] (2^-127 reads as 0)
FSG_DEV float fr_p2c(int k) { return __int_as_float((min(max(k, -127), 127) + 127) << 23); }
// unbiased exponent of |m| for a normal float, -127 for 0 and subnormals
FSG_DEV int fr_fexp(float m) { return ((__float_as_int(m) >> 23) & 0xff) - 127; }

FSG_DEV void frame_set_scale(BSFrame &S) {
    S.s = fr_p2c(S.E);
    S.cux = S.am * fr_p2c(S.ae - S.E);
    S.cuy = S.bm * fr_p2c(S.be - S.E);
}
FSG_DEV int frame_ec(const BSFrame &S) { return max(S.ae, S.be); }

// fr values -> frame (E >= the exponent of c minus 100, so that (a, b) 2^-E
// stays finite)
FSG_DEV void frame_in(BSFrame &S, fr xn, fr yn, const fr h[4]) {
    S.E = max(max(xn.e, yn.e), frame_ec(S) - 100);
    S.ux = xn.m * fr_p2c(xn.e - S.E);
    S.uy = yn.m * fr_p2c(yn.e - S.E);
    frame_set_scale(S);
    S.F = max(max(h[0].e, h[1].e), max(h[2].e, h[3].e));
    for (int k = 0; k < 4; k++) S.h[k] = h[k].m * fr_p2c(h[k].e - S.F);
}
FSG_DEV void frame_out(const BSFrame &S, fr &xn, fr &yn, fr h[4]) {
    xn = fr_norm(S.ux, S.E);
    yn = fr_norm(S.uy, S.E);
    for (int k = 0; k < 4; k++) h[k] = fr_norm(S.h[k], S.F);
}
// lazy renormalisation: max(|ux|, |uy|) and max |h| kept in [2^-30, 2^30]
FSG_DEV void frame_renorm(BSFrame &S) {
    const float m = fmaxf(fabsf(S.ux), fabsf(S.uy));
    if (!(m >= 0x1p-30f && m <= 0x1p30f)) {
        int En;
        if (m < 0x1p-126f) { S.ux = 0.f; S.uy = 0.f; En = frame_ec(S); }
        else {
            En = max(S.E + fr_fexp(m), frame_ec(S) - 100);
            const float sc = fr_p2c(S.E - En);
            S.ux *= sc; S.uy *= sc;
        }
        S.E = En;
        frame_set_scale(S);
    }
    const float mh = fmaxf(fmaxf(fabsf(S.h[0]), fabsf(S.h[1])),
                           fmaxf(fabsf(S.h[2]), fabsf(S.h[3])));
    if (!(mh >= 0x1p-30f && mh <= 0x1p30f)) {
        if (mh < 0x1p-126f) {
            for (int k = 0; k < 4; k++) S.h[k] = 0.f;
            S.F = FR_ZERO_E;
        } else {
            const int k = fr_fexp(mh);
            const float sc = fr_p2c(-k);
            for (int j = 0; j < 4; j++) S.h[j] *= sc;
            S.F += k;
        }
    }
}
// raise the Hessian's exponent to Fn (> F): entries below 2^(Fn - 127) drop
FSG_DEV void frame_raise_F(BSFrame &S, int Fn) {
    const float sc = fr_p2c(S.F - Fn);
    for (int k = 0; k < 4; k++) S.h[k] *= sc;
    S.F = Fn;
}
// h += Hm 2^g (the rebase's addition of the reference Hessian)
FSG_DEV void frame_add_hess(BSFrame &S, float4 Hm, int g) {
    if (Hm.x == 0.f && Hm.y == 0.f && Hm.z == 0.f && Hm.w == 0.f) return;
    if (g - S.F > 60) frame_raise_F(S, g - 30);
    const float k0 = fr_p2c(g - S.F);
    S.h[0] = fmaf(Hm.x, k0, S.h[0]); S.h[1] = fmaf(Hm.y, k0, S.h[1]);
    S.h[2] = fmaf(Hm.z, k0, S.h[2]); S.h[3] = fmaf(Hm.w, k0, S.h[3]);
}

// diffabs(P, d) for d = du 2^E and P known by its sign sp (0 when P = 0) and
// exponent bounds 2^elo <= |P| < 2^(ehi + 1) (burning_ship.py:19-60):
//   P = 0: |d| (with ddiffabsdX = -2 for d < 0, sgn(0) = +1);
//   |d| < |P| / 2: sgn(P) d;
//   |d| > 2^26 |P|: the sign of P + d is d's and 2 P is below FP32 resolution
//   against d.
// Returns false when the exponents leave the branch open.
FSG_DEV bool frame_diffabs(float sp, int elo, int ehi, float du, int E, float &val, float &dX,
                           float &dx) {
    const bool neg = du < 0.f;
    if (sp == 0.f) {
        val = neg ? -du : du; dX = neg ? -2.f : 0.f; dx = neg ? -1.f : 1.f;
        return true;
    }
    const float ad = fabsf(du);
    const int ed = ad == 0.f ? FR_ZERO_E : E + fr_fexp(ad);
    if (ed <= elo - 2) { val = sp * du; dX = 0.f; dx = sp; return true; }
    if (ed < ehi + 27) return false;
    if (sp > 0.f) { val = neg ? -du : du; dX = neg ? -2.f : 0.f; dx = neg ? -1.f : 1.f; }
    else { val = neg ? -du : du; dX = neg ? 0.f : 2.f; dx = neg ? -1.f : 1.f; }
    return true;
}
FSG_DEV float frame_sgn(float v, int e) {           // 0 for an exact 0
    return e == FR_ZERO_E ? 0.f : (signbit(v) ? -1.f : 1.f);
}

// One step of the loop at orbit point (X, Y) with the reference Hessian
// Hm 2^g (zero_ref: the zeros the loop uses right after a dynamic rebase),
// before renormalisation.  Returns false, leaving S untouched, when the step
// has to run in fr.
// DEEP: s = 0 (the deltas below 2^-127), where every product of two deltas,
// or of a delta and the Hessian, is 0 in the frame: those terms are left out.
template <bool DEEP>
FSG_DEV bool bs_frame_step(int flavor, bool hess, BSFrame &S, float X, float Y, int eX, int eY,
                           float4 Hm, int g, bool zero_ref) {
    const float s = DEEP ? 0.f : S.s, ux = S.ux, uy = S.uy;
    const float xs = DEEP ? 0.f : ux * s, ys = DEEP ? 0.f : uy * s;   // xn, yn as floats
    const float xx2 = ux * (DEEP ? 2.f * X : xs + 2.f * X);           // xn (xn + 2 X)
    const float yy2 = uy * (DEEP ? 2.f * Y : ys + 2.f * Y);           // yn (yn + 2 Y)
    const float xy = DEEP ? 0.f : ux * ys;                            // xn yn
    float v1 = 0.f, dX1 = 0.f, dx1 = 0.f, v2 = 0.f, dX2 = 0.f, dx2 = 0.f;
    float vy = 0.f, dXy = 0.f, dxy = 0.f;
    const bool use1 = flavor == 1 || flavor == 5, use2 = flavor >= 4;
    const bool usey = flavor == 2 || flavor == 3;
    const float sX = frame_sgn(X, eX), sY = frame_sgn(Y, eY);
    if (use1) {
        // P1 = X Y: 2^(eX + eY) <= |P1| < 2^(eX + eY + 2)
        // xn yn + xn Y + yn X
        const float o1 = DEEP ? fmaf(uy, X, ux * Y) : fmaf(uy, X, fmaf(ux, Y, xy));
        if (!frame_diffabs(sX * sY, eX + eY, eX + eY + 1, o1, S.E, v1, dX1, dx1)) return false;
    }
    if (use2) {
        // P2 = X^2 - Y^2 in the rounding of the fr closure (a component
        // below 2^-100 against one above 2^-60 drops out of it)
        const float P2 = __fsub_rn(__fmul_rn(X, X), __fmul_rn(Y, Y));
        const int e2 = fr_fexp(fabsf(P2));
        if (!frame_diffabs(P2 == 0.f ? 0.f : (P2 > 0.f ? 1.f : -1.f), e2, e2, xx2 - yy2, S.E,
                           v2, dX2, dx2))
            return false;
    }
    if (usey) {
        if (!frame_diffabs(sY, eY, eY, uy, S.E, vy, dXy, dxy)) return false;
    }
    // |Y + yn| and sgn(Y + yn) with sgn(0) = +1 (flavors 2, 3): the branch
    // is known here, so the sign is sgn(Y) unless |yn| dominates or Y = 0
    const float ab = DEEP ? fabsf(Y) : fabsf(Y + ys);
    const float sg = (sY != 0.f && dXy == 0.f) ? sY : (uy < 0.f ? -1.f : 1.f);
    if (hess) {
        const bool hz = zero_ref || (Hm.x == 0.f && Hm.y == 0.f && Hm.z == 0.f && Hm.w == 0.f);
        float k1 = 0.f, k0 = 0.f;
        if (!hz) {
            // the terms in 2^(g - F) are products with X or Y
            const bool need0 = (dX1 != 0.f || dX2 != 0.f || dXy != 0.f) && (X != 0.f || Y != 0.f);
            if (g + S.E - S.F > 60) frame_raise_F(S, g + S.E - 30);
            if (need0 && g - S.F > 60) frame_raise_F(S, g - 30);
            k1 = fr_p2c(g + S.E - S.F);
            k0 = need0 ? fr_p2c(g - S.F) : 0.f;
        } else {
            Hm = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        const float h0 = S.h[0], h1 = S.h[1], h2 = S.h[2], h3 = S.h[3];
        float nxa, nxb, nya, nyb;
        if (DEEP) {
            // the same closures without the terms in s (xn = yn = 0 against X, Y)
            if (flavor == 1 || flavor == 2) {
                nxa = 2.f * (X * h0 + Hm.x * ux * k1) - 2.f * (Y * h2 + Hm.z * uy * k1);
                nxb = 2.f * (X * h1 + Hm.y * ux * k1) - 2.f * (Y * h3 + Hm.w * uy * k1);
            } else if (flavor == 3) {
                nxa = h0 * (2.f * X) + ux * (2.f * Hm.x * k1) - Hm.z * vy * k1
                      - Y * (Hm.z * dXy * k0 + h2 * dxy) - h2 * ab - sg * (uy * Hm.z * k1);
                nxb = h1 * (2.f * X) + ux * (2.f * Hm.y * k1) - Hm.w * vy * k1
                      - Y * (Hm.w * dXy * k0 + h3 * dxy) - h3 * ab - sg * (uy * Hm.w * k1);
            } else {
                const float dxa2 = h0 * (2.f * X) + ux * (2.f * Hm.x * k1)
                                   - h2 * (2.f * Y) - uy * (2.f * Hm.z * k1);
                const float dxb2 = h1 * (2.f * X) + ux * (2.f * Hm.y * k1)
                                   - h3 * (2.f * Y) - uy * (2.f * Hm.w * k1);
                const float dXa2 = 2.f * (X * Hm.x - Y * Hm.z) * k0;
                const float dXb2 = 2.f * (X * Hm.y - Y * Hm.w) * k0;
                nxa = dX2 * dXa2 + dx2 * dxa2;
                nxb = dX2 * dXb2 + dx2 * dxb2;
            }
            if (flavor == 1 || flavor == 5) {
                const float dxa = h0 * Y + h2 * X + (ux * Hm.z + uy * Hm.x) * k1;
                const float dxb = h1 * Y + h3 * X + (ux * Hm.w + uy * Hm.y) * k1;
                const float dXa = (Hm.x * Y + X * Hm.z) * k0, dXb = (Hm.y * Y + X * Hm.w) * k0;
                nya = 2.f * (dX1 * dXa + dx1 * dxa);
                nyb = 2.f * (dX1 * dXb + dx1 * dxb);
            } else if (flavor == 2) {
                nya = 2.f * (Hm.x * vy * k1 + X * (dXy * Hm.z * k0 + dxy * h2) + h0 * ab
                             + sg * (ux * Hm.z * k1));
                nyb = 2.f * (Hm.y * vy * k1 + X * (dXy * Hm.w * k0 + dxy * h3) + h1 * ab
                             + sg * (ux * Hm.w * k1));
            } else {
                nya = 2.f * ((Hm.x * uy + Hm.z * ux) * k1 + X * h2 + Y * h0);
                nyb = 2.f * ((Hm.y * uy + Hm.w * ux) * k1 + X * h3 + Y * h1);
            }
        } else if (flavor == 1 || flavor == 2) {
            nxa = 2.f * ((X + xs) * h0 + Hm.x * ux * k1) - 2.f * ((Y + ys) * h2 + Hm.z * uy * k1);
            nxb = 2.f * ((X + xs) * h1 + Hm.y * ux * k1) - 2.f * ((Y + ys) * h3 + Hm.w * uy * k1);
        } else if (flavor == 3) {
            nxa = h0 * (xs + 2.f * X) + ux * (h0 * s + 2.f * Hm.x * k1) - Hm.z * vy * k1
                  - Y * (Hm.z * dXy * k0 + h2 * dxy) - h2 * ab
                  - sg * (uy * Hm.z * k1 + uy * h2 * s);
            nxb = h1 * (xs + 2.f * X) + ux * (h1 * s + 2.f * Hm.y * k1) - Hm.w * vy * k1
                  - Y * (Hm.w * dXy * k0 + h3 * dxy) - h3 * ab
                  - sg * (uy * Hm.w * k1 + uy * h3 * s);
        } else {
            const float dxa2 = h0 * (xs + 2.f * X) + ux * (h0 * s + 2.f * Hm.x * k1)
                               - h2 * (ys + 2.f * Y) - uy * (h2 * s + 2.f * Hm.z * k1);
            const float dxb2 = h1 * (xs + 2.f * X) + ux * (h1 * s + 2.f * Hm.y * k1)
                               - h3 * (ys + 2.f * Y) - uy * (h3 * s + 2.f * Hm.w * k1);
            const float dXa2 = 2.f * (X * Hm.x - Y * Hm.z) * k0;
            const float dXb2 = 2.f * (X * Hm.y - Y * Hm.w) * k0;
            nxa = dX2 * dXa2 + dx2 * dxa2;
            nxb = dX2 * dXb2 + dx2 * dxb2;
        }
        if (DEEP) {
        } else if (flavor == 1 || flavor == 5) {
            const float dxa = (h0 * uy + ux * h2) * s + h0 * Y + h2 * X
                              + (ux * Hm.z + uy * Hm.x) * k1;
            const float dxb = (h1 * uy + ux * h3) * s + h1 * Y + h3 * X
                              + (ux * Hm.w + uy * Hm.y) * k1;
            const float dXa = (Hm.x * Y + X * Hm.z) * k0, dXb = (Hm.y * Y + X * Hm.w) * k0;
            nya = 2.f * (dX1 * dXa + dx1 * dxa);
            nyb = 2.f * (dX1 * dXb + dx1 * dxb);
        } else if (flavor == 2) {
            nya = 2.f * (Hm.x * vy * k1 + X * (dXy * Hm.z * k0 + dxy * h2) + h0 * ab
                         + sg * (ux * Hm.z * k1 + ux * h2 * s));
            nyb = 2.f * (Hm.y * vy * k1 + X * (dXy * Hm.w * k0 + dxy * h3) + h1 * ab
                         + sg * (ux * Hm.w * k1 + ux * h3 * s));
        } else {
            nya = 2.f * ((Hm.x * uy + Hm.z * ux) * k1 + X * h2 + Y * h0 + (h0 * uy + ux * h2) * s);
            nyb = 2.f * ((Hm.y * uy + Hm.w * ux) * k1 + X * h3 + Y * h1 + (h1 * uy + ux * h3) * s);
        }
        S.h[0] = nxa; S.h[1] = nxb; S.h[2] = nya; S.h[3] = nyb;
    }
    float nx, ny;
    if (flavor == 1) {
        nx = xx2 - yy2 + S.cux; ny = 2.f * v1 - S.cuy;
    } else if (flavor == 2) {
        nx = xx2 - yy2 + S.cux; ny = 2.f * (X * vy + ux * ab) - S.cuy;
    } else if (flavor == 3) {
        nx = xx2 - Y * vy - uy * ab + S.cux;
        ny = 2.f * (DEEP ? X * uy + Y * ux : X * uy + Y * ux + xy) - S.cuy;
    } else if (flavor == 4) {
        nx = v2 + S.cux; ny = 2.f * (DEEP ? X * uy + Y * ux : X * uy + Y * ux + xy) - S.cuy;
    } else {
        nx = v2 + S.cux; ny = 2.f * v1 - S.cuy;
    }
    S.ux = nx; S.uy = ny;
    return true;
}

// The step at an orbit point X = Y = 0 (every term is a product of two deltas
// or c): the deltas' exponent moves to E' = max(2 E, Ec - 100) and the
// Hessian's to F + E' - E, so that the general step's products "u u s" and
// "h u s" with s = 2^(2E - E') land in the new frames (its products with X
// and Y vanish).
FSG_DEV void bs_frame_step_zero(int flavor, bool hess, BSFrame &S, float4 Hm, int g,
                                bool zero_ref) {
    const int E = S.E;
    const int En = max(2 * E, frame_ec(S) - 100);
    BSFrame T = S;
    T.s = fr_p2c(2 * E - En);
    T.cux = S.am * fr_p2c(S.ae - En);
    T.cuy = S.bm * fr_p2c(S.be - En);
    if (T.F != FR_ZERO_E) T.F = S.F + En - E;
    // all diffabs arguments are 0 here: the step is always taken
    bs_frame_step<false>(flavor, hess, T, 0.f, 0.f, FR_ZERO_E, FR_ZERO_E, Hm, g, zero_ref);
    S = T;
    S.E = En;
    frame_set_scale(S);
}

// |X + d| <= |d| for one component (d = du 2^E), as the fr values round:
// true when X = 0 or |X| < 2^-25 |d| (X + d rounds to d), false when
// |d| < |X| / 2; open otherwise
FSG_DEV bool frame_le(float du, int E, int eX, bool &le) {
    if (eX == FR_ZERO_E) { le = true; return true; }
    const float ad = fabsf(du);
    const int ed = ad == 0.f ? FR_ZERO_E : E + fr_fexp(ad);
    if (ed <= eX - 2) { le = false; return true; }
    if (ed >= eX + 26) { le = true; return true; }
    return false;
}
// The loop's tests at orbit point (X, Y) (perturbation.py:1627-1711) in the
// frame form: 0 none, 1 escape, 2 rebase where X + xn, Y + yn round to xn, yn
// (the deltas stay), 3 to be decided in fr
FSG_DEV int bs_frame_tests(const BSFrame &S, float X, float Y, int eX, int eY, float M2s,
                           bool div_rebase) {
    bool lex, ley;
    if (S.E > 10) return 3;                             // deltas above 2^40: fr from here
    if (!frame_le(S.ux, S.E, eX, lex) || !frame_le(S.uy, S.E, eY, ley)) return 3;
    const float XX = fmaf(S.ux, S.s, X), YY = fmaf(S.uy, S.s, Y);
    const float q = fmaf(XX, XX, YY * YY);
    if (fabsf(q - M2s) <= M2s * 0x1p-18f) return 3;
    if (q > M2s) return 1;
    if (div_rebase || (lex && ley)) return (lex && ley) ? 2 : 3;
    return 0;
}

template <class T> struct IsDouble { static constexpr bool value = false; };
template <> struct IsDouble<double> { static constexpr bool value = true; };
template <class T> struct IsFr { static constexpr bool value = false; };
template <> struct IsFr<fr> { static constexpr bool value = true; };
template <class T> struct IsXr { static constexpr bool value = false; };
template <> struct IsXr<xf> { static constexpr bool value = true; };

// FL: the flavor as a compile-time constant (1..5), or 0 to read C.flavor
template <class T, int FL>
FSG_DEV void pixel_bs(const TileDev &T_, const CalcDev &C, long long ip,
                      unsigned long long &nfull, unsigned long long &nbla,
                      unsigned long long &nreb, unsigned long long &itsum) {
    const TileDev &Tl = T_;
    const RefDev &R = *Tl.ref;
    const long long np = (long long)Tl.nx * Tl.ny;
    const int flavor = FL ? FL : C.flavor;
    const bool hess = C.calc_dzndc != 0;
    const int order = R.order, div_iter = R.div_iter;
    // perturbation.py:2260-2280 ref_path_c_from_pix_BS through Xrange values
    double2 pp = fsg_pixel(Tl, ip);
    double px = pp.x, py = pp.y;
    double x1 = Tl.lin[0] * px + Tl.lin[1] * py;
    double y1 = Tl.lin[2] * px + Tl.lin[3] * py;
    xf dxr; dxr.m = Tl.dx_m; dxr.e = Tl.dx_e;
    xc c_xr = xf_mul_c(dxr, cx(x1, y1));
    double ar, br; int ae, be;
    xr_coexp_r(c_xr.re, c_xr.e, Tl.drift_re, Tl.drift_e, ar, br, ae);
    const T a = from_me<T>(ar + br, ae);
    xr_coexp_r(c_xr.im, c_xr.e, Tl.drifty_m, Tl.drifty_e, ar, br, be);
    const T b = from_me<T>(ar + br, be);

    T xn = cst<T>(0.f), yn = cst<T>(0.f);
    T h[4] = {cst<T>(0.f), cst<T>(0.f), cst<T>(0.f), cst<T>(0.f)};
    const fr M2f = fr_from_d(C.M2);
    int w = 0, n = 0; signed char stop = -1; bool dyn = true;
    // calc_orbit snapshots (perturbation.py:1501-1508), the reference's two
    // forms only: the FP32 + exponent instantiation compiles without them
    constexpr bool FR_FORM = IsFr<T>::value;
    constexpr bool XR_FORM = IsXr<T>::value;
    constexpr bool ORB_FORM = !FR_FORM;
    const int bs = ORB_FORM ? C.backshift : 0;
    OrbitSnap<double2> S;
    S.init(bs, cx(0., 0.));
    // the reference's BLA step (perturbation.py:1520-1545, 1793-1811)
    auto apply_bla = [&](int step, int ib) {
        T M[8];
        BSRef<T>::bla(R, ib, M);
        n += step; w = (w + step) % order;
        T nx = M[0] * xn + M[1] * yn + M[4] * a + M[5] * b;
        T ny = M[2] * xn + M[3] * yn + M[6] * a + M[7] * b;
        xn = nx; yn = ny;
        if (hess) {
            T xa = M[0] * h[0] + M[1] * h[2], xb = M[0] * h[1] + M[1] * h[3];
            T ya = M[2] * h[0] + M[3] * h[2], yb = M[2] * h[1] + M[3] * h[3];
            h[0] = xa; h[1] = xb; h[2] = ya; h[3] = yb;
        }
        nbla++;
    };
    // frame form of the FP32 + exponent loop (BSFrame); the fr values are
    // current whenever frm is false
    BSFrame Fm;
    bool frm = false;
    float M2s = 0.f;
    // with |X|, |Y| and the deltas below 2^(eMlim + 1), |Z + dz|^2 < M2 / 8
    const int eMlim = min((M2f.e >> 1) - 4, 40);
    if constexpr (FR_FORM) {
        Fm.am = a.m; Fm.ae = a.e; Fm.bm = b.m; Fm.be = b.e;
        M2s = (float)C.M2;
    }
    for (;;) {
        bool bla_done = false, stepped = false;
        if constexpr (FR_FORM) {
            if (frm) {
            // Steps in the frame form from orbit point w on, until the loop ends
            // (0), a BLA step was taken (1), the step at w has to run in fr (2) or
            // the tests at w have to (3); the fr values are current on return.
            auto frame_run = [&]() -> int {
                int4 fz = __ldg(&R.bs_fz[w]);
                for (;;) {
                    if (C.bla && R.bla_len > 0 && (w & 7) == 0 &&
                        (1 << FSG_STG_COMPRESSED) < R.first_invalid - w && bla_possible(R, w)) {
                        int ib;
                        const int step = BLAGet<T>::get(R, fr_norm(Fm.ux, Fm.E),
                                                        fr_norm(Fm.uy, Fm.E), w, ib);
                        if (step != 0) {
                            frame_out(Fm, xn, yn, h);
                            apply_bla(step, ib);
                            return 1;
                        }
                    }
                    if (!(fz.x & 5)) { frame_out(Fm, xn, yn, h); return 2; }
                    float4 Hm = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (hess && !dyn) Hm = __ldg(&R.bs_fh[w]);
                    if (fz.x & 4) {
                        bs_frame_step_zero(flavor, hess, Fm, Hm, fz.y, dyn);
                    } else {
                        const float4 fa = __ldg(&R.bs_fa[w]);
                        const int eX = __float_as_int(fa.z), eY = __float_as_int(fa.w);
                        const bool ok = Fm.s == 0.f
                            ? bs_frame_step<true>(flavor, hess, Fm, fa.x, fa.y, eX, eY, Hm,
                                                  fz.y, dyn)
                            : bs_frame_step<false>(flavor, hess, Fm, fa.x, fa.y, eX, eY, Hm,
                                                   fz.y, dyn);
                        if (!ok) {
                            frame_out(Fm, xn, yn, h);
                            return 2;
                        }
                    }
                    frame_renorm(Fm);
                    n += 1;
                    nfull++;
                    if (n >= C.max_iter) { stop = 0; frame_out(Fm, xn, yn, h); return 0; }
                    w += 1;
                    if (w >= order) w = w % order;
                    fz = __ldg(&R.bs_fz[w]);
                    // deltas below the orbit point's bound: no escape, no rebase
                    const int ed = Fm.E + fr_fexp(fmaxf(fabsf(Fm.ux), fabsf(Fm.uy)));
                    if (ed <= min(fz.z, eMlim) && fz.w <= eMlim) { dyn = false; continue; }
                    const bool divr = w >= div_iter - 1;
                    int res = 3;
                    if (fz.x & 2) {
                        const float4 fb = __ldg(&R.bs_fa[w]);
                        res = bs_frame_tests(Fm, fb.x, fb.y, __float_as_int(fb.z),
                                             __float_as_int(fb.w), M2s, divr);
                    }
                    if (res == 0) { dyn = false; continue; }
                    if (res == 1) { stop = 1; frame_out(Fm, xn, yn, h); return 0; }
                    if (res == 2) {
                        // rebase where X + xn, Y + yn round to the deltas: they stay
                        if (hess) frame_add_hess(Fm, __ldg(&R.bs_fh[w]), fz.y);
                        if (!divr) dyn = true;
                        w = 0; nreb++;
                        fz = __ldg(&R.bs_fz[0]);
                        continue;
                    }
                    frame_out(Fm, xn, yn, h);
                    return 3;
                }
            };
                frm = false;
                const int r = frame_run();
                if (r == 0) break;
                if (r == 1) continue;
                bla_done = true;
                stepped = r == 3;
            }
        }
        if (!stepped) {
            if (C.bla && R.bla_len > 0 && !bla_done && (w & 7) == 0) {
                int ib;
                // the reference compares the double value of |dz| (0 when it
                // underflows, perturbation.py:1123-1135)
                const int step = BLAGet<T>::get(R, xn, yn, w, ib);
                if (step != 0) { apply_bla(step, ib); continue; }
            }
            n += 1;
            nfull++;
            T X, Y;
            BSRef<T>::orbit(R, w, X, Y);
            if (hess) {
                T Xa = cst<T>(0.f), Xb = cst<T>(0.f), Ya = cst<T>(0.f), Yb = cst<T>(0.f);
                if (!dyn) BSRef<T>::hess(R, w, Xa, Xb, Ya, Yb);
                bs_hess<T>(flavor, h, xn, yn, X, Y, Xa, Xb, Ya, Yb);
            }
            bs_zn<T>(flavor, xn, yn, X, Y, a, b);
            if (n >= C.max_iter) { stop = 0; break; }
            w += 1;
            if (w >= order) w = w % order;
        }
        if constexpr (XR_FORM) {
            // the Xrange branch's tests (perturbation.py:1627-1731): escape on
            // the standard values; rebase when the reference diverges from
            // the standard sum; the dynamic rebase tested componentwise on the
            // standard values, then confirmed with |Z + z|^2 <= |z|^2 in
            // Xrange (with the side table's value of the orbit where it holds
            // one) -- a refused confirmation leaves bool_dyn_rebase set
            const double2 Zs = __ldg(&R.Zn[w]);
            const double xs = to_d(xn), ys = to_d(yn);
            const double XXd = xs + Zs.x, YYd = ys + Zs.y;
            if (bs > 0) S.take(n, bs, cx(XXd, YYd));
            if (d_sq_gt(XXd * XXd + YYd * YYd, C.M2)) { stop = 1; break; }
            if (w >= div_iter - 1) {
                xn = from_d<T>(XXd); yn = from_d<T>(YYd);
                if (hess) {
                    T Ha, Hb, Hc, Hd;
                    BSRef<T>::hess(R, w, Ha, Hb, Hc, Hd);
                    h[0] += Ha; h[1] += Hb; h[2] += Hc; h[3] += Hd;
                }
                w = 0; nreb++; continue;
            }
            dyn = d_abs_le(XXd, xs) && d_abs_le(YYd, ys);
            if (dyn) {
                T Xt, Yt;
                const bool tab = BSRef<T>::table(R, w, Xt, Yt);
                const T XXx = tab ? xn + Xt : xf_add_s(xn, Zs.x);
                const T YYx = tab ? yn + Yt : xf_add_s(yn, Zs.y);
                if (xf_le(XXx * XXx + YYx * YYx, xn * xn + yn * yn)) {
                    xn = XXx; yn = YYx;
                    if (hess) {
                        T Ha, Hb, Hc, Hd;
                        BSRef<T>::hess(R, w, Ha, Hb, Hc, Hd);
                        h[0] += Ha; h[1] += Hb; h[2] += Hc; h[3] += Hd;
                    }
                    w = 0; nreb++; continue;
                }
            }
            continue;
        }
        T Xs, Ys;
        BSRef<T>::orbit(R, w, Xs, Ys);
        T XX = xn + Xs, YY = yn + Ys;
        if constexpr (ORB_FORM) {
            const double XXd = to_d(XX), YYd = to_d(YY);
            if (bs > 0) S.take(n, bs, cx(XXd, YYd));             // :1641-1651
            if (d_sq_gt(XXd * XXd + YYd * YYd, C.M2)) { stop = 1; break; }
        } else {
            if (fr_escaped(XX, YY, M2f, C.M2)) { stop = 1; break; }
        }
        if (w >= div_iter - 1) {
            xn = XX; yn = YY;
            if (hess) {
                T Ha, Hb, Hc, Hd;
                BSRef<T>::hess(R, w, Ha, Hb, Hc, Hd);
                h[0] += Ha; h[1] += Hb; h[2] += Hc; h[3] += Hd;
            }
            w = 0; nreb++; continue;
        }
        dyn = abs_le(XX, xn) && abs_le(YY, yn);
        if (dyn) {
            xn = XX; yn = YY;
            if (hess) {
                T Ha, Hb, Hc, Hd;
                BSRef<T>::hess(R, w, Ha, Hb, Hc, Hd);
                h[0] += Ha; h[1] += Hb; h[2] += Hc; h[3] += Hd;
            }
            w = 0; nreb++; continue;
        }
        if constexpr (FR_FORM) {
            // the frame form takes over while the deltas stay below 2^11 and
            // the next step can run there
            if (max(xn.e, yn.e) <= 10 && (__ldg(&R.bs_fz[w]).x & 5)) {
                frame_in(Fm, xn, yn, h);
                frm = true;
            }
        }
    }
    // end of iterations (:1745-1757): the Xrange branch adds the standard
    // orbit value to the Xrange delta
    double xo, yo;
    if constexpr (XR_FORM) {
        const double2 Zs = __ldg(&R.Zn[w]);
        xo = to_d(xf_add_s(xn, Zs.x)); yo = to_d(xf_add_s(yn, Zs.y));
    } else {
        T Xe, Ye;
        BSRef<T>::orbit(R, w, Xe, Ye);
        xo = to_d(xn + Xe); yo = to_d(yn + Ye);
    }
    double hd[4] = {0., 0., 0., 0.};
    if (hess) {
        // the Hessian in the tile's unit: the reference's scale times 2^dzs
        T Ha, Hb, Hc, Hd;
        BSRef<T>::hess(R, w, Ha, Hb, Hc, Hd);
        hd[0] = to_d(scale2(h[0] + Ha, Tl.dzs)); hd[1] = to_d(scale2(h[1] + Hb, Tl.dzs));
        hd[2] = to_d(scale2(h[2] + Hc, Tl.dzs)); hd[3] = to_d(scale2(h[3] + Hd, Tl.dzs));
        if (Tl.proj) {
            // Expmap (perturbation.py:1772-1776)
            const double m = fsg_dzndc_modifier(Tl, ip);
            hd[0] *= m; hd[1] *= m; hd[2] *= m; hd[3] *= m;
        }
    }
    double *Z = (double *)Tl.Z;
    if (bs > 0) {
        // :1778-1787: the reference replays with AA = a + Re(Z_1) and
        // BB = b + Im(Z_1) = b - b_ref (kept as is)
        const double2 Z1 = __ldg(&R.Zn[1]);
        const double AA = to_d(a) + Z1.x, BB = to_d(b) + Z1.y;
        double xr = S.z2.x, yr = S.z2.y;
        for (int i2 = S.i2; i2 < n - bs; i2++) {
            double nx_, ny_;
            bs_map(flavor, xr, yr, AA, BB, nx_, ny_);
            xr = nx_; yr = ny_;
        }
        Z[(long long)Tl.i_orb * np + ip] = xr;
        Z[(long long)(Tl.i_orb + 1) * np + ip] = yr;
    }
    Z[ip] = xo; Z[np + ip] = yo;
    if (hess) { Z[2 * np + ip] = hd[0]; Z[3 * np + ip] = hd[1]; Z[4 * np + ip] = hd[2]; Z[5 * np + ip] = hd[3]; }
    if (Tl.U) Tl.U[ip] = w;
    Tl.stop_iter[ip] = n; Tl.stop_reason[ip] = stop;
    double absd = 0.5 * (hypot(hd[0] + hd[3], hd[1] - hd[2]) + hypot(hd[0] - hd[3], hd[1] + hd[2]));
    fsg_epilogue(Tl, C, ip, cx(xo, yo), absd, n);
    itsum += (unsigned long long)n;
}

// the FP32 + exponent kernels hold three 256-thread blocks per SM (at most 85
// registers a thread)
template <class T, int FL>
__global__ void __launch_bounds__(256, IsFr<T>::value ? 3 : 1)
k_perturb_bs(WorkDev W, CalcDev C) {
    extern __shared__ long long s_start[];          // [W.ntiles + 1], sized at launch
    fsg_load_starts(W, s_start);
    unsigned long long nfull = 0, nbla = 0, nreb = 0, itsum = 0;
    int t; long long ip;
    while (true) {
        if (*W.cancel) { *W.status = 1; break; }
        if (!fsg_claim(W, s_start, t, ip)) break;
        const unsigned long long before = itsum;
        pixel_bs<T, FL>(W.tiles[t], C, ip, nfull, nbla, nreb, itsum);
        fsg_account(W, itsum - before);
    }
    fsg_flush_stats(W, itsum, nfull, nbla, nreb);
}
