/*
 * fs_oracle.c -- CPU restatement of Fractalshades' per-pixel iteration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA kernels of
 * fractalshades_gb300 are checked against.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load it; the product path never does.
 *
 * Every function restates the numba code of the reference (Fractalshades 1.2.1)
 * and cites the file:line it follows (paths relative to src/fractalshades/).
 * It is compiled with strict IEEE semantics (-O2 -ffp-contract=off, no
 * fast-math) so that each operation rounds exactly once, in the order written
 * in the reference source.
 *
 * Conventions
 *   complex arrays are interleaved (re, im) doubles, i.e. numpy complex128;
 *   Z is laid out [nZ][npts] (numpy C order of the reference's Z[nZ, npts]).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------- */
/* Complex helpers: numba / CPython / numpy complex128 semantics              */
/* ------------------------------------------------------------------------- */
typedef struct { double re, im; } cplx;

static inline cplx C(double re, double im) { cplx z = {re, im}; return z; }
static inline cplx cadd(cplx a, cplx b) { return C(a.re + b.re, a.im + b.im); }
/* (a+bi)(c+di) = (ac-bd) + (ad+bc)i : numba complex_mul_impl, CPython _Py_c_prod */
static inline cplx cmul(cplx a, cplx b) {
    return C(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
/* float * complex: the float is promoted to complex(x, 0.) first */
static inline cplx rmul(double x, cplx b) { return cmul(C(x, 0.), b); }
/* complex + float: the float is promoted to complex(x, 0.) first */
static inline cplx caddr(cplx a, double x) { return C(a.re + x, a.im + 0.); }

/* ------------------------------------------------------------------------- */
/* Xrange scalars: numpy_utils/numba_xr.py                                    */
/* value = mantissa * 2**exp ; complex values share one exponent              */
/* ------------------------------------------------------------------------- */
typedef struct { double re, im; int32_t e; } xc;  /* complex128 Xrange record */
typedef struct { double m; int32_t e; } xf;       /* float64 Xrange record    */

static inline uint64_t d2u(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double u2d(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }

/* numba_xr.py:662-675 _frexp: rewrite the biased exponent to 1023 (m in [1, 2)) */
static inline double xr_frexp(double m, int32_t *e) {
    uint64_t b = d2u(m);
    *e = (int32_t)((b >> 52) & 0x7ff) - 0x3ff;
    return u2d((b & 0x8000000000000000ULL) + (0x3ffULL << 52) + (b & 0xfffffffffffffULL));
}
/* numba_xr.py:677-684 _normalize_real */
static inline double xr_norm_real(double m, int32_t exp, int32_t *eo) {
    if (m == 0.) { *eo = 0; return m; }
    int32_t ne; double nm = xr_frexp(m, &ne);
    *eo = exp + ne; return nm;
}
/* numba_xr.py:686-695 _exp2_shift: add to the biased exponent, clamped at 0 */
static inline double xr_exp2_shift(double m, int64_t shift) {
    uint64_t b = d2u(m);
    int64_t ex = (int64_t)((b >> 52) & 0x7ff) + shift;
    if (ex < 0) ex = 0;
    return u2d((b & 0x8000000000000000ULL) + ((uint64_t)ex << 52) + (b & 0xfffffffffffffULL));
}
/* numba_xr.py:390-413 _need_renorm: |unbiased exponent| > 100 */
static inline int xr_need_renorm_r(double m) {
    int64_t d = (int64_t)((d2u(m) >> 52) & 0x7ff) - 1023;
    return (d < 0 ? -d : d) > 100;
}
static inline int xr_need_renorm_c(cplx m) { return xr_need_renorm_r(m.re) || xr_need_renorm_r(m.im); }

/* numba_xr.py:708-727 _coexp_ufunc, real implementation */
static inline void xr_coexp_r(double m0, int32_t e0, double m1, int32_t e1,
                              double *o0, double *o1, int32_t *eo) {
    int64_t d = (int64_t)e0 - (int64_t)e1;
    if (m0 == 0.) { *eo = e1; }
    else if (m1 == 0.) { *eo = e0; }
    else if (e1 > e0) { m0 = xr_exp2_shift(m0, d); *eo = e1; }
    else if (e0 > e1) { m1 = xr_exp2_shift(m1, -d); *eo = e0; }
    else { *eo = e0; }
    *o0 = m0; *o1 = m1;
}
/* numba_xr.py:729-750 _coexp_ufunc, complex implementation */
static inline void xr_coexp_c(cplx m0, int32_t e0, cplx m1, int32_t e1,
                              cplx *o0, cplx *o1, int32_t *eo) {
    int64_t d = (int64_t)e0 - (int64_t)e1;
    if (m0.re == 0. && m0.im == 0.) { *eo = e1; }
    else if (m1.re == 0. && m1.im == 0.) { *eo = e0; }
    else if (e1 > e0) { m0 = C(xr_exp2_shift(m0.re, d), xr_exp2_shift(m0.im, d)); *eo = e1; }
    else if (e0 > e1) { m1 = C(xr_exp2_shift(m1.re, -d), xr_exp2_shift(m1.im, -d)); *eo = e0; }
    else { *eo = e0; }
    *o0 = m0; *o1 = m1;
}
/* numba_xr.py:636-656 _normalize, complex: each part then co-exponent */
static inline xc xr_normalize_c(cplx m, int32_t exp) {
    int32_t ere, eim; double nre = xr_norm_real(m.re, exp, &ere);
    double nim = xr_norm_real(m.im, exp, &eim);
    double cr, ci; int32_t ce; xr_coexp_r(nre, ere, nim, eim, &cr, &ci, &ce);
    xc r = {cr, ci, ce}; return r;
}
static inline xf xr_normalize_r(double m, int32_t exp) {
    int32_t e; double nm = xr_norm_real(m, exp, &e); xf r = {nm, e}; return r;
}
/* numba_xr.py:782-795 to_Xrange_scalar(number) */
static inline xc xr_from_c(cplx z) { return xr_normalize_c(z, 0); }
static inline xf xr_from_r(double x) { return xr_normalize_r(x, 0); }
static inline cplx xm(xc a) { return C(a.re, a.im); }

/* numba_xr.py:318-352 extended_add, xr + xr */
static inline xc xr_add(xc a, xc b) {
    cplx o0, o1; int32_t e; xr_coexp_c(xm(a), a.e, xm(b), b.e, &o0, &o1, &e);
    cplx s = cadd(o0, o1); xc r = {s.re, s.im, e}; return r;
}
/* extended_add, xr + complex std */
static inline xc xr_add_s(xc a, cplx z) {
    xc b;
    if (xr_need_renorm_c(z)) b = xr_normalize_c(z, 0); else { b.re = z.re; b.im = z.im; b.e = 0; }
    return xr_add(a, b);
}
/* real xr + real xr */
static inline xf xf_add(xf a, xf b) {
    double o0, o1; int32_t e; xr_coexp_r(a.m, a.e, b.m, b.e, &o0, &o1, &e);
    xf r = {o0 + o1, e}; return r;
}
static inline xf xf_sub(xf a, xf b) {
    double o0, o1; int32_t e; xr_coexp_r(a.m, a.e, b.m, b.e, &o0, &o1, &e);
    xf r = {o0 - o1, e}; return r;
}
/* real xr + float std */
static inline xf xf_add_s(xf a, double x) {
    xf b; if (xr_need_renorm_r(x)) b = xr_normalize_r(x, 0); else { b.m = x; b.e = 0; }
    return xf_add(a, b);
}
/* complex xr + real xr (mixed coexp, numba_xr.py:729-750 with a float m1) */
static inline xc xr_add_xf(xc a, xf b) {
    xc bb = {b.m, 0., b.e};
    return xr_add(a, bb);
}
/* numba_xr.py:416-444 extended_mul */
static inline xc xr_mul(xc a, xc b) {
    cplx m = cmul(xm(a), xm(b)); int32_t e = (int32_t)((uint32_t)a.e + (uint32_t)b.e);
    if (xr_need_renorm_c(m)) return xr_normalize_c(m, e);
    xc r = {m.re, m.im, e}; return r;
}
static inline xc xr_mul_s(cplx s, xc b) {   /* complex std * xr */
    cplx m = cmul(s, xm(b));
    if (xr_need_renorm_c(m)) return xr_normalize_c(m, b.e);
    xc r = {m.re, m.im, b.e}; return r;
}
static inline xc xr_mul_r(double s, xc b) { /* float std * complex xr */
    cplx m = rmul(s, xm(b));
    if (xr_need_renorm_c(m)) return xr_normalize_c(m, b.e);
    xc r = {m.re, m.im, b.e}; return r;
}
static inline xc xf_mul_c(xf a, cplx z) {   /* real xr * complex std */
    cplx m = rmul(a.m, z);
    if (xr_need_renorm_c(m)) return xr_normalize_c(m, a.e);
    xc r = {m.re, m.im, a.e}; return r;
}
static inline xf xf_mul(xf a, xf b) {
    double m = a.m * b.m; int32_t e = (int32_t)((uint32_t)a.e + (uint32_t)b.e);
    if (xr_need_renorm_r(m)) return xr_normalize_r(m, e);
    xf r = {m, e}; return r;
}
static inline xf xf_mul_s(double s, xf b) {
    double m = s * b.m;
    if (xr_need_renorm_r(m)) return xr_normalize_r(m, b.e);
    xf r = {m, b.e}; return r;
}
/* numba_xr.py:531-561 extended_abs2 (no renormalisation) */
static inline xf xr_abs2(xc a) {
    xf r = {a.re * a.re + a.im * a.im, (int32_t)((uint32_t)a.e + (uint32_t)a.e)}; return r;
}
/* numba_xr.py:476-510 comparisons through the co-exponent */
static inline int xf_lt_s(xf a, double x) {
    double o0, o1; int32_t e; xr_coexp_r(a.m, a.e, x, 0, &o0, &o1, &e); return o0 < o1;
}
static inline int xf_ge_s(xf a, double x) {
    double o0, o1; int32_t e; xr_coexp_r(a.m, a.e, x, 0, &o0, &o1, &e); return o0 >= o1;
}
static inline int xf_le_s(xf a, double x) {
    double o0, o1; int32_t e; xr_coexp_r(a.m, a.e, x, 0, &o0, &o1, &e); return o0 <= o1;
}
static inline int xf_le(xf a, xf b) {
    double o0, o1; int32_t e; xr_coexp_r(a.m, a.e, b.m, b.e, &o0, &o1, &e); return o0 <= o1;
}
/* numba_xr.py:802-829 to_standard */
static inline cplx xr_to_std(xc a) {
    int32_t ere, eim; double nre = xr_norm_real(a.re, a.e, &ere);
    double nim = xr_norm_real(a.im, a.e, &eim);
    double cr, ci; int32_t ce; xr_coexp_r(nre, ere, nim, eim, &cr, &ci, &ce);
    return rmul(ldexp(1., ce), C(cr, ci));
}
static inline double xf_to_std(xf a) { return ldexp(a.m, a.e); }

/* ------------------------------------------------------------------------- */
/* Exported Xrange kernels (checked against numpy / mpmath in tests)          */
/* op: 0 add, 1 mul, 2 abs2(a) -> real, 3 to_standard(a), 4 a + std(b)        */
/* ------------------------------------------------------------------------- */
EXPORT void orc_xr_binop(int op, int64_t n,
                         const double *are, const double *aim, const int32_t *ae,
                         const double *bre, const double *bim, const int32_t *be,
                         double *ore, double *oim, int32_t *oe) {
    for (int64_t i = 0; i < n; i++) {
        xc a = {are[i], aim[i], ae[i]}, b = {bre[i], bim[i], be[i]}, r = {0., 0., 0};
        switch (op) {
        case 0: r = xr_add(a, b); break;
        case 1: r = xr_mul(a, b); break;
        case 2: { xf q = xr_abs2(a); r.re = q.m; r.im = 0.; r.e = q.e; } break;
        case 3: { cplx s = xr_to_std(a); r.re = s.re; r.im = s.im; r.e = 0; } break;
        case 4: r = xr_add_s(a, C(bre[i], bim[i])); break;
        case 5: r = xr_from_c(C(are[i], aim[i])); break;
        default: break;
        }
        ore[i] = r.re; oim[i] = r.im; oe[i] = r.e;
    }
}

/* ========================================================================= */
/* Standard (non-perturbation) loops                                         */
/* ========================================================================= */

/* core.py:3161-3194 c_from_pix with a Cartesian projection (identity f)     */
static inline cplx c_from_pix(cplx pix, const double *lin_mat, double dx, cplx center) {
    double x1 = lin_mat[0] * pix.re + lin_mat[1] * pix.im;
    double y1 = lin_mat[2] * pix.re + lin_mat[3] * pix.im;
    return cadd(center, rmul(dx, C(x1, y1)));
}

/*
 * Standard power-2 Mandelbrot: core.py:2935-2963 numba_cycles,
 * core.py:2965-3004 numba_iterate, models/mandelbrot_M2.py:309-334 iterate_once.
 * Z codes: zn = 0, dzndz = 1, dzndc = 2 (mandelbrot_M2.py:107-111).
 */
/* Orbit snapshots of calc_orbit (core.py:2965-3004 numba_iterate,
 * perturbation.py:1096-1101, 1265-1273, 1389-1396): every time n // backshift
 * grows, the two last snapshots shift; at exit the older one is iterated
 * forward to iteration n - backshift. */
typedef struct { int64_t div_shift, i1, i2; cplx z1, z2; } orbit_snap;
static inline void snap_init(orbit_snap *s, cplx z0) {
    s->div_shift = 0; s->i1 = 0; s->i2 = 0; s->z1 = z0; s->z2 = z0;
}
static inline void snap_take(orbit_snap *s, int64_t n, int64_t backshift, cplx z) {
    int64_t div = n / backshift;
    if (div > s->div_shift) { s->div_shift = div; s->i2 = s->i1; s->z2 = s->z1; s->i1 = n; s->z1 = z; }
}

/* Burning Ship maps, models/burning_ship.py:82-123 BS_iterate (xn ** 2 as
 * xn * xn, the lowering numba applies) */
static inline void bs_iterate(int flavor, double X, double Y, double a, double b,
                              double *nX, double *nY) {
    switch (flavor) {
    case 1: *nX = X * X - Y * Y + a; *nY = 2. * fabs(X * Y) - b; break;
    case 2: *nX = X * X - Y * Y + a; *nY = 2. * X * fabs(Y) - b; break;
    case 3: *nX = X * X - Y * fabs(Y) + a; *nY = 2. * X * Y - b; break;
    case 4: *nX = fabs(X * X - Y * Y) + a; *nY = 2. * X * Y - b; break;
    default: *nX = fabs(X * X - Y * Y) + a; *nY = 2. * fabs(X * Y) - b; break;
    }
}

EXPORT int orc_std_m2(int64_t npts, const double *pix, double cx, double cy,
                      const double *lin_mat, double dx, int64_t max_iter,
                      double M2, double eps2, double *Z, int32_t *stop_iter,
                      int8_t *stop_reason, int32_t nZ, int32_t calc_d2, int32_t backshift) {
    /* Z rows: zn, dzndz, dzndc, [d2zndc2], [zn_orbit] (mandelbrot_M2.py:107-124) */
    cplx *Zc = (cplx *)Z;
    const int64_t i_d2 = 3, i_orb = 3 + (calc_d2 ? 1 : 0);
    for (int64_t i = 0; i < npts; i++) {
        cplx c = c_from_pix(C(pix[2 * i], pix[2 * i + 1]), lin_mat, dx, C(cx, cy));
        cplx zn = Zc[i], dzndz = Zc[npts + i], dzndc = Zc[2 * npts + i];
        cplx d2 = calc_d2 ? Zc[i_d2 * npts + i] : C(0., 0.);
        orbit_snap S; snap_init(&S, zn);
        int64_t n = 0; int8_t reason = -1;
        for (;;) {
            n += 1;
            int ret = 1;
            if (n >= max_iter) { reason = 0; goto snap; }                    /* :312-314 */
            if (calc_d2)                                                      /* :316-317 */
                d2 = rmul(2., cadd(cmul(d2, zn), cmul(dzndc, dzndc)));
            dzndc = caddr(cmul(rmul(2., dzndc), zn), 1.);                     /* :319 */
            dzndz = cmul(rmul(2., dzndz), zn);                                /* :320 */
            zn = cadd(cmul(zn, zn), c);                                       /* :321 */
            if (n == 1) dzndz = C(1., 0.);                                    /* :323-324 */
            if (zn.re * zn.re + zn.im * zn.im > M2) { reason = 1; goto snap; } /* :326-328 */
            if (dzndz.re * dzndz.re + dzndz.im * dzndz.im < eps2) { reason = 2; goto snap; }
            ret = 0;
        snap:
            if (backshift > 0) snap_take(&S, n, backshift, zn);               /* core.py:2984-2991 */
            if (ret) break;
        }
        Zc[i] = zn; Zc[npts + i] = dzndz; Zc[2 * npts + i] = dzndc;
        if (calc_d2) Zc[i_d2 * npts + i] = d2;
        if (backshift > 0 && i_orb < nZ) {                                    /* core.py:2996-3001 */
            cplx zo = S.z2;
            while (S.i2 < n - backshift) { zo = cadd(cmul(zo, zo), c); S.i2 += 1; }
            Zc[i_orb * npts + i] = zo;
        }
        stop_iter[i] = (int32_t)n; stop_reason[i] = reason;
    }
    return 0;
}

/* models/burning_ship.py:12-17 sgn (0 maps to +1) */
static inline double sgn(double x) { return x < 0. ? -1. : 1.; }

/* ------------------------------------------------------------------------- */
/* Power-n Mandelbrot (models/mandelbrot_Mn.py).  nexp = 0 selects the power-2 */
/* model's own closures (models/mandelbrot_M2.py), nexp >= 2 the Mn ones.      */
/* ------------------------------------------------------------------------- */
/* integer power of a complex as numpy's npy_cpow does for |n| < 100 (the
 * reference's `zn ** deg_m1` on complex128 values): n = 1, 2, 3 directly,
 * else binary powering from 1 */
static inline cplx mn_ipow(cplx a, int n) {
    if (n == 1) return a;
    if (n == 2) return cmul(a, a);
    if (n == 3) return cmul(a, cmul(a, a));
    cplx aa = C(1., 0.), p = a;
    int mask = 1;
    for (;;) {
        if (n & mask) aa = cmul(aa, p);
        mask <<= 1;
        if (n < mask || mask <= 0) break;
        p = cmul(p, p);
    }
    return aa;
}
/* mandelbrot_Mn.py:645-652 dfdz = n z^(n-1) (products from z), M2: 2 z */
static inline cplx mn_dfdz_c(int nexp, cplx z) {
    if (nexp == 0) return rmul(2., z);
    cplx t = z;
    for (int k = 2; k < nexp; k++) t = cmul(t, z);
    return rmul((double)nexp, t);
}
/* binomial coefficients C(n, k) as float64 (mandelbrot_Mn.py:636-640) */
static inline void mn_binom(int n, double *Cb) {
    for (int k = 0; k <= n; k++) {
        double v = 1.;
        for (int j = 1; j <= k; j++) v = v * (double)(n - k + j) / (double)j;
        Cb[k] = v;
    }
}
/* mandelbrot_Mn.py:660-672 p_iter_zn */
static inline cplx mn_p_zn(int n, const double *Cb, cplx z, cplx ref, cplx c) {
    cplx tmp = cmul(z, cadd(z, rmul(Cb[1], ref)));
    cplx pk = ref;
    for (int k = 2; k < n; k++) { pk = cmul(pk, ref); tmp = cmul(z, cadd(tmp, rmul(Cb[k], pk))); }
    return cadd(tmp, c);
}
/* mandelbrot_Mn.py:674-733 p_iter_dzndz / p_iter_dzndc (same expansion) */
static inline cplx mn_p_deriv(int n, const double *Cb, cplx z, cplx d, cplx ref, cplx rd) {
    cplx mul = cadd(z, rmul(Cb[1], ref));
    cplx tmp = cmul(z, mul);
    cplx dt = cadd(cmul(d, mul), cmul(z, cadd(d, rmul(Cb[1], rd))));
    cplx pk = ref;
    for (int k = 2; k < n; k++) {
        cplx dpk = cmul(rmul((double)k, pk), rd);
        pk = cmul(pk, ref);
        mul = cadd(tmp, rmul(Cb[k], pk));
        dt = cadd(cmul(d, mul), cmul(z, cadd(dt, rmul(Cb[k], dpk))));
        tmp = cmul(z, mul);
    }
    return dt;
}

/* the same closures on Xrange values (the reference's Xrange branch) */
static inline xc mn_dfdz_x(int nexp, xc z) {
    if (nexp == 0) return xr_mul_r(2., z);
    xc t = z;
    for (int k = 2; k < nexp; k++) t = xr_mul(t, z);
    return xr_mul_r((double)nexp, t);
}
static inline xc mn_p_zn_x(int n, const double *Cb, xc z, xc ref, xc c) {
    xc tmp = xr_mul(z, xr_add(z, xr_mul_r(Cb[1], ref)));
    xc pk = ref;
    for (int k = 2; k < n; k++) { pk = xr_mul(pk, ref); tmp = xr_mul(z, xr_add(tmp, xr_mul_r(Cb[k], pk))); }
    return xr_add(tmp, c);
}
static inline xc mn_p_deriv_x(int n, const double *Cb, xc z, xc d, xc ref, xc rd) {
    xc mul = xr_add(z, xr_mul_r(Cb[1], ref));
    xc tmp = xr_mul(z, mul);
    xc dt = xr_add(xr_mul(d, mul), xr_mul(z, xr_add(d, xr_mul_r(Cb[1], rd))));
    xc pk = ref;
    for (int k = 2; k < n; k++) {
        xc dpk = xr_mul(xr_mul_r((double)k, pk), rd);
        pk = xr_mul(pk, ref);
        mul = xr_add(tmp, xr_mul_r(Cb[k], pk));
        dt = xr_add(xr_mul(d, mul), xr_mul(z, xr_add(dt, xr_mul_r(Cb[k], dpk))));
        tmp = xr_mul(z, mul);
    }
    return dt;
}

/*
 * Standard power-n Mandelbrot: core.py:2935-3004 numba_cycles / numba_iterate
 * with models/mandelbrot_Mn.py:317-355 iterate_once (calc_d2zndc2 False).
 */
EXPORT int orc_std_mn(int64_t npts, const double *pix, double cx, double cy,
                      const double *lin_mat, double dx, int64_t max_iter,
                      double M2, double eps2, int32_t nexp, double *Z, int32_t *stop_iter,
                      int8_t *stop_reason, int32_t nZ, int32_t calc_d2, int32_t backshift) {
    /* Z rows: zn, dzndz, dzndc, [d2zndc2], [zn_orbit] (mandelbrot_Mn.py:104-124) */
    cplx *Zc = (cplx *)Z;
    const double deg = (double)nexp;
    const int64_t i_d2 = 3, i_orb = 3 + (calc_d2 ? 1 : 0);
    for (int64_t i = 0; i < npts; i++) {
        cplx c = c_from_pix(C(pix[2 * i], pix[2 * i + 1]), lin_mat, dx, C(cx, cy));
        cplx zn = Zc[i], dzndz = Zc[npts + i], dzndc = Zc[2 * npts + i];
        cplx d2 = calc_d2 ? Zc[i_d2 * npts + i] : C(0., 0.);
        orbit_snap S; snap_init(&S, zn);
        int64_t n = 0; int8_t reason = -1;
        for (;;) {
            n += 1;
            int ret = 1;
            if (n >= max_iter) { reason = 0; goto snap; }
            cplx zm1, zm;
            if (calc_d2) {                                  /* mandelbrot_Mn.py:325-333 */
                cplx zm2 = mn_ipow(zn, nexp - 2);
                zm1 = cmul(zm2, zn);
                zm = cmul(zm1, zn);
                /* the reference multiplies by dzndz here, not by dzndc */
                d2 = rmul(deg, cadd(cmul(d2, zm1),
                                    cmul(cmul(rmul((double)(nexp - 1), dzndz), dzndc), zm2)));
            } else {
                zm1 = mn_ipow(zn, nexp - 1);
                zm = cmul(zm1, zn);
            }
            dzndc = caddr(cmul(rmul(deg, dzndc), zm1), 1.);
            dzndz = cmul(rmul(deg, dzndz), zm1);
            zn = cadd(zm, c);
            if (n == 1) dzndz = C(1., 0.);
            if (zn.re * zn.re + zn.im * zn.im > M2) { reason = 1; goto snap; }
            if (dzndz.re * dzndz.re + dzndz.im * dzndz.im < eps2) { reason = 2; goto snap; }
            ret = 0;
        snap:
            if (backshift > 0) snap_take(&S, n, backshift, zn);
            if (ret) break;
        }
        Zc[i] = zn; Zc[npts + i] = dzndz; Zc[2 * npts + i] = dzndc;
        if (calc_d2) Zc[i_d2 * npts + i] = d2;
        if (backshift > 0 && i_orb < nZ) {
            /* Mn_iterate (mandelbrot_Mn.py:13-17): zn ** n + c */
            cplx zo = S.z2;
            while (S.i2 < n - backshift) { zo = cadd(mn_ipow(zo, nexp), c); S.i2 += 1; }
            Zc[i_orb * npts + i] = zo;
        }
        stop_iter[i] = (int32_t)n; stop_reason[i] = reason;
    }
    return 0;
}


/*
 * Standard Burning Ship family: core.py:3007-3056 numba_iterate_BS,
 * models/burning_ship.py:350-423 iterate_once (flavors 1..5).
 * Z codes (float64): xn, yn, dxnda, dxndb, dynda, dyndb (burning_ship.py:283-289).
 */
EXPORT int orc_std_bs(int64_t npts, const double *pix, double cx, double cy,
                      const double *lin_mat, double dx, int32_t flavor,
                      int64_t max_iter, double M2, double *Z, int32_t *stop_iter,
                      int8_t *stop_reason, int32_t nZ, int32_t backshift) {
    /* Z rows: xn, yn, dxnda, dxndb, dynda, dyndb, [xn_orbit, yn_orbit]
     * (burning_ship.py:264-289); orbit snapshots core.py:3016-3047 */
    for (int64_t i = 0; i < npts; i++) {
        cplx c = c_from_pix(C(pix[2 * i], pix[2 * i + 1]), lin_mat, dx, C(cx, cy));
        double a = c.re, b = c.im;
        double X = Z[i], Y = Z[npts + i];
        double dXdA = Z[2 * npts + i], dXdB = Z[3 * npts + i];
        double dYdA = Z[4 * npts + i], dYdB = Z[5 * npts + i];
        orbit_snap S; snap_init(&S, C(X, Y));
        int64_t n = 0; int8_t reason = -1;
        for (;;) {
            n += 1;
            if (n >= max_iter) {
                reason = 0;
                if (backshift > 0) snap_take(&S, n, backshift, C(X, Y));
                break;
            }
            double nX, nY, ndXdA, ndXdB, ndYdA, ndYdB;
            switch (flavor) {
            case 1: /* burning_ship.py:383-390 */
                nX = X * X - Y * Y + a;
                nY = 2. * fabs(X * Y) - b;
                ndXdA = 2 * (X * dXdA - Y * dYdA) + 1.;
                ndXdB = 2 * (X * dXdB - Y * dYdB);
                ndYdA = 2 * (fabs(X) * sgn(Y) * dYdA + sgn(X) * dXdA * fabs(Y));
                ndYdB = 2 * (fabs(X) * sgn(Y) * dYdB + sgn(X) * dXdB * fabs(Y)) - 1.;
                break;
            case 2: /* :392-399 */
                nX = X * X - Y * Y + a;
                nY = 2. * X * fabs(Y) - b;
                ndXdA = 2 * (X * dXdA - Y * dYdA) + 1.;
                ndXdB = 2 * (X * dXdB - Y * dYdB);
                ndYdA = 2 * (X * sgn(Y) * dYdA + dXdA * fabs(Y));
                ndYdB = 2 * (X * sgn(Y) * dYdB + dXdB * fabs(Y)) - 1.;
                break;
            case 3: /* :401-408 */
                nX = X * X - Y * fabs(Y) + a;
                nY = 2. * X * Y - b;
                ndXdA = 2 * (X * dXdA - fabs(Y) * dYdA) + 1.;
                ndXdB = 2 * (X * dXdB - fabs(Y) * dYdB);
                ndYdA = 2. * (dXdA * Y + X * dYdA);
                ndYdB = 2. * (dXdB * Y + X * dYdB) - 1.;
                break;
            case 4: { /* :410-418 */
                double x2my2 = X * X - Y * Y;
                nX = fabs(x2my2) + a;
                nY = 2. * X * Y - b;
                ndXdA = 2. * sgn(x2my2) * (X * dXdA - Y * dYdA);
                ndXdB = 2. * sgn(x2my2) * (X * dXdB - Y * dYdB);
                ndYdA = 2. * (dXdA * Y + X * dYdA);
                ndYdB = 2. * (dXdB * Y + X * dYdB) - 1.;
            } break;
            default: { /* 5, :420-428 */
                double x2my2 = X * X - Y * Y;
                nX = fabs(x2my2) + a;
                nY = 2. * fabs(X * Y) - b;
                ndXdA = 2. * sgn(x2my2) * (X * dXdA - Y * dYdA);
                ndXdB = 2. * sgn(x2my2) * (X * dXdB - Y * dYdB);
                ndYdA = 2. * (fabs(X) * sgn(Y) * dYdA + sgn(X) * dXdA * fabs(Y));
                ndYdB = 2. * (fabs(X) * sgn(Y) * dYdB + sgn(X) * dXdB * fabs(Y)) - 1.;
            } break;
            }
            X = nX; Y = nY; dXdA = ndXdA; dXdB = ndXdB; dYdA = ndYdA; dYdB = ndYdB;
            int esc = X * X + Y * Y > M2;                                   /* :431-433 */
            if (backshift > 0) snap_take(&S, n, backshift, C(X, Y));
            if (esc) { reason = 1; break; }
        }
        Z[i] = X; Z[npts + i] = Y; Z[2 * npts + i] = dXdA; Z[3 * npts + i] = dXdB;
        Z[4 * npts + i] = dYdA; Z[5 * npts + i] = dYdB;
        if (backshift > 0 && nZ >= 8) {
            double xo = S.z2.re, yo = S.z2.im;
            while (S.i2 < n - backshift) {
                double nx_, ny_;
                bs_iterate(flavor, xo, yo, a, b, &nx_, &ny_);
                xo = nx_; yo = ny_; S.i2 += 1;
            }
            Z[6 * npts + i] = xo; Z[7 * npts + i] = yo;
        }
        stop_iter[i] = (int32_t)n; stop_reason[i] = reason;
    }
    return 0;
}

/* ========================================================================= */
/* Reference-orbit derived data: BLA tree and derivative paths               */
/* ========================================================================= */
#define STG_COMPRESSED 3    /* settings.py:40 BLA_compression, perturbation.py:985 */

/* perturbation.py:2108-2114 BLA_index */
static inline int64_t bla_index(int64_t i, int stg) { return 2 * i + (((int64_t)1 << stg) - 1); }

/* perturbation.py:1976-1981 _stages_bla: ceil(log2(len)) */
EXPORT int32_t orc_stages_bla(int64_t len) { return (int32_t)ceil(log2((double)len)); }

/* perturbation.py:1983-2024 combine_BLA (M is complex [.., 2]) */
static void combine_bla(cplx *M, double *r, double kc, int stg, int64_t len, double eps) {
    int64_t step = (int64_t)1 << stg;
    for (int64_t i = 0; i < len - step + 1; i += step) {
        int64_t ii = i + step / 2;
        if (ii >= len) break;
        int64_t i1 = bla_index(i, stg - 1), i2 = bla_index(ii, stg - 1), ir = bla_index(i, stg);
        M[2 * ir] = cmul(M[2 * i2], M[2 * i1]);
        M[2 * ir + 1] = cadd(cmul(M[2 * i2], M[2 * i1 + 1]), M[2 * i2 + 1]);
        double r1 = r[i1], r2 = r[i2];
        double mA1 = hypot(M[2 * i1].re, M[2 * i1].im), mB1 = hypot(M[2 * i1 + 1].re, M[2 * i1 + 1].im);
        /* Python max(a, b) / min(a, b) semantics: the first argument wins ties */
        double num = r2 - mB1 * kc, den = (eps > mA1) ? eps : mA1;
        double q = num / den; double r2b = 0.95 * ((q > 0.) ? q : 0.);
        r[ir] = (r2b < r1) ? r2b : r1;
    }
}

/*
 * perturbation.py:1819-1881 numba_make_BLA, M2 (dfdz(z) = 2z,
 * models/mandelbrot_M2.py:595-597).  Output: M complex [2L][2] (A, B),
 * r [2L] with L = len // 8.  Returns stages.
 */
EXPORT int32_t orc_make_bla_m2(const double *Zn, int64_t len, double kc, double eps,
                               double *M_out, double *r_out, int32_t nexp) {
    const int64_t kcomp = 1 << STG_COMPRESSED;
    int64_t L = len / kcomp;
    cplx *M = (cplx *)M_out;
    memset(M_out, 0, sizeof(double) * 2 * 2 * 2 * L);
    memset(r_out, 0, sizeof(double) * 2 * L);
    cplx tM[2 * 8 * 2]; double tr[2 * 8];
    for (int64_t i = 0; i < L; i++) {
        memset(tM, 0, sizeof(tM)); memset(tr, 0, sizeof(tr));
        for (int64_t j = 0; j < kcomp; j++) {
            cplx z = C(Zn[2 * (i * kcomp + j)], Zn[2 * (i * kcomp + j) + 1]);
            tM[2 * (2 * j)] = mn_dfdz_c(nexp, z);
            tM[2 * (2 * j) + 1] = C(1., 0.);
            tr[2 * j] = eps * hypot(tM[2 * (2 * j)].re, tM[2 * (2 * j)].im);
        }
        for (int stg = 1; stg <= STG_COMPRESSED; stg++) combine_bla(tM, tr, kc, stg, kcomp, eps);
        M[2 * (2 * i)] = tM[2 * (kcomp - 1)];
        M[2 * (2 * i) + 1] = tM[2 * (kcomp - 1) + 1];
        r_out[2 * i] = tr[kcomp - 1];
    }
    int32_t stages = orc_stages_bla(len);
    for (int stg = 1; stg < stages - STG_COMPRESSED; stg++) combine_bla(M, r_out, kc, stg, L, eps);
    return stages;
}

/* models/burning_ship.py:441-532 partial derivatives of the BS maps */
static inline void bs_dfdxy(int flavor, double x, double y, double *fxx, double *fxy, double *fyx, double *fyy) {
    switch (flavor) {
    case 1: *fxx = 2. * x; *fxy = -2. * y; *fyx = 2. * sgn(x) * fabs(y); *fyy = 2. * sgn(y) * fabs(x); break;
    case 2: *fxx = 2. * x; *fxy = -2. * y; *fyx = 2. * fabs(y); *fyy = 2. * sgn(y) * x; break;
    case 3: *fxx = 2. * x; *fxy = -2. * fabs(y); *fyx = 2. * y; *fyy = 2. * x; break;
    case 4: { double q = x * x - y * y; *fxx = 2. * sgn(q) * x; *fxy = -2. * sgn(q) * y; *fyx = 2. * y; *fyy = 2. * x; } break;
    default: { double q = x * x - y * y; *fxx = 2. * sgn(q) * x; *fxy = -2. * sgn(q) * y;
               *fyx = 2. * sgn(x) * fabs(y); *fyy = 2. * sgn(y) * fabs(x); } break;
    }
}

/* perturbation.py:2027-2105 combine_BLA_BS (M is float64 [.., 8]) */
static void combine_bla_bs(double *M, double *r, double kc, int stg, int64_t len, double eps) {
    int64_t step = (int64_t)1 << stg;
    for (int64_t i = 0; i < len - step + 1; i += step) {
        int64_t ii = i + step / 2;
        if (ii >= len) break;
        int64_t i1 = bla_index(i, stg - 1), i2 = bla_index(ii, stg - 1), ir = bla_index(i, stg);
        double *m1 = M + 8 * i1, *m2 = M + 8 * i2, *mr = M + 8 * ir;
        mr[0] = m2[0] * m1[0] + m2[1] * m1[2];
        mr[1] = m2[0] * m1[1] + m2[1] * m1[3];
        mr[2] = m2[2] * m1[0] + m2[3] * m1[2];
        mr[3] = m2[2] * m1[1] + m2[3] * m1[3];
        mr[4] = m2[0] * m1[4] + m2[1] * m1[6] + m2[4];
        mr[5] = m2[0] * m1[5] + m2[1] * m1[7] + m2[5];
        mr[6] = m2[2] * m1[4] + m2[3] * m1[6] + m2[6];
        mr[7] = m2[2] * m1[5] + m2[3] * m1[7] + m2[7];
        double r1 = r[i1], r2 = r[i2];
        double mA1 = fmax(fmax(fabs(m1[0]), fabs(m1[1])), fmax(fabs(m1[2]), fabs(m1[3])));
        double mB1 = fmax(fmax(fabs(m1[4]), fabs(m1[5])), fmax(fabs(m1[6]), fabs(m1[7])));
        /* Python max(a, b) / min(a, b) semantics: the first argument wins ties */
        double num = r2 - mB1 * kc, den = (eps > mA1) ? eps : mA1;
        double q = num / den; double r2b = 0.95 * ((q > 0.) ? q : 0.);
        r[ir] = (r2b < r1) ? r2b : r1;
    }
}

/* perturbation.py:1884-1973 numba_make_BLA_BS. M: float64 [2L][8], r [2L] */
EXPORT int32_t orc_make_bla_bs(const double *Zn, int64_t len, int32_t flavor, double kc,
                               double eps, double *M, double *r_out) {
    const int64_t kcomp = 1 << STG_COMPRESSED;
    int64_t L = len / kcomp;
    memset(M, 0, sizeof(double) * 8 * 2 * L);
    memset(r_out, 0, sizeof(double) * 2 * L);
    double tM[2 * 8 * 8]; double tr[2 * 8];
    for (int64_t i = 0; i < L; i++) {
        memset(tM, 0, sizeof(tM)); memset(tr, 0, sizeof(tr));
        for (int64_t j = 0; j < kcomp; j++) {
            double x = Zn[2 * (i * kcomp + j)], y = Zn[2 * (i * kcomp + j) + 1];
            double *t = tM + 8 * (2 * j);
            bs_dfdxy(flavor, x, y, &t[0], &t[1], &t[2], &t[3]);
            t[4] = 1.; t[5] = 0.; t[6] = 0.; t[7] = -1.;
            tr[2 * j] = eps * fmin(fabs(x), fabs(y));
        }
        for (int stg = 1; stg <= STG_COMPRESSED; stg++) combine_bla_bs(tM, tr, kc, stg, kcomp, eps);
        memcpy(M + 8 * (2 * i), tM + 8 * (kcomp - 1), 8 * sizeof(double));
        r_out[2 * i] = tr[kcomp - 1];
    }
    int32_t stages = orc_stages_bla(len);
    for (int stg = 1; stg < stages - STG_COMPRESSED; stg++) combine_bla_bs(M, r_out, kc, stg, L, eps);
    return stages;
}

/*
 * perturbation.py:2116-2170 ref_BLA_get.  Returns the step (0 if no BLA
 * applies) and the index of the entry in the table through *idx.
 */
static inline int64_t bla_get(const double *r_bla, int32_t stages_bla, double abs_zn,
                              int64_t n_iter, int64_t first_invalid, int64_t *idx) {
    int64_t it = n_iter >> STG_COMPRESSED;
    int stages = STG_COMPRESSED;
    for (int s = STG_COMPRESSED; s < stages_bla; s++) {
        stages = s;
        if (it & 1) break;
        it >>= 1;
    }
    int64_t invalid_step = first_invalid - n_iter;
    for (int stg = stages; stg >= STG_COMPRESSED; stg--) {
        int64_t step = (int64_t)1 << stg;
        if (step >= invalid_step) continue;
        int64_t ib = bla_index(n_iter >> STG_COMPRESSED, stg - STG_COMPRESSED);
        if (abs_zn < r_bla[ib]) { *idx = ib; return step; }
    }
    return 0;
}

/* Sparse Xrange side table of the orbit: perturbation.py:2519-2588 ref_path_get.
 * The cursor in the reference is an optimisation of a membership lookup in the
 * sorted index list; the lookup result is identical. */
typedef struct {
    int32_t n; const int32_t *idx; const double *re, *im; const int32_t *e;
} xr_table;
static inline int xr_lookup(const xr_table *t, int64_t w, xc *out) {
    int lo = 0, hi = t->n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (t->idx[mid] == w) { out->re = t->re[mid]; out->im = t->im[mid]; out->e = t->e[mid]; return 1; }
        if (t->idx[mid] < w) lo = mid + 1; else hi = mid - 1;
    }
    return 0;
}

/*
 * perturbation.py:2282-2336 numba_dZndc_path (M2, dfdz = 2z).
 * Standard form: out complex [len].  Xrange form: out_re/out_im/out_e [len].
 * scale: dx * projection.scale as a float64 Xrange (perturbation.py:459-468).
 */
EXPORT void orc_dzndc_path_m2(const double *Zn, int64_t len, int64_t ref_div_iter,
                              int64_t ref_order, int32_t xr_mode,
                              int32_t n_xr, const int32_t *xr_idx, const double *xr_re,
                              const double *xr_im, const int32_t *xr_e,
                              double scale_m, int32_t scale_e,
                              double *out_std, double *out_re, double *out_im, int32_t *out_e,
                              int32_t nexp) {
    int64_t valid = len < ref_div_iter ? len : ref_div_iter;
    xr_table t = {n_xr, xr_idx, xr_re, xr_im, xr_e};
    int has_xr = n_xr > 0;
    int64_t i = 0;
    if (xr_mode) {
        xf scale = {scale_m, scale_e};
        for (int64_t k = 0; k < len; k++) { out_re[k] = 0.; out_im[k] = 0.; out_e[k] = 0; }
        for (i = 1; i < valid; i++) {
            xc zx; cplx zs = C(Zn[2 * (i - 1)], Zn[2 * (i - 1) + 1]);
            if (!(has_xr && xr_lookup(&t, i - 1, &zx))) zx = xr_from_c(zs);
            xc prev = {out_re[i - 1], out_im[i - 1], out_e[i - 1]};
            xc v = xr_add_xf(xr_mul(mn_dfdz_x(nexp, zx), prev), scale);
            out_re[i] = v.re; out_im[i] = v.im; out_e[i] = v.e;
        }
        i -= 1;
        if (i == ref_order - 1) {
            /* the wrapped value uses the standard orbit value (perturbation.py:2320) */
            cplx zs = C(Zn[2 * i], Zn[2 * i + 1]);
            xc prev = {out_re[i], out_im[i], out_e[i]};
            xc v = xr_add_xf(xr_mul_s(mn_dfdz_c(nexp, zs), prev), scale);
            out_re[0] = v.re; out_im[0] = v.im; out_e[0] = v.e;
        }
    } else {
        double scale = ldexp(scale_m, scale_e);
        cplx *o = (cplx *)out_std;
        for (int64_t k = 0; k < len; k++) o[k] = C(0., 0.);
        for (i = 1; i < valid; i++)
            o[i] = caddr(cmul(mn_dfdz_c(nexp, C(Zn[2 * (i - 1)], Zn[2 * (i - 1) + 1])), o[i - 1]), scale);
        i -= 1;
        if (i == ref_order - 1)
            o[0] = caddr(cmul(mn_dfdz_c(nexp, C(Zn[2 * i], Zn[2 * i + 1])), o[i]), scale);
    }
}

/* perturbation.py:2466-2516 numba_dZndz_path (M2).  Output length len + 1. */
EXPORT void orc_dzndz_path_m2(const double *Zn, int64_t len, int64_t ref_div_iter,
                              int32_t xr_mode, int32_t n_xr, const int32_t *xr_idx,
                              const double *xr_re, const double *xr_im, const int32_t *xr_e,
                              double *out_std, double *out_re, double *out_im, int32_t *out_e,
                              int32_t nexp) {
    int64_t valid = len < ref_div_iter ? len : ref_div_iter;
    xr_table t = {n_xr, xr_idx, xr_re, xr_im, xr_e};
    int has_xr = n_xr > 0;
    int64_t i;
    if (xr_mode) {
        for (int64_t k = 0; k <= len; k++) { out_re[k] = 0.; out_im[k] = 0.; out_e[k] = 0; }
        out_re[1] = 1.; out_e[1] = 0;
        for (i = 2; i < valid; i++) {
            xc zx; cplx zs = C(Zn[2 * (i - 1)], Zn[2 * (i - 1) + 1]);
            if (!(has_xr && xr_lookup(&t, i - 1, &zx))) zx = xr_from_c(zs);
            xc prev = {out_re[i - 1], out_im[i - 1], out_e[i - 1]};
            xc v = xr_mul(mn_dfdz_x(nexp, zx), prev);
            out_re[i] = v.re; out_im[i] = v.im; out_e[i] = v.e;
        }
        i -= 1;
        xc zx; cplx zs = C(Zn[2 * i], Zn[2 * i + 1]);
        if (!(has_xr && xr_lookup(&t, i, &zx))) zx = xr_from_c(zs);
        xc prev = {out_re[i], out_im[i], out_e[i]};
        xc v = xr_mul(mn_dfdz_x(nexp, zx), prev);
        out_re[len] = v.re; out_im[len] = v.im; out_e[len] = v.e;
    } else {
        cplx *o = (cplx *)out_std;
        for (int64_t k = 0; k <= len; k++) o[k] = C(0., 0.);
        o[1] = C(1., 0.);
        for (i = 2; i < valid; i++)
            o[i] = cmul(mn_dfdz_c(nexp, C(Zn[2 * (i - 1)], Zn[2 * (i - 1) + 1])), o[i - 1]);
        i -= 1;
        o[len] = cmul(mn_dfdz_c(nexp, C(Zn[2 * i], Zn[2 * i + 1])), o[i]);
    }
}

/* perturbation.py:2339-2463 numba_dZndc_path_BS + incr_deriv_ref_BS, standard form.
 * out: 4 x float64 [len] (dXnda, dXndb, dYnda, dYndb) */
EXPORT void orc_dzndc_path_bs(const double *Zn, int64_t len, int64_t ref_div_iter,
                              int64_t ref_order, int32_t flavor, double scale,
                              double *dXa, double *dXb, double *dYa, double *dYb) {
    int64_t valid = len < ref_div_iter ? len : ref_div_iter;
    for (int64_t k = 0; k < len; k++) { dXa[k] = 0.; dXb[k] = 0.; dYa[k] = 0.; dYb[k] = 0.; }
    int64_t i;
    for (i = 1; i <= valid; i++) {
        int64_t from = i - 1, to = i;
        if (i == valid) {
            if (!(from == ref_order - 1)) break;
            to = 0;
        }
        double fxx, fxy, fyx, fyy;
        bs_dfdxy(flavor, Zn[2 * from], Zn[2 * from + 1], &fxx, &fxy, &fyx, &fyy);
        double a = dXa[from], b = dXb[from], c = dYa[from], d = dYb[from];
        dXa[to] = fxx * a + fxy * c + scale;
        dXb[to] = fxx * b + fxy * d;
        dYa[to] = fyx * a + fyy * c;
        dYb[to] = fyx * b + fyy * d - scale;
    }
}

/* ========================================================================= */
/* Perturbation loop, power-2 Mandelbrot                                      */
/* perturbation.py:988-1045 numba_cycles_perturb, :1048-1061 numba_initialize,*/
/* :1065-1400 numba_iterate; closures models/mandelbrot_M2.py:591-627.        */
/* ========================================================================= */
typedef struct {
    /* reference orbit (perturbation.py:317-375 get_path_data) */
    const double *Zn; int64_t ref_len; int64_t ref_div_iter; int64_t ref_order;
    int32_t n_xr; const int32_t *xr_idx; const double *xr_re; const double *xr_im; const int32_t *xr_e;
    /* derivative paths: standard (complex) or Xrange arrays */
    const double *dZndc; const double *dZndc_re; const double *dZndc_im; const int32_t *dZndc_e;
    const double *dZndz; const double *dZndz_re; const double *dZndz_im; const int32_t *dZndz_e;
    /* BLA table */
    const double *M_bla; const double *r_bla; int32_t stages_bla; int32_t bla_on;
    /* calc options */
    int64_t max_iter; double M2; double eps2; int32_t xr_mode;
    int32_t i_dzndz; int32_t i_dzndc; int32_t dzndz_carryover;
    /* pixel mapping (perturbation.py:2214-2230, 2666-2672) */
    double lin_mat[4]; double dx_m; int32_t dx_e; double drift_re; double drift_im; int32_t drift_e;
    /* 0: power-2 model (mandelbrot_M2.py closures); n >= 2: power-n (mandelbrot_Mn.py) */
    int32_t nexp;
    /* calc_orbit: snapshots every backshift iterations (0: off) into row i_znorbit */
    int32_t backshift; int32_t i_znorbit;
} orc_pm2_args;

static inline cplx path_c(const double *p, int64_t i) { return C(p[2 * i], p[2 * i + 1]); }
static inline xc path_x(const double *re, const double *im, const int32_t *e, int64_t i) {
    xc r = {re[i], im[i], e[i]}; return r;
}

/* perturbation.py:2214-2230 ref_path_c_from_pix (Cartesian) */
static inline xc pm_c_from_pix(cplx pix, const double *lin_mat, xf dx, xc drift) {
    double x1 = lin_mat[0] * pix.re + lin_mat[1] * pix.im;
    double y1 = lin_mat[2] * pix.re + lin_mat[3] * pix.im;
    return xr_add(xf_mul_c(dx, C(x1, y1)), drift);
}

EXPORT int orc_perturb_m2(const orc_pm2_args *P, int64_t npts, const double *pix,
                          double *Zout, int32_t nZ, int32_t *U, int8_t *stop_reason,
                          int32_t *stop_iter) {
    cplx *Zc = (cplx *)Zout;
    const int zn = 0, dzndz = P->i_dzndz, dzndc = P->i_dzndc;
    const int calc_dzndz = dzndz >= 0, calc_dzndc = dzndc >= 0;
    const int xr = P->xr_mode, bla = P->bla_on;
    const int64_t order = P->ref_order, div_iter = P->ref_div_iter, plen = P->ref_len;
    xr_table T = {P->n_xr, P->xr_idx, P->xr_re, P->xr_im, P->xr_e};
    const int has_xr = P->n_xr > 0;
    xf dxr = {P->dx_m, P->dx_e};
    xc drift = {P->drift_re, P->drift_im, P->drift_e};
    const xc xzero = {0., 0., 0};
    xc Zx[8]; for (int k = 0; k < 8; k++) Zx[k] = xzero;   /* per tile, :1012-1014 */
    int64_t first_invalid = plen;
    if (div_iter < first_invalid) first_invalid = div_iter;
    if (order < first_invalid) first_invalid = order;
    const int nexp = P->nexp;
    double Cb[64];
    if (nexp) mn_binom(nexp, Cb);
    for (int64_t ip = 0; ip < npts; ip++) {
        xc c_xr = pm_c_from_pix(C(pix[2 * ip], pix[2 * ip + 1]), P->lin_mat, dxr, drift);
        cplx c = xr_to_std(c_xr);
        cplx Z[8];
        for (int k = 0; k < nZ; k++) Z[k] = Zc[k * npts + ip];
        /* numba_initialize :1055-1060 */
        Zx[zn] = xr_from_c(Z[zn]);
        if (calc_dzndc) Zx[dzndc] = xr_from_c(Z[dzndc]);
        if (calc_dzndz) { Z[dzndz] = C(0., 0.); if (!P->dzndz_carryover) Zx[dzndz] = xzero; }

        int64_t w = 0, n = 0; int8_t stop = -1;
        int nullify = 0; int64_t w_wrapped = plen;   /* len(dZndz_path) - 1 */
        orbit_snap S; snap_init(&S, Z[zn]);          /* :1096-1101 */
        int dyn = 1;
        for (;;) {
            /* BLA step :1121-1154 */
            if (bla && (w & 7) == 0) {
                int64_t ib;
                int64_t step = bla_get(P->r_bla, P->stages_bla, hypot(Z[zn].re, Z[zn].im), w, first_invalid, &ib);
                if (step != 0) {
                    cplx A = path_c(P->M_bla, 2 * ib), B = path_c(P->M_bla, 2 * ib + 1);
                    n += step;
                    w = (w + step) % order;
                    if (xr) {
                        Zx[zn] = xr_add(xr_mul_s(A, Zx[zn]), xr_mul_s(B, c_xr));
                        Z[zn] = xr_to_std(Zx[zn]);
                        if (calc_dzndc) Zx[dzndc] = xr_mul_s(A, Zx[dzndc]);
                        if (calc_dzndz) Zx[dzndz] = xr_mul_s(A, Zx[dzndz]);
                    } else {
                        Z[zn] = cadd(cmul(A, Z[zn]), cmul(B, c));
                        if (calc_dzndc) Z[dzndc] = cmul(A, Z[dzndc]);
                        if (calc_dzndz) Z[dzndz] = cmul(A, Z[dzndz]);
                    }
                    continue;
                }
            }
            /* full perturbation step :1158-1214 */
            n += 1;
            cplx ref_zn = path_c(P->Zn, w);
            xc ref_zn_xr;
            if (xr) { if (!(has_xr && xr_lookup(&T, w, &ref_zn_xr))) ref_zn_xr = xr_from_c(ref_zn); }
            if (calc_dzndc) {
                if (xr) {
                    xc rd = dyn ? xzero : path_x(P->dZndc_re, P->dZndc_im, P->dZndc_e, w);
                    Zx[dzndc] = nexp ? mn_p_deriv_x(nexp, Cb, Zx[zn], Zx[dzndc], ref_zn_xr, rd)
                                     : xr_mul_r(2., xr_add(xr_mul(xr_add(ref_zn_xr, Zx[zn]), Zx[dzndc]), xr_mul(rd, Zx[zn])));
                } else {
                    cplx rd = path_c(P->dZndc, w);
                    if (dyn) rd = C(0., 0.);
                    Z[dzndc] = nexp ? mn_p_deriv(nexp, Cb, Z[zn], Z[dzndc], ref_zn, rd)
                                    : rmul(2., cadd(cmul(cadd(ref_zn, Z[zn]), Z[dzndc]), cmul(rd, Z[zn])));
                }
            }
            if (calc_dzndz) {
                int64_t k = nullify ? 0 : w;
                if (xr) {
                    xc rd = path_x(P->dZndz_re, P->dZndz_im, P->dZndz_e, k);
                    Zx[dzndz] = nexp ? mn_p_deriv_x(nexp, Cb, Zx[zn], Zx[dzndz], ref_zn_xr, rd)
                                     : xr_mul_r(2., xr_add(xr_mul(xr_add(ref_zn_xr, Zx[zn]), Zx[dzndz]), xr_mul(rd, Zx[zn])));
                } else {
                    cplx rd = path_c(P->dZndz, k);
                    Z[dzndz] = nexp ? mn_p_deriv(nexp, Cb, Z[zn], Z[dzndz], ref_zn, rd)
                                    : rmul(2., cadd(cmul(cadd(ref_zn, Z[zn]), Z[dzndz]), cmul(rd, Z[zn])));
                }
            }
            if (xr) {
                Zx[zn] = nexp ? mn_p_zn_x(nexp, Cb, Zx[zn], ref_zn_xr, c_xr)
                              : xr_add(xr_mul(Zx[zn], xr_add(Zx[zn], xr_mul_r(2., ref_zn_xr))), c_xr);
                Z[zn] = xr_to_std(Zx[zn]);
            } else {
                Z[zn] = nexp ? mn_p_zn(nexp, Cb, Z[zn], ref_zn, c)
                             : cadd(cmul(Z[zn], cadd(Z[zn], rmul(2., ref_zn))), c);
            }
            w += 1;
            if (w >= order) w = w % order;
            /* max_iter :1218-1220 */
            if (n >= P->max_iter) { stop = 0; break; }
            /* interior detection :1224-1246 */
            if (calc_dzndz) {
                int64_t k = nullify ? 0 : ((n == order) ? w_wrapped : w);
                int stat;
                if (xr) {
                    xc ZdZ = xr_add(Zx[dzndz], path_x(P->dZndz_re, P->dZndz_im, P->dZndz_e, k));
                    stat = xf_lt_s(xr_abs2(ZdZ), P->eps2);
                } else {
                    cplx ZdZ = cadd(Z[dzndz], path_c(P->dZndz, k));
                    stat = ZdZ.re * ZdZ.re + ZdZ.im * ZdZ.im < P->eps2;
                }
                if (stat) { stop = 2; break; }
            }
            /* divergence :1252-1279 */
            cplx ref_next = path_c(P->Zn, w);
            xc ref_next_xr = xzero; int next_is_xr = 0;
            if (xr && has_xr) next_is_xr = xr_lookup(&T, w, &ref_next_xr);
            cplx ZZ = cadd(Z[zn], ref_next);
            double sq = ZZ.re * ZZ.re + ZZ.im * ZZ.im;
            if (P->backshift > 0) snap_take(&S, n, P->backshift, ZZ);       /* :1265-1273 */
            if (sq > P->M2) { stop = 1; break; }
            /* rebase when the reference diverges :1283-1313 */
            if (w >= div_iter - 1) {
                Z[zn] = ZZ;
                if (xr) {
                    Zx[zn] = xr_from_c(ZZ);
                    if (calc_dzndc) Zx[dzndc] = xr_add(Zx[dzndc], path_x(P->dZndc_re, P->dZndc_im, P->dZndc_e, w));
                    if (calc_dzndz) {
                        if (!nullify) {
                            int64_t k = (n == order) ? w_wrapped : w;
                            Zx[dzndz] = xr_add(Zx[dzndz], path_x(P->dZndz_re, P->dZndz_im, P->dZndz_e, k));
                        }
                        nullify = 1;
                    }
                } else {
                    if (calc_dzndc) Z[dzndc] = cadd(Z[dzndc], path_c(P->dZndc, w));
                    if (calc_dzndz) {
                        if (!nullify) Z[dzndz] = cadd(Z[dzndz], path_c(P->dZndz, (n == order) ? w_wrapped : w));
                        nullify = 1;
                    }
                }
                w = 0;
                continue;
            }
            /* dynamic rebase (Zhuoran) :1317-1372 -- componentwise test */
            dyn = (fabs(ZZ.re) <= fabs(Z[zn].re)) && (fabs(ZZ.im) <= fabs(Z[zn].im));
            if (dyn) {
                if (xr) {
                    xc Zxn = Zx[zn];
                    xc ZZx = next_is_xr ? xr_add(Zxn, ref_next_xr) : xr_add_s(Zxn, ref_next);
                    if (xf_le(xr_abs2(ZZx), xr_abs2(Zxn))) {
                        Zx[zn] = ZZx;
                        Z[zn] = xr_to_std(ZZx);
                        if (calc_dzndc) Zx[dzndc] = xr_add(Zx[dzndc], path_x(P->dZndc_re, P->dZndc_im, P->dZndc_e, w));
                        if (calc_dzndz) {
                            if (!nullify) {
                                int64_t k = (n == order) ? w_wrapped : w;
                                Zx[dzndz] = xr_add(Zx[dzndz], path_x(P->dZndz_re, P->dZndz_im, P->dZndz_e, k));
                            }
                            nullify = 1;
                        }
                        w = 0;
                        continue;
                    }
                } else {
                    Z[zn] = ZZ;
                    if (calc_dzndc) Z[dzndc] = cadd(Z[dzndc], path_c(P->dZndc, w));
                    if (calc_dzndz) {
                        if (!nullify) Z[dzndz] = cadd(Z[dzndz], path_c(P->dZndz, (n == order) ? w_wrapped : w));
                        nullify = 1;
                    }
                    w = 0;
                    continue;
                }
            }
        }
        /* end of iterations :1375-1385 */
        U[ip] = (int32_t)w;
        if (xr) {
            Z[zn] = cadd(xr_to_std(Zx[zn]), path_c(P->Zn, w));
            if (calc_dzndc) Z[dzndc] = xr_to_std(xr_add(Zx[dzndc], path_x(P->dZndc_re, P->dZndc_im, P->dZndc_e, w)));
        } else {
            Z[zn] = cadd(Z[zn], path_c(P->Zn, w));
            if (calc_dzndc) Z[dzndc] = cadd(Z[dzndc], path_c(P->dZndc, w));
        }
        if (P->backshift > 0 && P->i_znorbit >= 0) {                          /* :1389-1396 */
            cplx CC = cadd(c, path_c(P->Zn, 1));
            cplx zo = S.z2;
            while (S.i2 < n - P->backshift) {
                zo = nexp ? cadd(mn_ipow(zo, nexp), CC) : cadd(cmul(zo, zo), CC);
                S.i2 += 1;
            }
            Z[P->i_znorbit] = zo;
        }
        for (int k = 0; k < nZ; k++) Zc[k * npts + ip] = Z[k];
        stop_iter[ip] = (int32_t)n; stop_reason[ip] = stop;
    }
    return 0;
}

/* ========================================================================= */
/* Perturbation loop, Burning Ship family (standard FP64 form)                */
/* perturbation.py:1406-1451 numba_cycles_perturb_BS, :1468-1791             */
/* numba_iterate_BS, :1793-1811 apply_BLA_BS; closures                        */
/* models/burning_ship.py:19-60, 535-859.                                     */
/* ========================================================================= */
/* burning_ship.py:19-32 diffabs: |X + x| - |X| */
static inline double diffabs(double X, double x) {
    if (X >= 0.) { if ((X + x) >= 0.) return 1. * x; else return -(2. * X + x); }
    else { if ((X + x) <= 0.) return -x; else return (2. * X + x); }
}
/* burning_ship.py:34-46 */
static inline double ddiffabsdX(double X, double x) {
    if (X >= 0.) { if ((X + x) >= 0.) return 0.; else return -2.; }
    else { if ((X + x) <= 0.) return 0.; else return 2.; }
}
/* burning_ship.py:48-60 */
static inline double ddiffabsdx(double X, double x) {
    if (X >= 0.) { if ((X + x) >= 0.) return 1.; else return -1.; }
    else { if ((X + x) <= 0.) return -1.; else return 1.; }
}

/* burning_ship.py:535-619 _p_iter_zn */
static inline void bs_p_iter_zn(int flavor, double *x, double *y, double X, double Y, double a, double b) {
    double nx, ny, xn = *x, yn = *y;
    switch (flavor) {
    case 1: {
        double ref_xyn = X * Y;
        nx = xn * (xn + 2. * X) - yn * (yn + 2. * Y) + a;
        ny = 2. * diffabs(ref_xyn, xn * yn + xn * Y + yn * X) - b;
    } break;
    case 2:
        nx = xn * (xn + 2. * X) - yn * (yn + 2. * Y) + a;
        ny = 2. * (X * diffabs(Y, yn) + xn * fabs(Y + yn)) - b;
        break;
    case 3:
        nx = xn * (xn + 2. * X) - Y * diffabs(Y, yn) - yn * fabs(Y + yn) + a;
        ny = 2. * (X * yn + Y * xn + xn * yn) - b;
        break;
    case 4: {
        double ref_x2my2 = X * X - Y * Y;
        nx = diffabs(ref_x2my2, xn * (xn + 2. * X) - yn * (yn + 2. * Y)) + a;
        ny = 2. * (X * yn + Y * xn + xn * yn) - b;
    } break;
    default: {
        double ref_xyn = X * Y, ref_x2my2 = X * X - Y * Y;
        nx = diffabs(ref_x2my2, xn * (xn + 2. * X) - yn * (yn + 2. * Y)) + a;
        ny = 2. * diffabs(ref_xyn, xn * yn + xn * Y + yn * X) - b;
    } break;
    }
    *x = nx; *y = ny;
}

/* burning_ship.py:622-859 _p_iter_hessian.  h = (dxnda, dxndb, dynda, dyndb) */
static inline void bs_p_iter_hessian(int flavor, double *h, double xn, double yn, double X, double Y,
                                     double Xa, double Xb, double Ya, double Yb) {
    double xa = h[0], xb = h[1], ya = h[2], yb = h[3];
    double nxa, nxb, nya, nyb;
    switch (flavor) {
    case 1: {
        double opX = X * Y;
        double dXa = Xa * Y + X * Ya, dXb = Xb * Y + X * Yb;
        double opx = xn * yn + xn * Y + yn * X;
        double dxa = xa * yn + xn * ya + xa * Y + xn * Ya + ya * X + yn * Xa;
        double dxb = xb * yn + xn * yb + xb * Y + xn * Yb + yb * X + yn * Xb;
        double dX = ddiffabsdX(opX, opx), dx = ddiffabsdx(opX, opx);
        nxa = 2. * ((X + xn) * xa + Xa * xn) - 2. * ((Y + yn) * ya + Ya * yn);
        nxb = 2. * ((X + xn) * xb + Xb * xn) - 2. * ((Y + yn) * yb + Yb * yn);
        nya = 2. * (dX * dXa + dx * dxa);
        nyb = 2. * (dX * dXb + dx * dxb);
    } break;
    case 2: {
        double da = diffabs(Y, yn), dX = ddiffabsdX(Y, yn), dx = ddiffabsdx(Y, yn);
        double Yy = Y + yn, ab = fabs(Yy), sg = sgn(Yy);
        nxa = 2. * (((X + xn) * xa + Xa * xn) - ((Y + yn) * ya + Ya * yn));
        nxb = 2. * (((X + xn) * xb + Xb * xn) - ((Y + yn) * yb + Yb * yn));
        nya = 2. * (Xa * da + X * (dX * Ya + dx * ya) + xa * ab + xn * sg * (Ya + ya));
        nyb = 2. * (Xb * da + X * (dX * Yb + dx * yb) + xb * ab + xn * sg * (Yb + yb));
    } break;
    case 3: {
        double da = diffabs(Y, yn), dX = ddiffabsdX(Y, yn), dx = ddiffabsdx(Y, yn);
        double Yy = Y + yn, ab = fabs(Yy), sg = sgn(Yy);
        nxa = xa * (xn + 2. * X) + xn * (xa + 2. * Xa) - Ya * da - Y * (Ya * dX + ya * dx)
              - ya * ab - yn * sg * (Ya + ya);
        nxb = xb * (xn + 2. * X) + xn * (xb + 2. * Xb) - Yb * da - Y * (Yb * dX + yb * dx)
              - yb * ab - yn * sg * (Yb + yb);
        nya = 2. * (Xa * yn + X * ya + Ya * xn + Y * xa + xa * yn + xn * ya);
        nyb = 2. * (Xb * yn + X * yb + Yb * xn + Y * xb + xb * yn + xn * yb);
    } break;
    case 4: {
        double opX = X * X - Y * Y;
        double dXa = 2. * (X * Xa - Y * Ya), dXb = 2. * (X * Xb - Y * Yb);
        double opx = xn * (xn + 2. * X) - yn * (yn + 2. * Y);
        double dxa = xa * (xn + 2. * X) + xn * (xa + 2. * Xa) - ya * (yn + 2. * Y) - yn * (ya + 2. * Ya);
        double dxb = xb * (xn + 2. * X) + xn * (xb + 2. * Xb) - yb * (yn + 2. * Y) - yn * (yb + 2. * Yb);
        double dX = ddiffabsdX(opX, opx), dx = ddiffabsdx(opX, opx);
        nxa = dX * dXa + dx * dxa;
        nxb = dX * dXb + dx * dxb;
        nya = 2. * (Xa * yn + X * ya + Ya * xn + Y * xa + xa * yn + xn * ya);
        nyb = 2. * (Xb * yn + X * yb + Yb * xn + Y * xb + xb * yn + xn * yb);
    } break;
    default: {
        double opX = X * X - Y * Y;
        double dXa = 2. * (X * Xa - Y * Ya), dXb = 2. * (X * Xb - Y * Yb);
        double opx = xn * (xn + 2. * X) - yn * (yn + 2. * Y);
        double dxa = xa * (xn + 2. * X) + xn * (xa + 2. * Xa) - ya * (yn + 2. * Y) - yn * (ya + 2. * Ya);
        double dxb = xb * (xn + 2. * X) + xn * (xb + 2. * Xb) - yb * (yn + 2. * Y) - yn * (yb + 2. * Yb);
        double dX = ddiffabsdX(opX, opx), dx = ddiffabsdx(opX, opx);
        nxa = dX * dXa + dx * dxa;
        nxb = dX * dXb + dx * dxb;
        double opX2 = X * Y;
        double dXa2 = Xa * Y + X * Ya, dXb2 = Xb * Y + X * Yb;
        double opx2 = xn * yn + xn * Y + yn * X;
        double dxa2 = xa * yn + xn * ya + xa * Y + xn * Ya + ya * X + yn * Xa;
        double dxb2 = xb * yn + xn * yb + xb * Y + xn * Yb + yb * X + yn * Xb;
        double dX2 = ddiffabsdX(opX2, opx2), dx2 = ddiffabsdx(opX2, opx2);
        nya = 2. * (dX2 * dXa2 + dx2 * dxa2);
        nyb = 2. * (dX2 * dXb2 + dx2 * dxb2);
    } break;
    }
    h[0] = nxa; h[1] = nxb; h[2] = nya; h[3] = nyb;
}

typedef struct {
    const double *Zn; int64_t ref_len; int64_t ref_div_iter; int64_t ref_order;
    const double *dXa, *dXb, *dYa, *dYb;
    const double *M_bla; const double *r_bla; int32_t stages_bla; int32_t bla_on;
    int64_t max_iter; double M2; int32_t flavor; int32_t calc_hessian;
    double lin_mat[4]; double dx_m; int32_t dx_e; double driftx_m; int32_t driftx_e;
    double drifty_m; int32_t drifty_e;
    /* calc_orbit: snapshots every backshift iterations (0: off) into rows
     * i_xnorbit, i_xnorbit + 1 */
    int32_t backshift; int32_t i_xnorbit;
} orc_pbs_args;

EXPORT int orc_perturb_bs(const orc_pbs_args *P, int64_t npts, const double *pix,
                          double *Zout, int32_t nZ, int32_t *U, int8_t *stop_reason,
                          int32_t *stop_iter) {
    const int64_t order = P->ref_order, div_iter = P->ref_div_iter, plen = P->ref_len;
    const int hess = P->calc_hessian;
    int64_t first_invalid = plen;
    if (div_iter < first_invalid) first_invalid = div_iter;
    if (order < first_invalid) first_invalid = order;
    for (int64_t ip = 0; ip < npts; ip++) {
        /* perturbation.py:2260-2280 ref_path_c_from_pix_BS through Xrange values */
        double px = pix[2 * ip], py = pix[2 * ip + 1];
        double x1 = P->lin_mat[0] * px + P->lin_mat[1] * py;
        double y1 = P->lin_mat[2] * px + P->lin_mat[3] * py;
        xf dxr = {P->dx_m, P->dx_e};
        xc c_xr = xf_mul_c(dxr, C(x1, y1));
        xf a_xr = {c_xr.re, c_xr.e}, b_xr = {c_xr.im, c_xr.e};
        xf ddx = {P->driftx_m, P->driftx_e}, ddy = {P->drifty_m, P->drifty_e};
        double a = xf_to_std(xf_add(a_xr, ddx)), b = xf_to_std(xf_add(b_xr, ddy));
        double xn = Zout[ip], yn = Zout[npts + ip];
        double h[4] = {0., 0., 0., 0.};
        if (hess) for (int k = 0; k < 4; k++) h[k] = Zout[(2 + k) * npts + ip];
        int64_t w = 0, n = 0; int8_t stop = -1; int dyn = 1;
        orbit_snap S; snap_init(&S, C(xn, yn));      /* perturbation.py:1501-1508 */
        for (;;) {
            if (P->bla_on && (w & 7) == 0) {
                int64_t ib;
                int64_t step = bla_get(P->r_bla, P->stages_bla, hypot(xn, yn), w, first_invalid, &ib);
                if (step != 0) {
                    const double *M = P->M_bla + 8 * ib;
                    n += step; w = (w + step) % order;
                    double nx = M[0] * xn + M[1] * yn + M[4] * a + M[5] * b;
                    double ny = M[2] * xn + M[3] * yn + M[6] * a + M[7] * b;
                    xn = nx; yn = ny;
                    if (hess) {
                        double xa = M[0] * h[0] + M[1] * h[2], xb = M[0] * h[1] + M[1] * h[3];
                        double ya = M[2] * h[0] + M[3] * h[2], yb = M[2] * h[1] + M[3] * h[3];
                        h[0] = xa; h[1] = xb; h[2] = ya; h[3] = yb;
                    }
                    continue;
                }
            }
            n += 1;
            double X = P->Zn[2 * w], Y = P->Zn[2 * w + 1];
            if (hess) {
                double Xa = P->dXa[w], Xb = P->dXb[w], Ya = P->dYa[w], Yb = P->dYb[w];
                if (dyn) { Xa = 0.; Xb = 0.; Ya = 0.; Yb = 0.; }
                bs_p_iter_hessian(P->flavor, h, xn, yn, X, Y, Xa, Xb, Ya, Yb);
            }
            bs_p_iter_zn(P->flavor, &xn, &yn, X, Y, a, b);
            if (n >= P->max_iter) { stop = 0; break; }
            w += 1;
            if (w >= order) w = w % order;
            double XX = xn + P->Zn[2 * w], YY = yn + P->Zn[2 * w + 1];
            double sq = XX * XX + YY * YY;
            if (P->backshift > 0) snap_take(&S, n, P->backshift, C(XX, YY));  /* :1641-1651 */
            if (sq > P->M2) { stop = 1; break; }
            if (w >= div_iter - 1) {
                xn = XX; yn = YY;
                if (hess) { h[0] += P->dXa[w]; h[1] += P->dXb[w]; h[2] += P->dYa[w]; h[3] += P->dYb[w]; }
                w = 0; continue;
            }
            dyn = (fabs(XX) <= fabs(xn)) && (fabs(YY) <= fabs(yn));
            if (dyn) {
                xn = XX; yn = YY;
                if (hess) { h[0] += P->dXa[w]; h[1] += P->dXb[w]; h[2] += P->dYa[w]; h[3] += P->dYb[w]; }
                w = 0; continue;
            }
        }
        U[ip] = (int32_t)w;
        xn += P->Zn[2 * w]; yn += P->Zn[2 * w + 1];
        if (hess) { h[0] += P->dXa[w]; h[1] += P->dXb[w]; h[2] += P->dYa[w]; h[3] += P->dYb[w]; }
        Zout[ip] = xn; Zout[npts + ip] = yn;
        if (hess) for (int k = 0; k < 4; k++) Zout[(2 + k) * npts + ip] = h[k];
        if (P->backshift > 0 && P->i_xnorbit >= 0) {                          /* :1778-1787 */
            /* AA, BB as the reference forms them: b + Im(Z_1) with Im(Z_1) = -b_ref,
             * so BB = b - b_ref rather than the pixel's b + b_ref */
            double AA = a + P->Zn[2], BB = b + P->Zn[3];
            double xo = S.z2.re, yo = S.z2.im;
            while (S.i2 < n - P->backshift) {
                double nx_, ny_;
                bs_iterate(P->flavor, xo, yo, AA, BB, &nx_, &ny_);
                xo = nx_; yo = ny_; S.i2 += 1;
            }
            Zout[P->i_xnorbit * npts + ip] = xo; Zout[(P->i_xnorbit + 1) * npts + ip] = yo;
        }
        stop_iter[ip] = (int32_t)n; stop_reason[ip] = stop;
    }
    return 0;
}

/* ========================================================================= */
/* Burning Ship perturbation, Xrange branch (xr_detect_activated):            */
/* perturbation.py:1468-1791 with the deltas, c and the Jacobian as float64   */
/* Xrange records; the closures of models/burning_ship.py:19-60, 535-859 are  */
/* the double ones above, each operation on Xrange operands (numba_xr.py), in */
/* the same order.  Derivative paths: numba_dZndc_path_BS's Xrange branch     */
/* (perturbation.py:2339-2438) with incr_deriv_ref_BS (:2440-2463).           */
/* ========================================================================= */
#define XA(a, b) xf_add((a), (b))
#define XS(a, b) xf_sub((a), (b))
#define XM(a, b) xf_mul((a), (b))
#define XK(s, b) xf_mul_s((s), (b))            /* float * Xrange */
static inline xf xf_neg(xf a) { a.m = -a.m; return a; }
static inline xf xf_abs(xf a) { a.m = fabs(a.m); return a; }
static inline int xf_ge0(xf a) { return xf_ge_s(a, 0.); }
static inline int xf_le0(xf a) { return xf_le_s(a, 0.); }
static inline double xf_sgn(xf a) { return xf_lt_s(a, 0.) ? -1. : 1.; }
static const xf XF0 = {0., 0};

/* burning_ship.py:19-60 on Xrange operands */
static inline xf diffabs_x(xf X, xf x) {
    if (xf_ge0(X)) { if (xf_ge0(XA(X, x))) return XK(1., x); return xf_neg(XA(XK(2., X), x)); }
    if (xf_le0(XA(X, x))) return xf_neg(x);
    return XA(XK(2., X), x);
}
static inline double ddiffabsdX_x(xf X, xf x) {
    if (xf_ge0(X)) return xf_ge0(XA(X, x)) ? 0. : -2.;
    return xf_le0(XA(X, x)) ? 0. : 2.;
}
static inline double ddiffabsdx_x(xf X, xf x) {
    if (xf_ge0(X)) return xf_ge0(XA(X, x)) ? 1. : -1.;
    return xf_le0(XA(X, x)) ? -1. : 1.;
}

/* xn * (xn + 2 X) - yn * (yn + 2 Y) */
static inline xf bsx_sq(xf xn, xf yn, xf X, xf Y) {
    return XS(XM(xn, XA(xn, XK(2., X))), XM(yn, XA(yn, XK(2., Y))));
}
/* xn * yn + xn * Y + yn * X */
static inline xf bsx_cross(xf xn, xf yn, xf X, xf Y) {
    return XA(XA(XM(xn, yn), XM(xn, Y)), XM(yn, X));
}
/* X * yn + Y * xn + xn * yn */
static inline xf bsx_cross2(xf xn, xf yn, xf X, xf Y) {
    return XA(XA(XM(X, yn), XM(Y, xn)), XM(xn, yn));
}

static inline void bsx_p_iter_zn(int flavor, xf *x, xf *y, xf X, xf Y, xf a, xf b) {
    xf nx, ny, xn = *x, yn = *y;
    switch (flavor) {
    case 1:
        nx = XA(bsx_sq(xn, yn, X, Y), a);
        ny = XS(XK(2., diffabs_x(XM(X, Y), bsx_cross(xn, yn, X, Y))), b);
        break;
    case 2:
        nx = XA(bsx_sq(xn, yn, X, Y), a);
        ny = XS(XK(2., XA(XM(X, diffabs_x(Y, yn)), XM(xn, xf_abs(XA(Y, yn))))), b);
        break;
    case 3:
        nx = XA(XS(XS(XM(xn, XA(xn, XK(2., X))), XM(Y, diffabs_x(Y, yn))),
                   XM(yn, xf_abs(XA(Y, yn)))), a);
        ny = XS(XK(2., bsx_cross2(xn, yn, X, Y)), b);
        break;
    case 4:
        nx = XA(diffabs_x(XS(XM(X, X), XM(Y, Y)), bsx_sq(xn, yn, X, Y)), a);
        ny = XS(XK(2., bsx_cross2(xn, yn, X, Y)), b);
        break;
    default: {
        xf ref_xyn = XM(X, Y), ref_x2my2 = XS(XM(X, X), XM(Y, Y));
        nx = XA(diffabs_x(ref_x2my2, bsx_sq(xn, yn, X, Y)), a);
        ny = XS(XK(2., diffabs_x(ref_xyn, bsx_cross(xn, yn, X, Y))), b);
    } break;
    }
    *x = nx; *y = ny;
}

/* d/da of xn * yn + xn * Y + yn * X (flavors 1, 5): the six products in order */
static inline xf bsx_dcross(xf xa, xf ya, xf xn, xf yn, xf X, xf Y, xf Xa, xf Ya) {
    return XA(XA(XA(XA(XA(XM(xa, yn), XM(xn, ya)), XM(xa, Y)), XM(xn, Ya)), XM(ya, X)),
              XM(yn, Xa));
}
/* d/da of xn (xn + 2 X) - yn (yn + 2 Y) (flavors 4, 5) */
static inline xf bsx_dsq(xf xa, xf ya, xf xn, xf yn, xf X, xf Y, xf Xa, xf Ya) {
    return XS(XS(XA(XM(xa, XA(xn, XK(2., X))), XM(xn, XA(xa, XK(2., Xa)))),
                 XM(ya, XA(yn, XK(2., Y)))), XM(yn, XA(ya, XK(2., Ya))));
}
/* 2 (Xa yn + X ya + Ya xn + Y xa + xa yn + xn ya) (flavors 3, 4) */
static inline xf bsx_dcross2(xf xa, xf ya, xf xn, xf yn, xf X, xf Y, xf Xa, xf Ya) {
    return XK(2., XA(XA(XA(XA(XA(XM(Xa, yn), XM(X, ya)), XM(Ya, xn)), XM(Y, xa)), XM(xa, yn)),
                     XM(xn, ya)));
}
/* 2 ((X + xn) xa + Xa xn) - 2 ((Y + yn) ya + Ya yn) (flavor 1) */
static inline xf bsx_dsq1(xf xa, xf ya, xf xn, xf yn, xf X, xf Y, xf Xa, xf Ya) {
    return XS(XK(2., XA(XM(XA(X, xn), xa), XM(Xa, xn))),
              XK(2., XA(XM(XA(Y, yn), ya), XM(Ya, yn))));
}

/* burning_ship.py:622-859 on Xrange operands; h = (dxnda, dxndb, dynda, dyndb) */
static inline void bsx_p_iter_hessian(int flavor, xf *h, xf xn, xf yn, xf X, xf Y,
                                      xf Xa, xf Xb, xf Ya, xf Yb) {
    xf xa = h[0], xb = h[1], ya = h[2], yb = h[3];
    xf nxa, nxb, nya, nyb;
    switch (flavor) {
    case 1: {
        xf opX = XM(X, Y);
        xf dXa = XA(XM(Xa, Y), XM(X, Ya)), dXb = XA(XM(Xb, Y), XM(X, Yb));
        xf opx = bsx_cross(xn, yn, X, Y);
        xf dxa = bsx_dcross(xa, ya, xn, yn, X, Y, Xa, Ya);
        xf dxb = bsx_dcross(xb, yb, xn, yn, X, Y, Xb, Yb);
        double dX = ddiffabsdX_x(opX, opx), dx = ddiffabsdx_x(opX, opx);
        nxa = bsx_dsq1(xa, ya, xn, yn, X, Y, Xa, Ya);
        nxb = bsx_dsq1(xb, yb, xn, yn, X, Y, Xb, Yb);
        nya = XK(2., XA(XK(dX, dXa), XK(dx, dxa)));
        nyb = XK(2., XA(XK(dX, dXb), XK(dx, dxb)));
    } break;
    case 2: {
        xf da = diffabs_x(Y, yn);
        double dX = ddiffabsdX_x(Y, yn), dx = ddiffabsdx_x(Y, yn);
        xf Yy = XA(Y, yn), ab = xf_abs(Yy);
        double sg = xf_sgn(Yy);
        nxa = XK(2., XS(XA(XM(XA(X, xn), xa), XM(Xa, xn)), XA(XM(XA(Y, yn), ya), XM(Ya, yn))));
        nxb = XK(2., XS(XA(XM(XA(X, xn), xb), XM(Xb, xn)), XA(XM(XA(Y, yn), yb), XM(Yb, yn))));
        nya = XK(2., XA(XA(XA(XM(Xa, da), XM(X, XA(XK(dX, Ya), XK(dx, ya)))), XM(xa, ab)),
                        XM(XK(sg, xn), XA(Ya, ya))));
        nyb = XK(2., XA(XA(XA(XM(Xb, da), XM(X, XA(XK(dX, Yb), XK(dx, yb)))), XM(xb, ab)),
                        XM(XK(sg, xn), XA(Yb, yb))));
    } break;
    case 3: {
        xf da = diffabs_x(Y, yn);
        double dX = ddiffabsdX_x(Y, yn), dx = ddiffabsdx_x(Y, yn);
        xf Yy = XA(Y, yn), ab = xf_abs(Yy);
        double sg = xf_sgn(Yy);
        nxa = XS(XS(XS(XS(XA(XM(xa, XA(xn, XK(2., X))), XM(xn, XA(xa, XK(2., Xa)))), XM(Ya, da)),
                       XM(Y, XA(XK(dX, Ya), XK(dx, ya)))), XM(ya, ab)),
                 XM(XK(sg, yn), XA(Ya, ya)));
        nxb = XS(XS(XS(XS(XA(XM(xb, XA(xn, XK(2., X))), XM(xn, XA(xb, XK(2., Xb)))), XM(Yb, da)),
                       XM(Y, XA(XK(dX, Yb), XK(dx, yb)))), XM(yb, ab)),
                 XM(XK(sg, yn), XA(Yb, yb)));
        nya = bsx_dcross2(xa, ya, xn, yn, X, Y, Xa, Ya);
        nyb = bsx_dcross2(xb, yb, xn, yn, X, Y, Xb, Yb);
    } break;
    case 4: {
        xf opX = XS(XM(X, X), XM(Y, Y));
        xf dXa = XK(2., XS(XM(X, Xa), XM(Y, Ya))), dXb = XK(2., XS(XM(X, Xb), XM(Y, Yb)));
        xf opx = bsx_sq(xn, yn, X, Y);
        xf dxa = bsx_dsq(xa, ya, xn, yn, X, Y, Xa, Ya);
        xf dxb = bsx_dsq(xb, yb, xn, yn, X, Y, Xb, Yb);
        double dX = ddiffabsdX_x(opX, opx), dx = ddiffabsdx_x(opX, opx);
        nxa = XA(XK(dX, dXa), XK(dx, dxa));
        nxb = XA(XK(dX, dXb), XK(dx, dxb));
        nya = bsx_dcross2(xa, ya, xn, yn, X, Y, Xa, Ya);
        nyb = bsx_dcross2(xb, yb, xn, yn, X, Y, Xb, Yb);
    } break;
    default: {
        xf opX = XS(XM(X, X), XM(Y, Y));
        xf dXa = XK(2., XS(XM(X, Xa), XM(Y, Ya))), dXb = XK(2., XS(XM(X, Xb), XM(Y, Yb)));
        xf opx = bsx_sq(xn, yn, X, Y);
        xf dxa = bsx_dsq(xa, ya, xn, yn, X, Y, Xa, Ya);
        xf dxb = bsx_dsq(xb, yb, xn, yn, X, Y, Xb, Yb);
        double dX = ddiffabsdX_x(opX, opx), dx = ddiffabsdx_x(opX, opx);
        nxa = XA(XK(dX, dXa), XK(dx, dxa));
        nxb = XA(XK(dX, dXb), XK(dx, dxb));
        xf opX2 = XM(X, Y);
        xf dXa2 = XA(XM(Xa, Y), XM(X, Ya)), dXb2 = XA(XM(Xb, Y), XM(X, Yb));
        xf opx2 = bsx_cross(xn, yn, X, Y);
        xf dxa2 = bsx_dcross(xa, ya, xn, yn, X, Y, Xa, Ya);
        xf dxb2 = bsx_dcross(xb, yb, xn, yn, X, Y, Xb, Yb);
        double dX2 = ddiffabsdX_x(opX2, opx2), dx2 = ddiffabsdx_x(opX2, opx2);
        nya = XK(2., XA(XK(dX2, dXa2), XK(dx2, dxa2)));
        nyb = XK(2., XA(XK(dX2, dXb2), XK(dx2, dxb2)));
    } break;
    }
    h[0] = nxa; h[1] = nxb; h[2] = nya; h[3] = nyb;
}

/* models/burning_ship.py:441-532 on Xrange operands: the float factors
 * (2., the signs) first, as the reference's 2. * sgn(x) * abs(y) */
static inline void bsx_dfdxy(int flavor, xf x, xf y, xf *fxx, xf *fxy, xf *fyx, xf *fyy) {
    switch (flavor) {
    case 1: *fxx = XK(2., x); *fxy = XK(-2., y); *fyx = XK(2. * xf_sgn(x), xf_abs(y));
            *fyy = XK(2. * xf_sgn(y), xf_abs(x)); break;
    case 2: *fxx = XK(2., x); *fxy = XK(-2., y); *fyx = XK(2., xf_abs(y));
            *fyy = XK(2. * xf_sgn(y), x); break;
    case 3: *fxx = XK(2., x); *fxy = XK(-2., xf_abs(y)); *fyx = XK(2., y); *fyy = XK(2., x); break;
    case 4: { double s = xf_sgn(XS(XM(x, x), XM(y, y)));
              *fxx = XK(2. * s, x); *fxy = XK(-2. * s, y); *fyx = XK(2., y); *fyy = XK(2., x); } break;
    default: { double s = xf_sgn(XS(XM(x, x), XM(y, y)));
               *fxx = XK(2. * s, x); *fxy = XK(-2. * s, y);
               *fyx = XK(2. * xf_sgn(x), xf_abs(y)); *fyy = XK(2. * xf_sgn(y), xf_abs(x)); } break;
    }
}

/* The BS orbit's side table: perturbation.py:2591-2663 ref_path_get_BS as a
 * membership lookup (the cursor is an optimisation of it). */
typedef struct {
    int32_t n; const int32_t *idx; const double *xm, *ym; const int32_t *xe, *ye;
} xr_table_bs;
static inline int xr_lookup_bs(const xr_table_bs *t, int64_t w, xf *X, xf *Y) {
    int lo = 0, hi = t->n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (t->idx[mid] == w) {
            X->m = t->xm[mid]; X->e = t->xe[mid]; Y->m = t->ym[mid]; Y->e = t->ye[mid];
            return 1;
        }
        if (t->idx[mid] < w) lo = mid + 1; else hi = mid - 1;
    }
    return 0;
}
/* ensure_xr_BS (perturbation.py:2182-2193): the side-table value, else the
 * standard value as Xrange */
static inline void bsx_ref(const xr_table_bs *t, const double *Zn, int64_t w, xf *X, xf *Y,
                           int *is_xr) {
    *is_xr = t->n > 0 && xr_lookup_bs(t, w, X, Y);
    if (!*is_xr) { *X = xr_from_r(Zn[2 * w]); *Y = xr_from_r(Zn[2 * w + 1]); }
}

/* numba_dZndc_path_BS, Xrange branch: out_m / out_e [4][len] (dXnda, dXndb,
 * dYnda, dYndb); scale = dx * projection scale as a float64 Xrange */
EXPORT void orc_dzndc_path_bs_xr(const double *Zn, int64_t len, int64_t ref_div_iter,
                                 int64_t ref_order, int32_t flavor, double scale_m,
                                 int32_t scale_e, int32_t n_xr, const int32_t *xr_idx,
                                 const double *xr_xm, const int32_t *xr_xe, const double *xr_ym,
                                 const int32_t *xr_ye, double *out_m, int32_t *out_e) {
    const xr_table_bs t = {n_xr, xr_idx, xr_xm, xr_ym, xr_xe, xr_ye};
    const xf dx = {scale_m, scale_e};
    int64_t valid = len < ref_div_iter ? len : ref_div_iter;
    for (int64_t k = 0; k < 4 * len; k++) { out_m[k] = 0.; out_e[k] = 0; }
#define PM(j, i) out_m[(j) * len + (i)]
#define PE(j, i) out_e[(j) * len + (i)]
    int64_t i;
    for (i = 1; i <= valid; i++) {
        int64_t from = i - 1, to = i;
        if (i == valid) {
            if (!(from == ref_order - 1)) break;
            to = 0;
        }
        xf X, Y; int isx;
        bsx_ref(&t, Zn, from, &X, &Y, &isx);
        xf fxx, fxy, fyx, fyy;
        bsx_dfdxy(flavor, X, Y, &fxx, &fxy, &fyx, &fyy);
        xf a = {PM(0, from), PE(0, from)}, b = {PM(1, from), PE(1, from)};
        xf c = {PM(2, from), PE(2, from)}, d = {PM(3, from), PE(3, from)};
        xf r[4];
        r[0] = XA(XA(XM(fxx, a), XM(fxy, c)), dx);
        r[1] = XA(XM(fxx, b), XM(fxy, d));
        r[2] = XA(XM(fyx, a), XM(fyy, c));
        r[3] = XS(XA(XM(fyx, b), XM(fyy, d)), dx);
        for (int j = 0; j < 4; j++) { PM(j, to) = r[j].m; PE(j, to) = r[j].e; }
    }
#undef PM
#undef PE
}

typedef struct {
    const double *Zn; int64_t ref_len; int64_t ref_div_iter; int64_t ref_order;
    int32_t n_xr; const int32_t *xr_idx; const double *xr_xm; const int32_t *xr_xe;
    const double *xr_ym; const int32_t *xr_ye;
    const double *path_m; const int32_t *path_e;          /* [4][ref_len] Xrange Jacobian */
    const double *M_bla; const double *r_bla; int32_t stages_bla; int32_t bla_on;
    int64_t max_iter; double M2; int32_t flavor; int32_t calc_hessian;
    double lin_mat[4]; double dx_m; int32_t dx_e; double driftx_m; int32_t driftx_e;
    double drifty_m; int32_t drifty_e;
} orc_pbs_xr_args;

EXPORT int orc_perturb_bs_xr(const orc_pbs_xr_args *P, int64_t npts, const double *pix,
                             double *Zout, int32_t nZ, int32_t *U, int8_t *stop_reason,
                             int32_t *stop_iter) {
    const int64_t order = P->ref_order, div_iter = P->ref_div_iter, plen = P->ref_len;
    const int hess = P->calc_hessian;
    const xr_table_bs t = {P->n_xr, P->xr_idx, P->xr_xm, P->xr_ym, P->xr_xe, P->xr_ye};
    int64_t first_invalid = plen;
    if (div_iter < first_invalid) first_invalid = div_iter;
    if (order < first_invalid) first_invalid = order;
#define PATH(j, w) ((xf){P->path_m[(j) * plen + (w)], P->path_e[(j) * plen + (w)]})
    for (int64_t ip = 0; ip < npts; ip++) {
        /* perturbation.py:2260-2280 ref_path_c_from_pix_BS */
        double px = pix[2 * ip], py = pix[2 * ip + 1];
        double x1 = P->lin_mat[0] * px + P->lin_mat[1] * py;
        double y1 = P->lin_mat[2] * px + P->lin_mat[3] * py;
        xf dxr = {P->dx_m, P->dx_e};
        xc c_xr = xf_mul_c(dxr, C(x1, y1));
        xf ddx = {P->driftx_m, P->driftx_e}, ddy = {P->drifty_m, P->drifty_e};
        xf cre = {c_xr.re, c_xr.e}, cim = {c_xr.im, c_xr.e};
        const xf a_xr = XA(cre, ddx), b_xr = XA(cim, ddy);
        /* numba_initialize_BS: the Xrange deltas from the tile's Z, the
         * standard copies as the tile's values */
        double xs = Zout[ip], ys = Zout[npts + ip];
        xf xn = xr_from_r(xs), yn = xr_from_r(ys);
        xf h[4] = {XF0, XF0, XF0, XF0};
        if (hess) for (int k = 0; k < 4; k++) h[k] = xr_from_r(Zout[(2 + k) * npts + ip]);
        int64_t w = 0, n = 0; int8_t stop = -1; int dyn = 1;
        for (;;) {
            if (P->bla_on && (w & 7) == 0) {                   /* :1520-1545 */
                int64_t ib;
                int64_t step = bla_get(P->r_bla, P->stages_bla, hypot(xs, ys), w, first_invalid, &ib);
                if (step != 0) {
                    const double *M = P->M_bla + 8 * ib;
                    n += step; w = (w + step) % order;
                    xf nx = XA(XA(XA(XK(M[0], xn), XK(M[1], yn)), XK(M[4], a_xr)), XK(M[5], b_xr));
                    xf ny = XA(XA(XA(XK(M[2], xn), XK(M[3], yn)), XK(M[6], a_xr)), XK(M[7], b_xr));
                    xn = nx; yn = ny;
                    xs = xf_to_std(xn); ys = xf_to_std(yn);
                    if (hess) {
                        xf xa = XA(XK(M[0], h[0]), XK(M[1], h[2])), xb = XA(XK(M[0], h[1]), XK(M[1], h[3]));
                        xf ya = XA(XK(M[2], h[0]), XK(M[3], h[2])), yb = XA(XK(M[2], h[1]), XK(M[3], h[3]));
                        h[0] = xa; h[1] = xb; h[2] = ya; h[3] = yb;
                    }
                    continue;
                }
            }
            n += 1;                                                /* :1548-1611 */
            xf X, Y; int isx;
            bsx_ref(&t, P->Zn, w, &X, &Y, &isx);
            if (hess) {
                xf Xa = XF0, Xb = XF0, Ya = XF0, Yb = XF0;
                if (!dyn) { Xa = PATH(0, w); Xb = PATH(1, w); Ya = PATH(2, w); Yb = PATH(3, w); }
                bsx_p_iter_hessian(P->flavor, h, xn, yn, X, Y, Xa, Xb, Ya, Yb);
            }
            bsx_p_iter_zn(P->flavor, &xn, &yn, X, Y, a_xr, b_xr);
            xs = xf_to_std(xn); ys = xf_to_std(yn);
            if (n >= P->max_iter) { stop = 0; break; }
            w += 1;
            if (w >= order) w = w % order;
            xf Xn, Yn; int isn;                                    /* :1627-1636 */
            bsx_ref(&t, P->Zn, w, &Xn, &Yn, &isn);
            double XX = xs + P->Zn[2 * w], YY = ys + P->Zn[2 * w + 1];
            if (XX * XX + YY * YY > P->M2) { stop = 1; break; }
            if (w >= div_iter - 1) {                               /* :1660-1684 */
                xs = XX; ys = YY;
                xn = xr_from_r(XX); yn = xr_from_r(YY);
                if (hess) for (int k = 0; k < 4; k++) h[k] = XA(h[k], PATH(k, w));
                w = 0; continue;
            }
            dyn = (fabs(XX) <= fabs(xs)) && (fabs(YY) <= fabs(ys));   /* :1688-1731 */
            if (dyn) {
                xf XXx = isn ? XA(xn, Xn) : xf_add_s(xn, P->Zn[2 * w]);
                xf YYx = isn ? XA(yn, Yn) : xf_add_s(yn, P->Zn[2 * w + 1]);
                if (xf_le(XA(XM(XXx, XXx), XM(YYx, YYx)), XA(XM(xn, xn), XM(yn, yn)))) {
                    xn = XXx; yn = YYx;
                    xs = xf_to_std(XXx); ys = xf_to_std(YYx);
                    if (hess) for (int k = 0; k < 4; k++) h[k] = XA(h[k], PATH(k, w));
                    w = 0; continue;
                }
            }
        }
        U[ip] = (int32_t)w;                                        /* :1745-1757 */
        Zout[ip] = xf_to_std(xf_add_s(xn, P->Zn[2 * w]));
        Zout[npts + ip] = xf_to_std(xf_add_s(yn, P->Zn[2 * w + 1]));
        if (hess) for (int k = 0; k < 4; k++) Zout[(2 + k) * npts + ip] = xf_to_std(XA(h[k], PATH(k, w)));
        stop_iter[ip] = (int32_t)n; stop_reason[ip] = stop;
    }
#undef PATH
    return 0;
}
#undef XA
#undef XS
#undef XM
#undef XK
