// fsg_mn.cuh -- power-n Mandelbrot (z -> z^n + c) arithmetic of the standard
// loop, the perturbation closures and the reference tables.
//
// Follows models/mandelbrot_Mn.py: iterate_once :317-355 (standard loop,
// `zn ** (n - 1)` as numpy's integer power of a complex), the closures of
// from_numba_cache :626-733 (dfdz, p_iter_zn, p_iter_dzndz / p_iter_dzndc, a
// full binomial expansion in the perturbation) -- every product and sum in
// the reference's order, so that translation units built with -fmad=false
// reproduce its results bit for bit.  nexp = 0 stands for the power-2
// model's own closures (models/mandelbrot_M2.py), which round differently.
#pragma once
#include "fsg_num.cuh"

#ifndef FSG_MN_MAX_EXP
#define FSG_MN_MAX_EXP 32    // largest exponent of the power-n kernels (fsgpu.h)
#endif

// z^k for k >= 1 as numpy's complex integer power (n = 1, 2, 3 by direct
// products, else binary powering from 1).
FSG_DEV double2 mn_ipow(double2 a, int n) {
    if (n == 1) return a;
    if (n == 2) return csq(a);
    if (n == 3) return cmul(a, csq(a));
    double2 acc = cx(1., 0.), p = a;
    int mask = 1;
    for (;;) {
        if (n & mask) acc = cmul(acc, p);
        mask <<= 1;
        if (n < mask) break;
        p = csq(p);
    }
    return acc;
}

// df/dz: n z^(n-1) as z * z * ... * z times n (mandelbrot_Mn.py:645-652);
// the power-2 model's 2 z when nexp = 0
FSG_DEV double2 mn_dfdz(int nexp, double2 z) {
    if (nexp == 0) return rmul2(z);
    double2 t = z;
    for (int k = 2; k < nexp; k++) t = cmul(t, z);
    return rmul((double)nexp, t);
}
FSG_DEV xc mn_dfdz_x(int nexp, xc z) {
    if (nexp == 0) return xr_mul_2(z);
    xc t = z;
    for (int k = 2; k < nexp; k++) t = xr_mul(t, z);
    return xr_mul_r((double)nexp, t);
}

// p_iter_zn: (Z + z)^n - Z^n + c expanded in powers of z, Horner-like in z
// with increasing powers of the reference value Z (mandelbrot_Mn.py:660-672).
// Cb[k] = C(n, k) as float64.
FSG_DEV double2 mn_p_zn(int n, const double *Cb, double2 z, double2 ref, double2 c) {
    double2 tmp = cmul(z, cadd(z, rmul(Cb[1], ref)));
    double2 pk = ref;
    for (int k = 2; k < n; k++) {
        pk = cmul(pk, ref);
        tmp = cmul(z, cadd(tmp, rmul(Cb[k], pk)));
    }
    return cadd(tmp, c);
}
FSG_DEV xc mn_p_zn_x(int n, const double *Cb, xc z, xc ref, xc c) {
    xc tmp = xr_mul(z, xr_add(z, xr_mul_r(Cb[1], ref)));
    xc pk = ref;
    for (int k = 2; k < n; k++) {
        pk = xr_mul(pk, ref);
        tmp = xr_mul(z, xr_add(tmp, xr_mul_r(Cb[k], pk)));
    }
    return xr_add(tmp, c);
}

// p_iter_dzndz / p_iter_dzndc: derivative of the expansion above, d the
// delta's derivative, rd the reference's (mandelbrot_Mn.py:674-733)
FSG_DEV double2 mn_p_deriv(int n, const double *Cb, double2 z, double2 d, double2 ref,
                           double2 rd) {
    double2 mul = cadd(z, rmul(Cb[1], ref));
    double2 tmp = cmul(z, mul);
    double2 dt = cadd(cmul(d, mul), cmul(z, cadd(d, rmul(Cb[1], rd))));
    double2 pk = ref;
    for (int k = 2; k < n; k++) {
        double2 dpk = cmul(rmul((double)k, pk), rd);
        pk = cmul(pk, ref);
        mul = cadd(tmp, rmul(Cb[k], pk));
        dt = cadd(cmul(d, mul), cmul(z, cadd(dt, rmul(Cb[k], dpk))));
        tmp = cmul(z, mul);
    }
    return dt;
}
FSG_DEV xc mn_p_deriv_x(int n, const double *Cb, xc z, xc d, xc ref, xc rd) {
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
