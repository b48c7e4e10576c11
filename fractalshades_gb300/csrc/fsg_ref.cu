// fsg_ref.cu -- tables derived from the reference orbit, built on the GPU.
//
//   * derivative paths: numba_dZndc_path (perturbation.py:2282-2336),
//     with df/dz = 2 z (power-2 model) or n z^(n-1) (power-n model,
//     models/mandelbrot_Mn.py:645-652),
//     numba_dZndz_path (:2466-2516), numba_dZndc_path_BS + incr_deriv_ref_BS
//     (:2339-2463).  These are first-order linear recurrences evaluated in
//     the reference's order by one thread (they are O(len) and run once per
//     reference);
//   * the compressed BLA tree: numba_make_BLA (:1819-1881) / numba_make_BLA_BS
//     (:1884-1973) with combine_BLA (:1983-2024) / combine_BLA_BS
//     (:2027-2105).  The 8-iteration leaves are built one compressed block per
//     thread, then each level of the tree is one launch with one thread per
//     node (a parallel reduction over orbit levels);
//   * the fe (FP32 mantissa + int32 exponent) copies used by the fast kernel.
// Built with -fmad=false like the loops that consume these tables.
#include "fsg_internal.cuh"
#include "fsg_bs.cuh"

// ---------------------------------------------------------------------------
// derivative paths
// ---------------------------------------------------------------------------
__device__ __forceinline__ xc orbit_xr(const RefDev &R, int i) {
    double2 z = R.Zn[i];
    int slot = R.n_xr ? R.xr_slot[i] : -1;
    if (slot >= 0) return xc_make(R.xr_m[slot].x, R.xr_m[slot].y, R.xr_e[slot]);
    return xr_from(z);
}

__global__ void k_dzndc_m2(const RefDev *Rp, double2 *out_std, double2 *out_xm, int *out_xe,
                           int xr_mode, double scale_m, int scale_e) {
    const RefDev &R = *Rp;
    int len = R.len;
    int valid = len < R.div_iter ? len : R.div_iter;
    for (int k = 0; k <= len; k++) {
        if (xr_mode) { out_xm[k] = cx(0., 0.); out_xe[k] = 0; }
        else out_std[k] = cx(0., 0.);
    }
    int i;
    if (xr_mode) {
        for (i = 1; i < valid; i++) {
            xc zx = orbit_xr(R, i - 1);
            xc prev = xc_make(out_xm[i - 1].x, out_xm[i - 1].y, out_xe[i - 1]);
            xc v = xr_add(xr_mul(mn_dfdz_x(R.nexp, zx), prev), xc_make(scale_m, 0., scale_e));
            out_xm[i] = cx(v.re, v.im); out_xe[i] = v.e;
        }
        i -= 1;
        if (i == R.order - 1) {
            xc prev = xc_make(out_xm[i].x, out_xm[i].y, out_xe[i]);
            xc v = xr_add(xr_mul_s(mn_dfdz(R.nexp, R.Zn[i]), prev), xc_make(scale_m, 0., scale_e));
            out_xm[0] = cx(v.re, v.im); out_xe[0] = v.e;
        }
    } else {
        double scale = ldexp_d(scale_m, scale_e);
        for (i = 1; i < valid; i++)
            out_std[i] = caddr(cmul(mn_dfdz(R.nexp, R.Zn[i - 1]), out_std[i - 1]), scale);
        i -= 1;
        if (i == R.order - 1) out_std[0] = caddr(cmul(mn_dfdz(R.nexp, R.Zn[i]), out_std[i]), scale);
    }
}

__global__ void k_dzndz_m2(const RefDev *Rp, double2 *out_std, double2 *out_xm, int *out_xe,
                           int xr_mode) {
    const RefDev &R = *Rp;
    int len = R.len;
    int valid = len < R.div_iter ? len : R.div_iter;
    for (int k = 0; k <= len + 1; k++) {
        if (xr_mode) { out_xm[k] = cx(0., 0.); out_xe[k] = 0; }
        else out_std[k] = cx(0., 0.);
    }
    int i;
    if (xr_mode) {
        out_xm[1] = cx(1., 0.); out_xe[1] = 0;
        for (i = 2; i < valid; i++) {
            xc prev = xc_make(out_xm[i - 1].x, out_xm[i - 1].y, out_xe[i - 1]);
            xc v = xr_mul(mn_dfdz_x(R.nexp, orbit_xr(R, i - 1)), prev);
            out_xm[i] = cx(v.re, v.im); out_xe[i] = v.e;
        }
        i -= 1;
        xc prev = xc_make(out_xm[i].x, out_xm[i].y, out_xe[i]);
        xc v = xr_mul(mn_dfdz_x(R.nexp, orbit_xr(R, i)), prev);
        out_xm[len] = cx(v.re, v.im); out_xe[len] = v.e;
    } else {
        out_std[1] = cx(1., 0.);
        for (i = 2; i < valid; i++) out_std[i] = cmul(mn_dfdz(R.nexp, R.Zn[i - 1]), out_std[i - 1]);
        i -= 1;
        out_std[len] = cmul(mn_dfdz(R.nexp, R.Zn[i]), out_std[i]);
    }
}

__device__ __forceinline__ double sgnr(double x) { return x < 0. ? -1. : 1.; }

// models/burning_ship.py:441-532
__device__ __forceinline__ void bs_dfdxy(int flavor, double x, double y, double &fxx, double &fxy,
                                         double &fyx, double &fyy) {
    if (flavor == 1) { fxx = 2. * x; fxy = -2. * y; fyx = 2. * sgnr(x) * fabs(y); fyy = 2. * sgnr(y) * fabs(x); }
    else if (flavor == 2) { fxx = 2. * x; fxy = -2. * y; fyx = 2. * fabs(y); fyy = 2. * sgnr(y) * x; }
    else if (flavor == 3) { fxx = 2. * x; fxy = -2. * fabs(y); fyx = 2. * y; fyy = 2. * x; }
    else if (flavor == 4) { double q = x * x - y * y; fxx = 2. * sgnr(q) * x; fxy = -2. * sgnr(q) * y; fyx = 2. * y; fyy = 2. * x; }
    else { double q = x * x - y * y; fxx = 2. * sgnr(q) * x; fxy = -2. * sgnr(q) * y;
           fyx = 2. * sgnr(x) * fabs(y); fyy = 2. * sgnr(y) * fabs(x); }
}

__global__ void k_dzndc_bs(const RefDev *Rp, double *dXa, double *dXb, double *dYa, double *dYb,
                           double scale) {
    const RefDev &R = *Rp;
    int len = R.len;
    int valid = len < R.div_iter ? len : R.div_iter;
    for (int k = 0; k <= len; k++) { dXa[k] = 0.; dXb[k] = 0.; dYa[k] = 0.; dYb[k] = 0.; }
    for (int i = 1; i <= valid; i++) {
        int from = i - 1, to = i;
        if (i == valid) {
            if (!(from == R.order - 1)) break;
            to = 0;
        }
        double fxx, fxy, fyx, fyy;
        bs_dfdxy(R.flavor, R.Zn[from].x, R.Zn[from].y, fxx, fxy, fyx, fyy);
        double a = dXa[from], b = dXb[from], c = dYa[from], d = dYb[from];
        dXa[to] = fxx * a + fxy * c + scale;
        dXb[to] = fxx * b + fxy * d;
        dYa[to] = fyx * a + fyy * c;
        dYb[to] = fyx * b + fyy * d - scale;
    }
}

// ---------------------------------------------------------------------------
// BLA tree
// ---------------------------------------------------------------------------
__device__ __forceinline__ int bla_index(int i, int stg) { return 2 * i + ((1 << stg) - 1); }

// Python max / min semantics (first argument wins ties), as in combine_BLA
__device__ __forceinline__ double radius_combine(double r1, double r2, double mA1, double mB1,
                                                 double kc, double eps) {
    double num = r2 - mB1 * kc, den = (eps > mA1) ? eps : mA1;
    double q = num / den;
    double r2b = 0.95 * ((q > 0.) ? q : 0.);
    return (r2b < r1) ? r2b : r1;
}

__device__ __forceinline__ void combine_m2(double2 *M, double *r, int i1, int i2, int ir,
                                           double kc, double eps) {
    double2 A1 = M[2 * i1], B1 = M[2 * i1 + 1], A2 = M[2 * i2], B2 = M[2 * i2 + 1];
    M[2 * ir] = cmul(A2, A1);
    M[2 * ir + 1] = cadd(cmul(A2, B1), B2);
    r[ir] = radius_combine(r[i1], r[i2], hypot(A1.x, A1.y), hypot(B1.x, B1.y), kc, eps);
}

__global__ void k_bla_leaf_m2(const RefDev *Rp, double2 *M, double *r, int L, double kc,
                              double eps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L) return;
    const RefDev &R = *Rp;
    double2 tM[32]; double tr[16];
    for (int j = 0; j < 16; j++) { tM[2 * j] = cx(0., 0.); tM[2 * j + 1] = cx(0., 0.); tr[j] = 0.; }
    for (int j = 0; j < 8; j++) {
        double2 A = mn_dfdz(R.nexp, R.Zn[8 * i + j]);
        tM[4 * j] = A; tM[4 * j + 1] = cx(1., 0.);
        tr[2 * j] = eps * hypot(A.x, A.y);
    }
    for (int stg = 1; stg <= 3; stg++) {
        int step = 1 << stg;
        for (int k = 0; k < 8 - step + 1; k += step) {
            int kk = k + step / 2;
            combine_m2(tM, tr, bla_index(k, stg - 1), bla_index(kk, stg - 1), bla_index(k, stg), kc, eps);
        }
    }
    M[4 * i] = tM[14]; M[4 * i + 1] = tM[15];
    r[2 * i] = tr[7];
}

__global__ void k_bla_level_m2(double2 *M, double *r, int L, int stg, double kc, double eps) {
    int step = 1 << stg;
    int i = (blockIdx.x * blockDim.x + threadIdx.x) * step;
    if (i > L - step) return;
    int ii = i + step / 2;
    if (ii >= L) return;
    combine_m2(M, r, bla_index(i, stg - 1), bla_index(ii, stg - 1), bla_index(i, stg), kc, eps);
}

__device__ __forceinline__ void combine_bs(double *M, double *r, int i1, int i2, int ir, double kc,
                                           double eps) {
    const double *m1 = M + 8 * i1, *m2 = M + 8 * i2;
    double *mr = M + 8 * ir;
    double a0 = m2[0] * m1[0] + m2[1] * m1[2];
    double a1 = m2[0] * m1[1] + m2[1] * m1[3];
    double a2 = m2[2] * m1[0] + m2[3] * m1[2];
    double a3 = m2[2] * m1[1] + m2[3] * m1[3];
    double b0 = m2[0] * m1[4] + m2[1] * m1[6] + m2[4];
    double b1 = m2[0] * m1[5] + m2[1] * m1[7] + m2[5];
    double b2 = m2[2] * m1[4] + m2[3] * m1[6] + m2[6];
    double b3 = m2[2] * m1[5] + m2[3] * m1[7] + m2[7];
    double mA1 = fmax(fmax(fabs(m1[0]), fabs(m1[1])), fmax(fabs(m1[2]), fabs(m1[3])));
    double mB1 = fmax(fmax(fabs(m1[4]), fabs(m1[5])), fmax(fabs(m1[6]), fabs(m1[7])));
    double rr = radius_combine(r[i1], r[i2], mA1, mB1, kc, eps);
    mr[0] = a0; mr[1] = a1; mr[2] = a2; mr[3] = a3;
    mr[4] = b0; mr[5] = b1; mr[6] = b2; mr[7] = b3;
    r[ir] = rr;
}

__global__ void k_bla_leaf_bs(const RefDev *Rp, double *M, double *r, int L, double kc,
                              double eps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L) return;
    const RefDev &R = *Rp;
    double tM[16 * 8]; double tr[16];
    for (int j = 0; j < 16 * 8; j++) tM[j] = 0.;
    for (int j = 0; j < 16; j++) tr[j] = 0.;
    for (int j = 0; j < 8; j++) {
        double x = R.Zn[8 * i + j].x, y = R.Zn[8 * i + j].y;
        double *t = tM + 8 * (2 * j);
        bs_dfdxy(R.flavor, x, y, t[0], t[1], t[2], t[3]);
        t[4] = 1.; t[5] = 0.; t[6] = 0.; t[7] = -1.;
        tr[2 * j] = eps * fmin(fabs(x), fabs(y));
    }
    for (int stg = 1; stg <= 3; stg++) {
        int step = 1 << stg;
        for (int k = 0; k < 8 - step + 1; k += step) {
            int kk = k + step / 2;
            combine_bs(tM, tr, bla_index(k, stg - 1), bla_index(kk, stg - 1), bla_index(k, stg), kc, eps);
        }
    }
    for (int d = 0; d < 8; d++) M[8 * (2 * i) + d] = tM[8 * 7 + d];
    r[2 * i] = tr[7];
}

__global__ void k_bla_level_bs(double *M, double *r, int L, int stg, double kc, double eps) {
    int step = 1 << stg;
    int i = (blockIdx.x * blockDim.x + threadIdx.x) * step;
    if (i > L - step) return;
    int ii = i + step / 2;
    if (ii >= L) return;
    combine_bs(M, r, bla_index(i, stg - 1), bla_index(ii, stg - 1), bla_index(i, stg), kc, eps);
}

// ---------------------------------------------------------------------------
// fe tables
// ---------------------------------------------------------------------------
__device__ __forceinline__ int4 pack_fe(fe v) {
    fe n = fe_norm(v);
    return make_int4(__float_as_int(n.x), __float_as_int(n.y), n.e, n.e);
}

__global__ void k_fe_orbit(const RefDev *Rp, int4 *Zf) {
    const RefDev &R = *Rp;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > R.len) return;
    int slot = (R.n_xr && i < R.len) ? R.xr_slot[i] : -1;
    fe v = (slot >= 0) ? fe_from_xc(xc_make(R.xr_m[slot].x, R.xr_m[slot].y, R.xr_e[slot]))
                       : fe_from_d(R.Zn[i]);
    Zf[i] = pack_fe(v);
}

// plain-float copy of 2 Z for the fast steps, with the fast-step limit (the
// exponent of max(|Z.x|, |Z.y|) minus 26); values below 2^-100 or above 2^100
// get FE_ZERO_E so that the kernel takes its exact path there, and exact zeros
// are flagged (w = 1)
__global__ void k_plain_orbit(const RefDev *Rp, const int4 *Zf, int4 *Zp) {
    const RefDev &R = *Rp;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > R.len) return;
    int4 f = Zf[i];
    if (f.z == FE_ZERO_E || f.z < -100 || f.z > 100) {
        // flag 1: the orbit value is exactly 0 (no Xrange entry either)
        bool zero = (f.z == FE_ZERO_E) && R.Zn[i].x == 0. && R.Zn[i].y == 0.
                    && !(R.n_xr && i < R.len && R.xr_slot[i] >= 0);
        Zp[i] = make_int4(0, 0, FE_ZERO_E, zero ? 1 : 0);
        return;
    }
    float s = __int_as_float((f.z + 128) << 23);   // 2^(e + 1), e in [-100, 100]
    float x = __int_as_float(f.x) * s, y = __int_as_float(f.y) * s;
    Zp[i] = make_int4(__float_as_int(x), __float_as_int(y), f.z - 26, 0);
}

__global__ void k_fe_path(const double2 *std_p, const double2 *xm, const int *xe, int n,
                          int4 *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fe v = xm ? fe_from_xc(xc_make(xm[i].x, xm[i].y, xe[i])) : fe_from_d(std_p[i]);
    out[i] = pack_fe(v);
}

__global__ void k_fe_bla(const double2 *M, const double *r, int n, int4 *F) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fe a = fe_norm(fe_from_d(M[2 * i])), b = fe_norm(fe_from_d(M[2 * i + 1]));
    // r as (mantissa in [1, 2), exponent); r = 0 -> exponent FE_ZERO_E
    fe rf = fe_norm(fe_from_d(cx(r[i], 0.)));
    F[2 * i] = make_int4(__float_as_int(rf.x), rf.e, a.e, b.e);
    F[2 * i + 1] = make_int4(__float_as_int(a.x), __float_as_int(a.y), __float_as_int(b.x),
                             __float_as_int(b.y));
}

// the first stage ref_BLA_get (perturbation.py:2116-2170) tries at each start
// index it = w / 8: 3 + ctz(it) capped at stages - 1 (stages - 1 for it = 0),
// lowered to the largest stage whose step is below first_invalid - w; its
// bla_f record is copied beside it so that the kernel's first test needs one
// load
__global__ void k_fe_bla_first(const RefDev *Rp, const int4 *F, int nit, int4 *FF, int *FS) {
    const RefDev &R = *Rp;
    int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nit) return;
    const int inv = R.first_invalid - (it << 3);
    int4 h = make_int4(0, FE_ZERO_E, 0, 0), p = make_int4(0, 0, 0, 0);
    int step = 0;
    if (inv > 8 && R.stages - 1 >= 3) {
        int top = R.stages - 1;
        if (it != 0) top = min(top, 3 + __ffs(it) - 1);
        top = min(top, 31 - __clz(inv - 1));
        if (top >= 3) {
            const int idx = 2 * it + (1 << (top - 3)) - 1;
            if (idx < R.bla_len) { h = F[2 * idx]; p = F[2 * idx + 1]; step = 1 << top; }
        }
    }
    FF[2 * it] = h; FF[2 * it + 1] = p; FS[it] = step;
}

// ---------------------------------------------------------------------------
// Burning Ship FP32+exp tables (fr pairs, fsg_bs.cuh)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int2 fr_pack(fr v) { return make_int2(__float_as_int(v.m), v.e); }
__device__ __forceinline__ fr fr_of_xr(double m, int e) {
    fr r = fr_from_d(m);
    if (r.m != 0.f) r.e += e;
    return r;
}
// orbit values, from the Xrange side table where the orbit holds one
// (values below the double range, FP_loop.pyx:1828-1979)
__global__ void k_bs_fr_orbit(const RefDev *Rp, int4 *out) {
    const RefDev &R = *Rp;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > R.len) return;
    fr x, y;
    int s = (R.n_xr > 0 && i < R.len) ? R.xr_slot[i] : -1;
    if (s >= 0) {
        // planar layout: x mantissas / exponents, then y
        const double *m = (const double *)R.xr_m;
        x = fr_of_xr(m[s], R.xr_e[s]);
        y = fr_of_xr(m[R.n_xr + s], R.xr_e[R.n_xr + s]);
    }
    else { x = fr_from_d(R.Zn[i].x); y = fr_from_d(R.Zn[i].y); }
    int2 a = fr_pack(x), b = fr_pack(y);
    out[i] = make_int4(a.x, a.y, b.x, b.y);
}
__global__ void k_bs_fr_paths(const double *dXa, const double *dXb, const double *dYa,
                              const double *dYb, int n, int4 *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int2 a = fr_pack(fr_from_d(dXa[i])), b = fr_pack(fr_from_d(dXb[i]));
    int2 c = fr_pack(fr_from_d(dYa[i])), d = fr_pack(fr_from_d(dYb[i]));
    out[2 * i] = make_int4(a.x, a.y, b.x, b.y);
    out[2 * i + 1] = make_int4(c.x, c.y, d.x, d.y);
}
__global__ void k_bs_fr_bla(const double *M, int n, int4 *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * n) return;
    int2 a = fr_pack(fr_from_d(M[2 * i])), b = fr_pack(fr_from_d(M[2 * i + 1]));
    out[i] = make_int4(a.x, a.y, b.x, b.y);
}

void fsg_build_bs_fr(const RefDev *Rd, int len, int4 *Zf, const double *dXa, const double *dXb,
                     const double *dYa, const double *dYb, int4 *hf, cudaStream_t s) {
    int tb = 256;
    k_bs_fr_orbit<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(Rd, Zf);
    if (hf) k_bs_fr_paths<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(dXa, dXb, dYa, dYb, len + 1, hf);
}
void fsg_build_bs_fr_bla(const double *Mbs, int bla_len, int4 *blaf, cudaStream_t s) {
    int tb = 256;
    if (blaf && bla_len > 0) k_bs_fr_bla<<<(4 * bla_len + tb - 1) / tb, tb, 0, s>>>(Mbs, bla_len, blaf);
}

// ---------------------------------------------------------------------------
// host-side launchers (called by the C-ABI layer)
// ---------------------------------------------------------------------------
void fsg_build_paths_m2(const RefDev *Rd, double2 *dzndc, double2 *dzndc_xm, int *dzndc_xe,
                        double2 *dzndz, double2 *dzndz_xm, int *dzndz_xe, int xr_mode,
                        int want_dzndc, int want_dzndz, double scale_m, int scale_e,
                        cudaStream_t s) {
    if (want_dzndc) k_dzndc_m2<<<1, 1, 0, s>>>(Rd, dzndc, dzndc_xm, dzndc_xe, xr_mode, scale_m, scale_e);
    if (want_dzndz) k_dzndz_m2<<<1, 1, 0, s>>>(Rd, dzndz, dzndz_xm, dzndz_xe, xr_mode);
}

void fsg_build_paths_bs(const RefDev *Rd, double *dXa, double *dXb, double *dYa, double *dYb,
                        double scale, cudaStream_t s) {
    k_dzndc_bs<<<1, 1, 0, s>>>(Rd, dXa, dXb, dYa, dYb, scale);
}

void fsg_build_bla(const RefDev *Rd, int flavor, int len, double2 *M2, double *Mbs, double *r,
                   int stages, double kc, double eps, cudaStream_t s) {
    int L = len / 8;
    if (L <= 0) return;
    int tb = 128;
    if (flavor == 0) {
        k_bla_leaf_m2<<<(L + tb - 1) / tb, tb, 0, s>>>(Rd, M2, r, L, kc, eps);
        for (int stg = 1; stg < stages - 3; stg++) {
            int n = L >> stg;
            if (n <= 0) break;
            k_bla_level_m2<<<(n + tb - 1) / tb, tb, 0, s>>>(M2, r, L, stg, kc, eps);
        }
    } else {
        k_bla_leaf_bs<<<(L + tb - 1) / tb, tb, 0, s>>>(Rd, Mbs, r, L, kc, eps);
        for (int stg = 1; stg < stages - 3; stg++) {
            int n = L >> stg;
            if (n <= 0) break;
            k_bla_level_bs<<<(n + tb - 1) / tb, tb, 0, s>>>(Mbs, r, L, stg, kc, eps);
        }
    }
}

void fsg_build_plain_orbit(const RefDev *Rd, int len, const int4 *Zf, int4 *Zp, cudaStream_t s) {
    int tb = 256;
    k_plain_orbit<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(Rd, Zf, Zp);
}

void fsg_build_fe_bla(const RefDev *Rd, const double2 *Mbla, const double *rbla, int bla_len,
                      int4 *bla_f, int bla_nit, int4 *bla_first, int *bla_first_step,
                      cudaStream_t s);

void fsg_build_fe_tables(const RefDev *Rd, int len, int4 *Zf, const double2 *dzndc,
                         const double2 *dzndc_xm, const int *dzndc_xe, int4 *dzndc_f,
                         const double2 *dzndz, const double2 *dzndz_xm, const int *dzndz_xe,
                         int4 *dzndz_f, const double2 *Mbla, const double *rbla, int bla_len,
                         int4 *bla_f, int bla_nit, int4 *bla_first, int *bla_first_step,
                         cudaStream_t s) {
    int tb = 256;
    k_fe_orbit<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(Rd, Zf);
    if (dzndc_f) k_fe_path<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(dzndc, dzndc_xm, dzndc_xe, len + 1, dzndc_f);
    if (dzndz_f) k_fe_path<<<(len + 2 + tb - 1) / tb, tb, 0, s>>>(dzndz, dzndz_xm, dzndz_xe, len + 2, dzndz_f);
    fsg_build_fe_bla(Rd, Mbla, rbla, bla_len, bla_f, bla_nit, bla_first, bla_first_step, s);
}

void fsg_build_fe_bla(const RefDev *Rd, const double2 *Mbla, const double *rbla, int bla_len,
                      int4 *bla_f, int bla_nit, int4 *bla_first, int *bla_first_step,
                      cudaStream_t s) {
    int tb = 256;
    if (bla_f && bla_len > 0) {
        k_fe_bla<<<(bla_len + tb - 1) / tb, tb, 0, s>>>(Mbla, rbla, bla_len, bla_f);
        k_fe_bla_first<<<(bla_nit + tb - 1) / tb, tb, 0, s>>>(Rd, bla_f, bla_nit, bla_first,
                                                              bla_first_step);
    }
}
