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

// The orbit fields the sequential loops read, held in registers: the loops
// store into the paths, which the compiler cannot prove apart from the
// descriptor, so reading them through it would reload them every step
struct OrbitView {
    const double2 *__restrict__ Zn;
    const int *__restrict__ xr_slot;
    const double2 *__restrict__ xr_m;
    const int *__restrict__ xr_e;
    int n_xr, nexp;
    __device__ __forceinline__ explicit OrbitView(const RefDev &R)
        : Zn(R.Zn), xr_slot(R.xr_slot), xr_m(R.xr_m), xr_e(R.xr_e), n_xr(R.n_xr), nexp(R.nexp) {}
    __device__ __forceinline__ xc xr(int i) const {
        int slot = n_xr ? xr_slot[i] : -1;
        if (slot >= 0) return xc_make(xr_m[slot].x, xr_m[slot].y, xr_e[slot]);
        return xr_from(Zn[i]);
    }
};

// Sequential form (orbits up to FSG_PATH_SCAN_MIN = 8192 points): one thread, the
// reference's order, the previous value carried in registers.  The paths are
// zero-filled by the host (cudaMemsetAsync) before the launch.
__global__ void k_dzndc_m2(const RefDev *Rp, double2 *__restrict__ out_std,
                           double2 *__restrict__ out_xm, int *__restrict__ out_xe,
                           int xr_mode, double scale_m, int scale_e) {
    const RefDev &R = *Rp;
    const OrbitView O(R);
    const int len = R.len, order = R.order, nexp = O.nexp;
    const int valid = len < R.div_iter ? len : R.div_iter;
    int i;
    if (xr_mode) {
        const xc sc = xc_make(scale_m, 0., scale_e);
        xc prev = xc_zero();
        for (i = 1; i < valid; i++) {
            xc v = xr_add(xr_mul(mn_dfdz_x(nexp, O.xr(i - 1)), prev), sc);
            out_xm[i] = cx(v.re, v.im); out_xe[i] = v.e;
            prev = v;
        }
        i -= 1;
        if (i == order - 1) {
            xc v = xr_add(xr_mul_s(mn_dfdz(nexp, O.Zn[i]), prev), sc);
            out_xm[0] = cx(v.re, v.im); out_xe[0] = v.e;
        }
    } else {
        const double scale = ldexp_d(scale_m, scale_e);
        double2 prev = cx(0., 0.);
        double2 znext = O.Zn[0];
        for (i = 1; i < valid; i++) {
            const double2 z = znext;
            znext = O.Zn[i];
            prev = caddr(cmul(mn_dfdz(nexp, z), prev), scale);
            out_std[i] = prev;
        }
        i -= 1;
        if (i == order - 1) out_std[0] = caddr(cmul(mn_dfdz(nexp, O.Zn[i]), prev), scale);
    }
}

__global__ void k_dzndz_m2(const RefDev *Rp, double2 *__restrict__ out_std,
                           double2 *__restrict__ out_xm, int *__restrict__ out_xe, int xr_mode) {
    const RefDev &R = *Rp;
    const OrbitView O(R);
    const int len = R.len, nexp = O.nexp;
    const int valid = len < R.div_iter ? len : R.div_iter;
    int i;
    if (xr_mode) {
        out_xm[1] = cx(1., 0.); out_xe[1] = 0;
        xc prev = xc_make(1., 0., 0);
        for (i = 2; i < valid; i++) {
            xc v = xr_mul(mn_dfdz_x(nexp, O.xr(i - 1)), prev);
            out_xm[i] = cx(v.re, v.im); out_xe[i] = v.e;
            prev = v;
        }
        i -= 1;          // >= 1: prev holds the path at i
        xc v = xr_mul(mn_dfdz_x(nexp, O.xr(i)), prev);
        out_xm[len] = cx(v.re, v.im); out_xe[len] = v.e;
    } else {
        out_std[1] = cx(1., 0.);
        double2 prev = cx(1., 0.);
        double2 znext = O.Zn[1];
        for (i = 2; i < valid; i++) {
            const double2 z = znext;
            znext = O.Zn[i];
            prev = cmul(mn_dfdz(nexp, z), prev);
            out_std[i] = prev;
        }
        i -= 1;          // >= 1: prev holds the path at i
        out_std[len] = cmul(mn_dfdz(nexp, O.Zn[i]), prev);
    }
}

// ---------------------------------------------------------------------------
// Chunked scan of the same recurrences for long orbits.  D_i = a_i D_{i-1}
// + s (dZndc; s = 0 for dZndz) is affine: each chunk of FSG_PATH_CHUNK
// indices is composed into D -> A D + B (Xrange, so no product of a chunk
// overflows), a single thread chains the chunks to get every chunk's start
// value, then every chunk is replayed from its start value with the
// reference's per-step operations.  Results differ from the sequential form
// only through the chunks' start values (a few ulps).
// ---------------------------------------------------------------------------
#define FSG_PATH_CHUNK 256

struct PathScan {
    int first, end;            // indices [first, end) computed by the recurrence
    int nchunks;
    xc *A, *B, *start;         // [nchunks]
};

// a_i = df/dz(Z_{i-1}) as an Xrange value
__device__ __forceinline__ xc path_a(const RefDev &R, int i, int xr_mode) {
    return xr_mode ? mn_dfdz_x(R.nexp, orbit_xr(R, i - 1)) : xr_from(mn_dfdz(R.nexp, R.Zn[i - 1]));
}

__global__ void k_path_compose(const RefDev *Rp, PathScan P, int xr_mode, int affine, xc s) {
    const RefDev &R = *Rp;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.nchunks) return;
    const int lo = P.first + c * FSG_PATH_CHUNK;
    const int hi = min(lo + FSG_PATH_CHUNK, P.end);
    xc A = xc_make(1., 0., 0), B = xc_zero();
    for (int i = lo; i < hi; i++) {
        const xc a = path_a(R, i, xr_mode);
        A = xr_mul(a, A);
        B = affine ? xr_add(xr_mul(a, B), s) : xr_mul(a, B);
    }
    P.A[c] = A; P.B[c] = B;
}

__global__ void k_path_prefix(PathScan P, xc d0) {
    xc D = d0;
    for (int c = 0; c < P.nchunks; c++) {
        P.start[c] = D;
        D = xr_add(xr_mul(P.A[c], D), P.B[c]);
    }
}

__global__ void k_path_fill(const RefDev *Rp, PathScan P, int xr_mode, int affine, double scale_m,
                            int scale_e, double2 *out_std, double2 *out_xm, int *out_xe) {
    const RefDev &R = *Rp;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.nchunks) return;
    const int lo = P.first + c * FSG_PATH_CHUNK;
    const int hi = min(lo + FSG_PATH_CHUNK, P.end);
    if (xr_mode) {
        const xc sc = xc_make(scale_m, 0., scale_e);
        xc prev = P.start[c];
        for (int i = lo; i < hi; i++) {
            const xc a = mn_dfdz_x(R.nexp, orbit_xr(R, i - 1));
            prev = affine ? xr_add(xr_mul(a, prev), sc) : xr_mul(a, prev);
            out_xm[i] = cx(prev.re, prev.im); out_xe[i] = prev.e;
        }
    } else {
        const double scale = ldexp_d(scale_m, scale_e);
        double2 prev = xr_to_std(P.start[c]);
        for (int i = lo; i < hi; i++) {
            const double2 a = mn_dfdz(R.nexp, R.Zn[i - 1]);
            prev = affine ? caddr(cmul(a, prev), scale) : cmul(a, prev);
            out_std[i] = prev;
        }
    }
}

// the wrapped values at the end of the scanned paths (sequential form's tails)
__global__ void k_dzndc_tail(const RefDev *Rp, double2 *out_std, double2 *out_xm, int *out_xe,
                             int xr_mode, double scale_m, int scale_e) {
    const RefDev &R = *Rp;
    const int valid = R.len < R.div_iter ? R.len : R.div_iter;
    const int i = valid - 1;
    if (i != R.order - 1) return;
    if (xr_mode) {
        xc prev = xc_make(out_xm[i].x, out_xm[i].y, out_xe[i]);
        xc v = xr_add(xr_mul_s(mn_dfdz(R.nexp, R.Zn[i]), prev), xc_make(scale_m, 0., scale_e));
        out_xm[0] = cx(v.re, v.im); out_xe[0] = v.e;
    } else {
        out_std[0] = caddr(cmul(mn_dfdz(R.nexp, R.Zn[i]), out_std[i]), ldexp_d(scale_m, scale_e));
    }
}

__global__ void k_dzndz_tail(const RefDev *Rp, double2 *out_std, double2 *out_xm, int *out_xe,
                             int xr_mode) {
    const RefDev &R = *Rp;
    const int len = R.len;
    const int valid = len < R.div_iter ? len : R.div_iter;
    const int i = valid - 1 > 1 ? valid - 1 : 1;
    if (xr_mode) {
        out_xm[1] = cx(1., 0.); out_xe[1] = 0;
        xc prev = xc_make(out_xm[i].x, out_xm[i].y, out_xe[i]);
        xc v = xr_mul(mn_dfdz_x(R.nexp, orbit_xr(R, i)), prev);
        out_xm[len] = cx(v.re, v.im); out_xe[len] = v.e;
    } else {
        out_std[1] = cx(1., 0.);
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

__global__ void k_dzndc_bs(const RefDev *Rp, double *__restrict__ dXa, double *__restrict__ dXb,
                           double *__restrict__ dYa, double *__restrict__ dYb, double scale) {
    const RefDev &R = *Rp;
    const double2 *__restrict__ Zn = R.Zn;
    const int len = R.len, flavor = R.flavor, order = R.order;
    const int valid = len < R.div_iter ? len : R.div_iter;
    double a = 0., b = 0., c = 0., d = 0.;       // the Jacobian at index i - 1 (zero-filled path)
    for (int i = 1; i <= valid; i++) {
        int from = i - 1, to = i;
        if (i == valid) {
            if (!(from == order - 1)) break;
            to = 0;
        }
        double fxx, fxy, fyx, fyy;
        bs_dfdxy(flavor, Zn[from].x, Zn[from].y, fxx, fxy, fyx, fyy);
        const double na = fxx * a + fxy * c + scale;
        const double nb = fxx * b + fxy * d;
        const double nc = fyx * a + fyy * c;
        const double nd = fyx * b + fyy * d - scale;
        dXa[to] = na; dXb[to] = nb; dYa[to] = nc; dYb[to] = nd;
        a = na; b = nb; c = nc; d = nd;
    }
}

// numba_dZndc_path_BS, Xrange branch (perturbation.py:2339-2438): the
// Jacobian path as float64 Xrange records from the orbit's Xrange values
// (ensure_xr_BS: the side table's value where the orbit holds one), with the
// derivatives of burning_ship.py:441-532 on records -- the float factors
// (2., the signs) first, as the reference's 2. * sgn(x) * abs(y)
__device__ __forceinline__ double sgn_x(xf x) { return xf_lt_s(x, 0.) ? -1. : 1.; }
__device__ __forceinline__ xf abs_x(xf x) { x.m = fabs(x.m); return x; }
__device__ __forceinline__ void bs_dfdxy_x(int flavor, xf x, xf y, xf &fxx, xf &fxy, xf &fyx,
                                           xf &fyy) {
    if (flavor == 1) {
        fxx = xf_mul_s(2., x); fxy = xf_mul_s(-2., y);
        fyx = xf_mul_s(2. * sgn_x(x), abs_x(y)); fyy = xf_mul_s(2. * sgn_x(y), abs_x(x));
    } else if (flavor == 2) {
        fxx = xf_mul_s(2., x); fxy = xf_mul_s(-2., y);
        fyx = xf_mul_s(2., abs_x(y)); fyy = xf_mul_s(2. * sgn_x(y), x);
    } else if (flavor == 3) {
        fxx = xf_mul_s(2., x); fxy = xf_mul_s(-2., abs_x(y));
        fyx = xf_mul_s(2., y); fyy = xf_mul_s(2., x);
    } else {
        const double sq = sgn_x(xf_sub(xf_mul(x, x), xf_mul(y, y)));
        fxx = xf_mul_s(2. * sq, x); fxy = xf_mul_s(-2. * sq, y);
        if (flavor == 4) { fyx = xf_mul_s(2., y); fyy = xf_mul_s(2., x); }
        else { fyx = xf_mul_s(2. * sgn_x(x), abs_x(y)); fyy = xf_mul_s(2. * sgn_x(y), abs_x(x)); }
    }
}

__global__ void k_dzndc_bs_xr(const RefDev *Rp, double *__restrict__ pm, int *__restrict__ pe,
                              double scale_m, int scale_e) {
    const RefDev &R = *Rp;
    const int len = R.len, flavor = R.flavor, order = R.order, L = len + 1;
    const int valid = len < R.div_iter ? len : R.div_iter;
    const xf dx = xf_make(scale_m, scale_e);
    const double *tm = (const double *)R.xr_m;
    xf a = xf_make(0., 0), b = a, c = a, d = a;   // the Jacobian at index i - 1
    for (int i = 1; i <= valid; i++) {
        int from = i - 1, to = i;
        if (i == valid) {
            if (!(from == order - 1)) break;
            to = 0;
        }
        const int s = (R.n_xr > 0 && from < len) ? R.xr_slot[from] : -1;
        const xf X = s >= 0 ? xf_make(tm[s], R.xr_e[s]) : xr_from_r(R.Zn[from].x);
        const xf Y = s >= 0 ? xf_make(tm[R.n_xr + s], R.xr_e[R.n_xr + s]) : xr_from_r(R.Zn[from].y);
        xf fxx, fxy, fyx, fyy;
        bs_dfdxy_x(flavor, X, Y, fxx, fxy, fyx, fyy);
        const xf na = xf_add(xf_add(xf_mul(fxx, a), xf_mul(fxy, c)), dx);
        const xf nb = xf_add(xf_mul(fxx, b), xf_mul(fxy, d));
        const xf nc = xf_add(xf_mul(fyx, a), xf_mul(fyy, c));
        const xf nd = xf_sub(xf_add(xf_mul(fyx, b), xf_mul(fyy, d)), dx);
        pm[to] = na.m; pe[to] = na.e; pm[L + to] = nb.m; pe[L + to] = nb.e;
        pm[2 * L + to] = nc.m; pe[2 * L + to] = nc.e; pm[3 * L + to] = nd.m; pe[3 * L + to] = nd.e;
        a = na; b = nb; c = nc; d = nd;
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

// Composed runs of fast steps.  While |dz| < 2^-26 |Z| a fast step is affine
// (perturbation.py:1158-1214 with the dz^2 term below FP32 resolution):
// u' = 2Z u + c and v' = 2Z v + 2 D u (D the reference dZndc), so the k steps
// from w to the next multiple of 8 (a BLA attempt point) compose to
// U = P U0 + Q c and V = P V0 + R U0 + S c.  The entry also bounds the run:
// every intermediate U_j = P_j U0 + Q_j c stays below 2^(Zp.z) (the fast-step
// limit at w + j) when a |U0| + b |c| < 1/2, with a = max_j |P_j| 2^-Zp.z and
// b = max_j |Q_j| 2^-Zp.z; and the largest |2 Z|^2 the run's escape tests read.
// Products in double from the float 2Z of Zp and the fe values of dZndc (an
// exponent kept beside the R and S mantissas).  Not composable: runs of one
// step, past len, or through an orbit value outside the float range.
__device__ __forceinline__ void runs_acc(double2 &m, int &e, double2 t, int te) {
    // m 2^e += t 2^te
    if (t.x == 0. && t.y == 0.) return;
    if (m.x == 0. && m.y == 0.) { m = t; e = te; return; }
    if (te > e) { m = cx(ldexp(m.x, e - te), ldexp(m.y, e - te)); e = te; }
    else t = cx(ldexp(t.x, te - e), ldexp(t.y, te - e));
    m = cadd(m, t);
}
__device__ __forceinline__ void runs_norm(double2 &m, int &e) {
    const double a = fmax(fabs(m.x), fabs(m.y));
    if (a == 0.) { e = FE_ZERO_E; return; }
    int k;
    frexp(a, &k);
    m = cx(ldexp(m.x, -k), ldexp(m.y, -k));
    e += k;
}
__device__ __forceinline__ int4 runs_pack2(double2 m, int e, int e2) {
    return make_int4(__float_as_int((float)m.x), __float_as_int((float)m.y), e, e2);
}
__global__ void k_fe_runs(const RefDev *Rp, const int4 *Zp, const int4 *Df, int len, int4 *out) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w > len) return;
    int4 *o = out + 5 * (size_t)w;
    const int k = 8 - (w & 7);
    bool ok = k >= 2 && w + k <= len;
    double2 P = cx(1., 0.), Q = cx(0., 0.), Rm = cx(0., 0.), Sm = cx(0., 0.);
    int eR = 0, eS = 0;
    double amax = 0., bmax = 0., z2max = 0.;
    for (int j = 0; j < k && ok; j++) {
        const int4 z = Zp[w + j];
        if (z.z == FE_ZERO_E) { ok = false; break; }
        const double sc = ldexp(1., -z.z);
        amax = fmax(amax, hypot(P.x, P.y) * sc);
        bmax = fmax(bmax, hypot(Q.x, Q.y) * sc);
        const double2 T = cx((double)__int_as_float(z.x), (double)__int_as_float(z.y));
        if (j >= 1) z2max = fmax(z2max, T.x * T.x + T.y * T.y);
        if (Df) {
            const int4 d = Df[w + j];
            if (d.z != FE_ZERO_E) {
                const double2 D2 = cx(2. * (double)__int_as_float(d.x), 2. * (double)__int_as_float(d.y));
                Rm = cmul(T, Rm);
                Sm = cmul(T, Sm);
                runs_acc(Rm, eR, cmul(D2, P), d.z);
                runs_acc(Sm, eS, cmul(D2, Q), d.z);
            } else {
                Rm = cmul(T, Rm);
                Sm = cmul(T, Sm);
            }
            runs_norm(Rm, eR);
            if (eR == FE_ZERO_E) eR = 0;
            runs_norm(Sm, eS);
            if (eS == FE_ZERO_E) eS = 0;
        }
        P = cmul(T, P);
        Q = cadd(cmul(T, Q), cx(1., 0.));
    }
    if (!ok) {
        o[4] = make_int4(0, 0, 0, 0);
        return;
    }
    int eP = 0, eQ = 0;
    runs_norm(P, eP);
    runs_norm(Q, eQ);
    const bool r0 = Rm.x == 0. && Rm.y == 0., s0 = Sm.x == 0. && Sm.y == 0.;
    o[0] = runs_pack2(P, eP, eQ);
    o[1] = make_int4(__float_as_int((float)Q.x), __float_as_int((float)Q.y),
                     __float_as_int((float)Rm.x), __float_as_int((float)Rm.y));
    o[2] = make_int4(r0 ? FE_ZERO_E : eR, s0 ? FE_ZERO_E : eS,
                     __float_as_int((float)Sm.x), __float_as_int((float)Sm.y));
    int ea = 0, eb = 0;
    const double ma = frexp(amax, &ea), mb = frexp(bmax, &eb);
    // the mantissas rounded up to float: the bound stays an upper bound
    o[3] = make_int4(__float_as_int(__double2float_ru(ma)), ea,
                     __float_as_int(__double2float_ru(mb)), eb);
    o[4] = make_int4(__float_as_int(__double2float_ru(z2max)), k, 0, 0);
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
    // r as (mantissa, exponent e); r = 0 -> mantissa 0, exponent FE_ZERO_E.
    // The mantissa is r 2^-e (1 - 2^-20) rounded down: with it the kernel's
    // FP32 test |u|^2 < rm^2 2^(2 (e - E)) (two roundings of at most 2^-23 on
    // the left, one of 2^-24 on the right) holds only where |dz| < r holds
    // exactly -- no BLA step beyond the FP64 radius; within 2^-19 of it the
    // step is declined and the iterations run as full steps
    fe rf = fe_norm(fe_from_d(cx(r[i], 0.)));
    float rm = 0.f;
    if (rf.e != FE_ZERO_E) {
        const double rr = (rf.e >= -1021 && rf.e <= 1021)
                              ? r[i] * pow2d(-rf.e) : (double)rf.x;
        rm = __double2float_rd(rr * (1. - 0x1p-20));
    }
    F[2 * i] = make_int4(__float_as_int(rm), rf.e, a.e, b.e);
    F[2 * i + 1] = make_int4(__float_as_int(a.x), __float_as_int(a.y), __float_as_int(b.x),
                             __float_as_int(b.y));
}

// the first stage ref_BLA_get (perturbation.py:2116-2170) tries at each start
// index it = w / 8: 3 + ctz(it) capped at stages - 1 (stages - 1 for it = 0),
// lowered to the largest stage whose step is below first_invalid - w; its
// bla_f record is copied beside it so that the kernel's first test needs one
// load.  Where stage 3 has radius 0 no stage of the index admits any dz
// (radii never grow with the stage, :2023-2024; 0 < r is strict): step 0, no
// lookup -- at the orbit's critical point Z_0 = 0 (A = 2 Z_0 = 0, r = 0) the
// search failed once per period
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
        if (top >= 3 && 2 * it < R.bla_len && F[2 * (2 * it)].x != 0) {
            const int idx = 2 * it + (1 << (top - 3)) - 1;
            if (idx < R.bla_len) { h = F[2 * idx]; p = F[2 * idx + 1]; step = 1 << top; }
        }
    }
    FF[2 * it] = h; FF[2 * it + 1] = p; FS[it] = step;
}

// |a| of an Xrange complex as a double (0 below, inf above the double range)
__device__ __forceinline__ double xabs_d(xc a) {
    if (a.re == 0. && a.im == 0.) return 0.;
    return ldexp_d(hypot(a.re, a.im), a.e);
}

// Chains of first BLA candidates.  A BLA step of ref_BLA_get ends on a
// multiple of 8, where the next attempt starts (perturbation.py:1121-1154),
// so when every first candidate (the largest admissible stage) is valid the
// reference takes a run of BLA steps with no full step between them.  Their
// composite dz -> P dz + Q dc (P = A_L .. A_1, Q = sum of A_L .. A_{j+1} B_j)
// is valid wherever each step is: with |dc| <= kc,
//   |dz_j| <= |P_j| |dz| + |Q_j| kc < r_j   for every j,
// that is |dz| < min_j (r_j - |Q_j| kc) / |P_j|.  The table holds, per start
// index, that radius times 0.9 (every step of the run then passes with a
// margin), P and Q as an fe record like the tree's, the run's iterations and
// its number of steps.  A run stops before a step that would cut the radius
// below a quarter of the shorter run's (a long run that rarely applies) and
// after 64 steps; runs of fewer than 2 steps are not stored.
__global__ void k_fe_bla_chain(const RefDev *Rp, const int *FS, int nit, double kc, int4 *CH,
                               int2 *CS) {
    const RefDev &R = *Rp;
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nit) return;
    xc P = xr_from(cx(1., 0.)), Q = xc_zero();
    double rc = -1.;                       // < 0: no bound yet
    int j = it, total = 0, count = 0;
    while (j < nit && count < 64) {
        const int step = FS[j];
        if (step == 0) break;
        const int idx = 2 * j + (step >> FSG_STG_COMPRESSED) - 1;
        if (idx >= R.bla_len) break;
        const double num = R.rbla[idx] - xabs_d(Q) * kc;
        if (!(num > 0.)) break;
        const double pm = hypot(P.re, P.im);
        const double lim = (pm == 0.) ? INFINITY : ldexp_d(num / pm, -P.e);
        if (!(lim > 0.)) break;
        if (rc >= 0. && lim < 0.25 * rc) break;
        rc = (rc < 0.) ? lim : fmin(rc, lim);
        const double2 A = R.Mbla[2 * idx], B = R.Mbla[2 * idx + 1];
        P = xr_mul_s(A, P);
        Q = xr_add(xr_mul_s(A, Q), xr_from(B));
        total += step; count++;
        j += step >> FSG_STG_COMPRESSED;
    }
    int4 h = make_int4(0, FE_ZERO_E, 0, 0), p = make_int4(0, 0, 0, 0);
    if (count >= 2 && rc > 0. && rc < INFINITY) {
        const fe a = fe_norm(fe_from_xc(P)), b = fe_norm(fe_from_xc(Q));
        const fe rf = fe_norm(fe_from_d(cx(0.9 * rc, 0.)));
        if (rf.e != FE_ZERO_E && a.e != FE_ZERO_E) {
            h = make_int4(__float_as_int(rf.x), rf.e, a.e, b.e);
            p = make_int4(__float_as_int(a.x), __float_as_int(a.y), __float_as_int(b.x),
                          __float_as_int(b.y));
        } else {
            total = 0; count = 0;
        }
    } else {
        total = 0; count = 0;
    }
    CH[2 * it] = h; CH[2 * it + 1] = p;
    CS[it] = make_int2(total, count);
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
__global__ void k_bs_fr_bla(const double *M, const double *r, int n, int4 *out, int2 *rf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * n) return;
    int2 a = fr_pack(fr_from_d(M[2 * i])), b = fr_pack(fr_from_d(M[2 * i + 1]));
    out[i] = make_int4(a.x, a.y, b.x, b.y);
    if (i < n) rf[i] = fr_pack(fr_from_d(r[i]));
}

// Frame-step tables (fsg_bs.cuh, BSFrame): per orbit index w
//   fa[w] = {X, Y as floats, exponent of X, exponent of Y}: a component of
//           magnitude in [2^-60, 2^40) is its float value; one below 2^-100 is
//           a signed zero (its exponent stays exact); 0 has FR_ZERO_E
//   fz[w] = {flags, g, Tw, eZ}: flags bit 0, the frame step may run at w (one
//           component in [2^-60, 2^40), the other 0, below 2^-100 or in that
//           range); bit 1, the loop's tests can run at w (each component 0,
//           below 2^-100 or in [2^-60, 2^40)); bit 2, X = Y = 0 (the step
//           there is quadratic in the deltas); g the largest exponent of the
//           reference Hessian at w (0 when it is 0); Tw: while the deltas
//           are below 2^(Tw + 1), X + xn or Y + yn keeps the orbit's sign
//           and magnitude within a factor 2, so no rebase happens at w
//           (FR_ZERO_E where the tests must run: X = Y = 0, a component
//           outside the float range, w >= div_iter - 1); eZ the exponent of
//           max(|X|, |Y|)
//   fh[w] = {dXa, dXb, dYa, dYb} * 2^-g, entries below 2^-126 of the
//           largest read as 0
__device__ __forceinline__ int fr_frame_kind(fr v) {    // 0 zero, 1 tiny, 2 float, 3 other
    if (v.m == 0.f) return 0;
    if (v.e < -100) return 1;
    if (v.e >= -60 && v.e <= 39) return 2;
    return 3;
}
__device__ __forceinline__ float fr_frame_val(fr v, int kind) {
    if (kind == 2) return v.m * __int_as_float((v.e + 127) << 23);
    return v.m < 0.f ? -0.f : 0.f;
}
__device__ __forceinline__ float fr_rel(fr v, int g) {
    if (v.m == 0.f) return 0.f;
    const int k = v.e - g;
    return k < -126 ? 0.f : v.m * __int_as_float((k + 127) << 23);
}
__global__ void k_bs_frame_tab(const int4 *Zf, const int4 *hf, int n, int div_iter, float4 *fa,
                               int4 *fz, float4 *fh) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 z = Zf[i];
    fr x, y;
    x.m = __int_as_float(z.x); x.e = z.y; y.m = __int_as_float(z.z); y.e = z.w;
    const int kx = fr_frame_kind(x), ky = fr_frame_kind(y);
    int flags = (kx != 3 && ky != 3) ? 2 : 0;
    if ((flags & 2) && (kx == 2 || ky == 2)) flags |= 1;
    if (kx == 0 && ky == 0) flags |= 4;
    int g = 0;
    if (hf) {
        const int4 p = hf[2 * i], q = hf[2 * i + 1];
        fr h[4];
        h[0].m = __int_as_float(p.x); h[0].e = p.y; h[1].m = __int_as_float(p.z); h[1].e = p.w;
        h[2].m = __int_as_float(q.x); h[2].e = q.y; h[3].m = __int_as_float(q.z); h[3].e = q.w;
        bool any = false;
        g = -(1 << 30);
        for (int k = 0; k < 4; k++)
            if (h[k].m != 0.f) { any = true; g = max(g, h[k].e); }
        if (!any) g = 0;
        fh[i] = make_float4(fr_rel(h[0], g), fr_rel(h[1], g), fr_rel(h[2], g), fr_rel(h[3], g));
    }
    fa[i] = make_float4(fr_frame_val(x, kx), fr_frame_val(y, ky), __int_as_float(x.e),
                        __int_as_float(y.e));
    int Tw = FR_ZERO_E, eZ = FR_ZERO_E;
    if (kx != 0) { Tw = max(Tw, x.e - 2); eZ = max(eZ, x.e); }
    if (ky != 0) { Tw = max(Tw, y.e - 2); eZ = max(eZ, y.e); }
    if (!(flags & 2) || i >= div_iter - 1) Tw = FR_ZERO_E;
    fz[i] = make_int4(flags, g, Tw, eZ);
}

void fsg_build_bs_fr(const RefDev *Rd, int len, int4 *Zf, const double *dXa, const double *dXb,
                     const double *dYa, const double *dYb, int4 *hf, float4 *fa, int4 *fz,
                     float4 *fh, int div_iter, cudaStream_t s) {
    int tb = 256;
    k_bs_fr_orbit<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(Rd, Zf);
    if (hf) k_bs_fr_paths<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(dXa, dXb, dYa, dYb, len + 1, hf);
    k_bs_frame_tab<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(Zf, hf, len + 1, div_iter, fa, fz, fh);
}
void fsg_build_bs_fr_bla(const double *Mbs, const double *rbla, int bla_len, int4 *blaf,
                         int2 *rf, cudaStream_t s) {
    int tb = 256;
    if (blaf && rf && bla_len > 0)
        k_bs_fr_bla<<<(4 * bla_len + tb - 1) / tb, tb, 0, s>>>(Mbs, rbla, bla_len, blaf, rf);
}

// ---------------------------------------------------------------------------
// host-side launchers (called by the C-ABI layer)
// ---------------------------------------------------------------------------
#define FSG_PATH_SCAN_MIN 8192

static xc xc_host(double re, double im, int e) {
    xc v;
    v.re = re; v.im = im; v.e = e;
    return v;
}

static void build_path_scan(const RefDev *Rd, int len, int first, int end, int xr_mode, int affine,
                            double scale_m, int scale_e, xc d0, double2 *out_std, double2 *out_xm,
                            int *out_xe, cudaStream_t s) {
    PathScan P;
    P.first = first; P.end = end;
    P.nchunks = end > first ? (end - first + FSG_PATH_CHUNK - 1) / FSG_PATH_CHUNK : 0;
    if (P.nchunks == 0) return;
    xc *buf = nullptr;
    if (cudaMallocAsync((void **)&buf, 3 * sizeof(xc) * (size_t)P.nchunks, s) != cudaSuccess) return;
    P.A = buf; P.B = buf + P.nchunks; P.start = buf + 2 * P.nchunks;
    const int tb = 128, nb = (P.nchunks + tb - 1) / tb;
    const xc sc = xc_host(scale_m, 0., scale_e);
    k_path_compose<<<nb, tb, 0, s>>>(Rd, P, xr_mode, affine, sc);
    k_path_prefix<<<1, 1, 0, s>>>(P, d0);
    k_path_fill<<<nb, tb, 0, s>>>(Rd, P, xr_mode, affine, scale_m, scale_e, out_std, out_xm, out_xe);
    cudaFreeAsync(buf, s);
}

// Derivative paths (numba_dZndc_path, numba_dZndz_path): zero-filled, then
// the recurrence -- sequential in the reference's order up to
// FSG_PATH_SCAN_MIN points, chunked scan above
void fsg_build_paths_m2(const RefDev *Rd, int len, double2 *dzndc, double2 *dzndc_xm, int *dzndc_xe,
                        double2 *dzndz, double2 *dzndz_xm, int *dzndz_xe, int div_iter, int xr_mode,
                        int want_dzndc, int want_dzndz, double scale_m, int scale_e,
                        cudaStream_t s) {
    const int valid = len < div_iter ? len : div_iter;
    const bool scan = len > FSG_PATH_SCAN_MIN;
    if (want_dzndc) {
        if (xr_mode) {
            cudaMemsetAsync(dzndc_xm, 0, 16 * (size_t)(len + 1), s);
            cudaMemsetAsync(dzndc_xe, 0, 4 * (size_t)(len + 1), s);
        } else {
            cudaMemsetAsync(dzndc, 0, 16 * (size_t)(len + 1), s);
        }
        if (!scan) {
            k_dzndc_m2<<<1, 1, 0, s>>>(Rd, dzndc, dzndc_xm, dzndc_xe, xr_mode, scale_m, scale_e);
        } else {
            build_path_scan(Rd, len, 1, valid, xr_mode, 1, scale_m, scale_e, xc_host(0., 0., 0), dzndc,
                            dzndc_xm, dzndc_xe, s);
            k_dzndc_tail<<<1, 1, 0, s>>>(Rd, dzndc, dzndc_xm, dzndc_xe, xr_mode, scale_m, scale_e);
        }
    }
    if (want_dzndz) {
        if (xr_mode) {
            cudaMemsetAsync(dzndz_xm, 0, 16 * (size_t)(len + 2), s);
            cudaMemsetAsync(dzndz_xe, 0, 4 * (size_t)(len + 2), s);
        } else {
            cudaMemsetAsync(dzndz, 0, 16 * (size_t)(len + 2), s);
        }
        if (!scan) {
            k_dzndz_m2<<<1, 1, 0, s>>>(Rd, dzndz, dzndz_xm, dzndz_xe, xr_mode);
        } else {
            build_path_scan(Rd, len, 2, valid, xr_mode, 0, 0., 0, xc_host(1., 0., 0), dzndz,
                            dzndz_xm, dzndz_xe, s);
            k_dzndz_tail<<<1, 1, 0, s>>>(Rd, dzndz, dzndz_xm, dzndz_xe, xr_mode);
        }
    }
}
void fsg_build_paths_bs_xr(const RefDev *Rd, int len, double *pm, int *pe, double scale_m,
                           int scale_e, cudaStream_t s) {
    cudaMemsetAsync(pm, 0, 4 * 8 * (size_t)(len + 1), s);
    cudaMemsetAsync(pe, 0, 4 * 4 * (size_t)(len + 1), s);
    k_dzndc_bs_xr<<<1, 1, 0, s>>>(Rd, pm, pe, scale_m, scale_e);
}

void fsg_build_paths_bs(const RefDev *Rd, int len, double *dXa, double *dXb, double *dYa, double *dYb,
                        double scale, cudaStream_t s) {
    for (double *p : {dXa, dXb, dYa, dYb}) cudaMemsetAsync(p, 0, 8 * (size_t)(len + 1), s);
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

void fsg_build_fe_runs(const RefDev *Rd, int len, const int4 *Zp, const int4 *Df, int4 *runs,
                       cudaStream_t s) {
    const int tb = 128;
    k_fe_runs<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(Rd, Zp, Df, len, runs);
}
void fsg_build_plain_orbit(const RefDev *Rd, int len, const int4 *Zf, int4 *Zp, cudaStream_t s) {
    int tb = 256;
    k_plain_orbit<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(Rd, Zf, Zp);
}

void fsg_build_fe_bla(const RefDev *Rd, const double2 *Mbla, const double *rbla, int bla_len,
                      int4 *bla_f, int bla_nit, int4 *bla_first, int *bla_first_step,
                      double kc, int4 *bla_chain, int2 *bla_chain_step, cudaStream_t s);

void fsg_build_fe_tables(const RefDev *Rd, int len, int4 *Zf, const double2 *dzndc,
                         const double2 *dzndc_xm, const int *dzndc_xe, int4 *dzndc_f,
                         const double2 *dzndz, const double2 *dzndz_xm, const int *dzndz_xe,
                         int4 *dzndz_f, const double2 *Mbla, const double *rbla, int bla_len,
                         int4 *bla_f, int bla_nit, int4 *bla_first, int *bla_first_step,
                         double kc, int4 *bla_chain, int2 *bla_chain_step, cudaStream_t s) {
    int tb = 256;
    k_fe_orbit<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(Rd, Zf);
    if (dzndc_f) k_fe_path<<<(len + 1 + tb - 1) / tb, tb, 0, s>>>(dzndc, dzndc_xm, dzndc_xe, len + 1, dzndc_f);
    if (dzndz_f) k_fe_path<<<(len + 2 + tb - 1) / tb, tb, 0, s>>>(dzndz, dzndz_xm, dzndz_xe, len + 2, dzndz_f);
    fsg_build_fe_bla(Rd, Mbla, rbla, bla_len, bla_f, bla_nit, bla_first, bla_first_step, kc,
                     bla_chain, bla_chain_step, s);
}

void fsg_build_fe_bla(const RefDev *Rd, const double2 *Mbla, const double *rbla, int bla_len,
                      int4 *bla_f, int bla_nit, int4 *bla_first, int *bla_first_step,
                      double kc, int4 *bla_chain, int2 *bla_chain_step, cudaStream_t s) {
    int tb = 256;
    if (bla_f && bla_len > 0) {
        k_fe_bla<<<(bla_len + tb - 1) / tb, tb, 0, s>>>(Mbla, rbla, bla_len, bla_f);
        k_fe_bla_first<<<(bla_nit + tb - 1) / tb, tb, 0, s>>>(Rd, bla_f, bla_nit, bla_first,
                                                              bla_first_step);
        if (bla_chain)
            k_fe_bla_chain<<<(bla_nit + tb - 1) / tb, tb, 0, s>>>(Rd, bla_first_step, bla_nit, kc,
                                                                  bla_chain, bla_chain_step);
    }
}
