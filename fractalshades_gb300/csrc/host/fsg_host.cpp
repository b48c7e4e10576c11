// fsg_host.cpp -- arbitrary-precision host side (include/fsghost.h).
//
// Restates the reference's Cython module mpmath_utils/FP_loop.pyx on the
// same libraries (MPFR 4.2 / MPC 1.3), call for call and at the same
// precisions, so that orbits, periods and nuclei are those of the
// reference.  Paths are relative to src/fractalshades/ of the reference.
// No global state: concurrent calls on different threads are independent
// (MPFR keeps its caches per thread).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "fsg_mp.h"
#include "../../../include/fsghost.h"

// The registers of one orbit computation (FP_loop.pyx:335-336, 1898-1899)
struct fsh_registers {
    std::vector<int64_t> idx[2];
    std::vector<double> m[2];
    std::vector<int64_t> e[2];
};

namespace {

const int RN = 0;                      // MPFR_RNDN / MPC_RNDNN
const double PARTIAL_TSHOLD = 1e-5;    // FP_loop.pyx:142
const double XR_TSHOLD = 1e-300;       // FP_loop.pyx:143
const long MAX_PREC = 1L << 28;

struct Fr {
    fsg_mpfr_struct v[1];
    explicit Fr(long prec) { mpfr_init2(v, prec); }
    ~Fr() { mpfr_clear(v); }
    Fr(const Fr &) = delete;
    Fr &operator=(const Fr &) = delete;
    operator fsg_mpfr_ptr() { return v; }
};

struct Cx {
    fsg_mpc_struct v[1];
    explicit Cx(long prec) { mpc_init2(v, prec); }
    ~Cx() { mpc_clear(v); }
    Cx(const Cx &) = delete;
    Cx &operator=(const Cx &) = delete;
    operator fsg_mpc_ptr() { return v; }
    fsg_mpfr_ptr re() { return v->re; }
    fsg_mpfr_ptr im() { return v->im; }
};

bool bad_prec(int64_t prec) { return prec < 2 || prec > MAX_PREC; }

// mpc_t_to_Xrange / mpfr_t_to_Xrange (FP_loop.pyx:424-456)
void push(fsh_registers *r, int which, int64_t i, fsg_mpfr_srcptr x, fsg_mpfr_srcptr y) {
    long ex = 0, ey = 0;
    double mx = mpfr_get_d_2exp(&ex, x, RN);
    double my = mpfr_get_d_2exp(&ey, y, RN);
    r->idx[which].push_back(i);
    r->m[which].push_back(mx);
    r->m[which].push_back(my);
    r->e[which].push_back(ex);
    r->e[which].push_back(ey);
}

// exact value as base-16 digits (gmpy_to_mpmath_mpc, FP_loop.pyx:2759-2790)
int write_hex(fsg_mpfr_srcptr v, char *out, int64_t out_len, int64_t *exp) {
    fsg_mpfr_exp_t e = 0;
    char *s = mpfr_get_str(nullptr, &e, 16, 0, v, RN);
    if (!s) return FSH_ERR_NOMEM;
    size_t n = strlen(s);
    int rc = FSH_OK;
    if ((int64_t)n + 1 > out_len) rc = FSH_ERR_ARG;
    else {
        memcpy(out, s, n + 1);
        *exp = e;
    }
    mpfr_free_str(s);
    return rc;
}

// ---------------------------------------------------------------------------
// z -> z^n + c and its derivatives (FP_loop.pyx:158-235)
// ---------------------------------------------------------------------------
// iter_M2 / iter_Mn: z <- z^n + c
void iter_mn(unsigned long n, fsg_mpc_ptr z, fsg_mpc_ptr c, fsg_mpc_ptr tmp) {
    if (n == 2) mpc_sqr(tmp, z, RN);
    else mpc_pow_ui(tmp, z, n, RN);
    mpc_add(z, tmp, c, RN);
}

// iter_deriv_M2 / iter_deriv_Mn: d <- n d z^(n-1) (+ 1 when var_c_z == 0)
void iter_deriv_mn(unsigned long n, int var_c_z, fsg_mpc_ptr z, fsg_mpc_ptr d,
                   fsg_mpc_ptr tmp) {
    if (n == 2) {
        mpc_mul(tmp, z, d, RN);
        mpc_mul_si(d, tmp, 2, RN);
    } else {
        mpc_pow_ui(tmp, z, n - 1, RN);
        mpc_mul(tmp, d, tmp, RN);
        mpc_mul_ui(d, tmp, n, RN);
    }
    if (var_c_z == 0) mpc_add_ui(d, d, 1, RN);
}

// ---------------------------------------------------------------------------
// Burning Ship family (FP_loop.pyx:1343-1827)
// ---------------------------------------------------------------------------
struct BSWork {
    Fr xsq, ysq, xy, abs_x, abs_y, t_xx, t_xy, t_yx, t_yy, t;
    explicit BSWork(long p)
        : xsq(p), ysq(p), xy(p), abs_x(p), abs_y(p), t_xx(p), t_xy(p), t_yx(p), t_yy(p), t(p) {}
};

// sign (FP_loop.pyx:1778-1784): +1 for op >= 0
int sgn1(fsg_mpfr_srcptr op) { return mpfr_sgn(op) >= 0 ? 1 : -1; }

// iter_BS, iter_pBS, iter_sharkfin, iter_celtic, iter_buffalo (:1358-1455)
void iter_bs(int kind, fsg_mpfr_ptr x, fsg_mpfr_ptr y, fsg_mpfr_ptr a, fsg_mpfr_ptr b,
             BSWork &w) {
    switch (kind) {
    case 1:    // X <- X^2 - Y^2 + A, Y <- 2 |X Y| - B
        mpfr_sqr(w.xsq, x, RN); mpfr_sqr(w.ysq, y, RN); mpfr_mul(w.xy, x, y, RN);
        mpfr_sub(x, w.xsq, w.ysq, RN); mpfr_add(x, x, a, RN);
        mpfr_abs(w.xy, w.xy, RN); mpfr_mul_si(w.xy, w.xy, 2, RN);
        mpfr_sub(y, w.xy, b, RN);
        break;
    case 2:    // X <- X^2 - Y^2 + A, Y <- 2 X |Y| - B
        mpfr_sqr(w.xsq, x, RN); mpfr_sqr(w.ysq, y, RN);
        mpfr_abs(w.xy, y, RN); mpfr_mul(w.xy, x, w.xy, RN); mpfr_mul_si(w.xy, w.xy, 2, RN);
        mpfr_sub(x, w.xsq, w.ysq, RN); mpfr_add(x, x, a, RN);
        mpfr_sub(y, w.xy, b, RN);
        break;
    case 3:    // X <- X^2 - Y |Y| + A, Y <- 2 X Y - B
        mpfr_sqr(w.xsq, x, RN); mpfr_abs(w.ysq, y, RN); mpfr_mul(w.ysq, w.ysq, y, RN);
        mpfr_mul(w.xy, x, y, RN); mpfr_mul_si(w.xy, w.xy, 2, RN);
        mpfr_sub(x, w.xsq, w.ysq, RN); mpfr_add(x, x, a, RN);
        mpfr_sub(y, w.xy, b, RN);
        break;
    case 4:    // X <- |X^2 - Y^2| + A, Y <- 2 X Y - B
        mpfr_sqr(w.xsq, x, RN); mpfr_sqr(w.ysq, y, RN);
        mpfr_mul(w.xy, x, y, RN); mpfr_mul_si(w.xy, w.xy, 2, RN);
        mpfr_sub(x, w.xsq, w.ysq, RN); mpfr_abs(x, x, RN); mpfr_add(x, x, a, RN);
        mpfr_sub(y, w.xy, b, RN);
        break;
    default:   // 5, X <- |X^2 - Y^2| + A, Y <- 2 |X Y| - B
        mpfr_sqr(w.xsq, x, RN); mpfr_sqr(w.ysq, y, RN); mpfr_mul(w.xy, x, y, RN);
        mpfr_sub(x, w.xsq, w.ysq, RN); mpfr_abs(x, x, RN); mpfr_add(x, x, a, RN);
        mpfr_abs(w.xy, w.xy, RN); mpfr_mul_si(w.xy, w.xy, 2, RN);
        mpfr_sub(y, w.xy, b, RN);
        break;
    }
}

// iter_J_* (:1458-1742): J <- Df(x, y) J (+ diag(1, -1) when var_ab_xy == 0),
// with J = [[dxdx, dxdy], [dydx, dydy]]
void iter_jac_bs(int kind, int var_ab_xy, fsg_mpfr_ptr x, fsg_mpfr_ptr y, fsg_mpfr_ptr dxdx,
                 fsg_mpfr_ptr dxdy, fsg_mpfr_ptr dydx, fsg_mpfr_ptr dydy, BSWork &w) {
    int sx, sy, sq;
    switch (kind) {
    case 1:
        mpfr_abs(w.abs_x, x, RN); mpfr_abs(w.abs_y, y, RN);
        sx = sgn1(x); sy = sgn1(y);
        mpfr_mul(w.t_xx, x, dxdx, RN); mpfr_mul(w.t, y, dydx, RN); mpfr_sub(w.t_xx, w.t_xx, w.t, RN);
        mpfr_mul(w.t_xy, x, dxdy, RN); mpfr_mul(w.t, y, dydy, RN); mpfr_sub(w.t_xy, w.t_xy, w.t, RN);
        mpfr_mul(w.t_yx, w.abs_x, dydx, RN); mpfr_mul_si(w.t_yx, w.t_yx, sy, RN);
        mpfr_mul(w.t, w.abs_y, dxdx, RN); mpfr_mul_si(w.t, w.t, sx, RN);
        mpfr_add(w.t_yx, w.t_yx, w.t, RN);
        mpfr_mul(w.t_yy, w.abs_x, dydy, RN); mpfr_mul_si(w.t_yy, w.t_yy, sy, RN);
        mpfr_mul(w.t, w.abs_y, dxdy, RN); mpfr_mul_si(w.t, w.t, sx, RN);
        mpfr_add(w.t_yy, w.t_yy, w.t, RN);
        break;
    case 2:
        mpfr_abs(w.abs_y, y, RN);
        sy = sgn1(y);
        mpfr_mul(w.t_xx, x, dxdx, RN); mpfr_mul(w.t, y, dydx, RN); mpfr_sub(w.t_xx, w.t_xx, w.t, RN);
        mpfr_mul(w.t_xy, x, dxdy, RN); mpfr_mul(w.t, y, dydy, RN); mpfr_sub(w.t_xy, w.t_xy, w.t, RN);
        mpfr_mul(w.t_yx, x, dydx, RN); mpfr_mul_si(w.t_yx, w.t_yx, sy, RN);
        mpfr_mul(w.t, w.abs_y, dxdx, RN); mpfr_add(w.t_yx, w.t_yx, w.t, RN);
        mpfr_mul(w.t_yy, x, dydy, RN); mpfr_mul_si(w.t_yy, w.t_yy, sy, RN);
        mpfr_mul(w.t, w.abs_y, dxdy, RN); mpfr_add(w.t_yy, w.t_yy, w.t, RN);
        break;
    case 3:
        mpfr_abs(w.abs_y, y, RN);
        mpfr_mul(w.t_xx, x, dxdx, RN); mpfr_mul(w.t, w.abs_y, dydx, RN); mpfr_sub(w.t_xx, w.t_xx, w.t, RN);
        mpfr_mul(w.t_xy, x, dxdy, RN); mpfr_mul(w.t, w.abs_y, dydy, RN); mpfr_sub(w.t_xy, w.t_xy, w.t, RN);
        mpfr_mul(w.t_yx, x, dydx, RN); mpfr_mul(w.t, y, dxdx, RN); mpfr_add(w.t_yx, w.t_yx, w.t, RN);
        mpfr_mul(w.t_yy, x, dydy, RN); mpfr_mul(w.t, y, dxdy, RN); mpfr_add(w.t_yy, w.t_yy, w.t, RN);
        break;
    case 4:
        mpfr_sqr(w.t, x, RN); mpfr_sqr(w.t_xy, y, RN); mpfr_sub(w.t_xy, w.t, w.t_xy, RN);
        sq = sgn1(w.t_xy);
        mpfr_mul(w.t_xx, x, dxdx, RN); mpfr_mul(w.t, y, dydx, RN); mpfr_sub(w.t_xx, w.t_xx, w.t, RN);
        mpfr_mul_si(w.t_xx, w.t_xx, sq, RN);
        mpfr_mul(w.t_xy, x, dxdy, RN); mpfr_mul(w.t, y, dydy, RN); mpfr_sub(w.t_xy, w.t_xy, w.t, RN);
        mpfr_mul_si(w.t_xy, w.t_xy, sq, RN);
        mpfr_mul(w.t_yx, x, dydx, RN); mpfr_mul(w.t, y, dxdx, RN); mpfr_add(w.t_yx, w.t_yx, w.t, RN);
        mpfr_mul(w.t_yy, x, dydy, RN); mpfr_mul(w.t, y, dxdy, RN); mpfr_add(w.t_yy, w.t_yy, w.t, RN);
        break;
    default:
        mpfr_sqr(w.t, x, RN); mpfr_sqr(w.t_xy, y, RN); mpfr_sub(w.t_xy, w.t, w.t_xy, RN);
        sx = sgn1(x); sy = sgn1(y); sq = sgn1(w.t_xy);
        mpfr_abs(w.abs_x, x, RN); mpfr_abs(w.abs_y, y, RN);
        mpfr_mul(w.t_xx, x, dxdx, RN); mpfr_mul(w.t, y, dydx, RN); mpfr_sub(w.t_xx, w.t_xx, w.t, RN);
        mpfr_mul_si(w.t_xx, w.t_xx, sq, RN);
        mpfr_mul(w.t_xy, x, dxdy, RN); mpfr_mul(w.t, y, dydy, RN); mpfr_sub(w.t_xy, w.t_xy, w.t, RN);
        mpfr_mul_si(w.t_xy, w.t_xy, sq, RN);
        mpfr_mul(w.t_yx, w.abs_x, dydx, RN); mpfr_mul_si(w.t_yx, w.t_yx, sy, RN);
        mpfr_mul(w.t, w.abs_y, dxdx, RN); mpfr_mul_si(w.t, w.t, sx, RN);
        mpfr_add(w.t_yx, w.t_yx, w.t, RN);
        mpfr_mul(w.t_yy, w.abs_x, dydy, RN); mpfr_mul_si(w.t_yy, w.t_yy, sy, RN);
        mpfr_mul(w.t, w.abs_y, dxdy, RN); mpfr_mul_si(w.t, w.t, sx, RN);
        mpfr_add(w.t_yy, w.t_yy, w.t, RN);
        break;
    }
    mpfr_mul_si(dxdx, w.t_xx, 2, RN);
    mpfr_mul_si(dxdy, w.t_xy, 2, RN);
    mpfr_mul_si(dydx, w.t_yx, 2, RN);
    mpfr_mul_si(dydy, w.t_yy, 2, RN);
    if (var_ab_xy == 0) {
        mpfr_add_si(dxdx, dxdx, 1, RN);
        mpfr_add_si(dydy, dydy, -1, RN);
    }
}

// det (:1786-1792) and matsolve (:1795-1825): [[a, b], [c, d]] (x, y) = (e, f)
void det(fsg_mpfr_ptr delta, fsg_mpfr_ptr a, fsg_mpfr_ptr b, fsg_mpfr_ptr c, fsg_mpfr_ptr d,
         fsg_mpfr_ptr t) {
    mpfr_mul(delta, a, d, RN);
    mpfr_mul(t, c, b, RN);
    mpfr_sub(delta, delta, t, RN);
}

void matsolve(fsg_mpfr_ptr xr, fsg_mpfr_ptr yr, fsg_mpfr_ptr a, fsg_mpfr_ptr b, fsg_mpfr_ptr c,
              fsg_mpfr_ptr d, fsg_mpfr_ptr e, fsg_mpfr_ptr f, fsg_mpfr_ptr delta, fsg_mpfr_ptr t) {
    det(delta, a, b, c, d, t);
    mpfr_ui_div(delta, 1, delta, RN);
    mpfr_mul(xr, d, e, RN);
    mpfr_mul(t, b, f, RN);
    mpfr_sub(xr, xr, t, RN);
    mpfr_mul(xr, xr, delta, RN);
    mpfr_mul(yr, a, f, RN);
    mpfr_mul(t, c, e, RN);
    mpfr_sub(yr, yr, t, RN);
    mpfr_mul(yr, yr, delta, RN);
}

// the partials register test (:360-376, 1927-1951): is |z|^2 below the
// current minimum (or below PARTIAL_TSHOLD^2 for the first entry)?  The
// squared moduli are held at 2 prec + 8 bits.
struct Partials {
    Fr best, cand;
    bool have = false;
    double curr = PARTIAL_TSHOLD;
    explicit Partials(long prec) : best(2 * prec + 8), cand(2 * prec + 8) {}
    bool smaller() {
        if (!have) {
            mpfr_set_d(best, curr, RN);
            mpfr_sqr(best, best, RN);
        }
        return mpfr_cmp(cand, best) < 0;
    }
    void take(double x, double y) {
        mpfr_set(best, cand, RN);
        have = true;
        curr = std::hypot(x, y);
    }
};

}  // namespace

// ---------------------------------------------------------------------------
// registers
// ---------------------------------------------------------------------------
extern "C" int64_t fsh_registers_count(const fsh_registers *r, int32_t which) {
    if (!r || which < 0 || which > 1) return FSH_ERR_ARG;
    return (int64_t)r->idx[which].size();
}

extern "C" int fsh_registers_copy(const fsh_registers *r, int32_t which, int64_t *idx,
                                  double *mantissas, int64_t *exponents) {
    if (!r || which < 0 || which > 1) return FSH_ERR_ARG;
    size_t n = r->idx[which].size();
    if (n == 0) return FSH_OK;
    if (!idx || !mantissas || !exponents) return FSH_ERR_ARG;
    memcpy(idx, r->idx[which].data(), n * sizeof(int64_t));
    memcpy(mantissas, r->m[which].data(), 2 * n * sizeof(double));
    memcpy(exponents, r->e[which].data(), 2 * n * sizeof(int64_t));
    return FSH_OK;
}

extern "C" void fsh_registers_free(fsh_registers *r) { delete r; }

// ---------------------------------------------------------------------------
// orbits
// ---------------------------------------------------------------------------
// perturbation_mandelbrotN_select_FP_loop (FP_loop.pyx:274-421)
extern "C" int64_t fsh_orbit_mn(const char *seed_x, const char *seed_y, int64_t prec,
                                int64_t max_iter, uint32_t exponent, double M, int32_t need_xr,
                                double *orbit, fsh_registers **regs) {
    if (!seed_x || !seed_y || !orbit || !regs || bad_prec(prec) || max_iter < 0 || exponent < 2)
        return FSH_ERR_ARG;
    *regs = nullptr;
    fsh_registers *R = new (std::nothrow) fsh_registers();
    if (!R) return FSH_ERR_NOMEM;
    Cx z(prec), c(prec), tmp(prec);
    Fr x(prec), y(prec);
    if (mpfr_set_str(x, seed_x, 10, RN) != 0 || mpfr_set_str(y, seed_y, 10, RN) != 0) {
        delete R;
        return FSH_ERR_ARG;
    }
    mpc_set_fr_fr(c, x, y, RN);
    mpc_set_si_si(z, 0, 0, RN);
    orbit[0] = 0.;
    orbit[1] = 0.;
    Partials P(prec);
    int64_t i;
    double abs_i = 0.;
    for (i = 1; i <= max_iter; i++) {
        iter_mn(exponent, z, c, tmp);
        double xd = mpfr_get_d(z.re(), RN), yd = mpfr_get_d(z.im(), RN);
        orbit[2 * i] = xd;
        orbit[2 * i + 1] = yd;
        abs_i = std::hypot(xd, yd);
        if (abs_i > M) break;
        if (need_xr && abs_i < XR_TSHOLD) push(R, 0, i, z.re(), z.im());
        if (abs_i <= P.curr) {
            mpc_norm(P.cand, z, RN);
            if (P.smaller()) {
                push(R, 1, i, z.re(), z.im());
                P.take(xd, yd);
            }
        }
    }
    // without an escape the loop ends at max_iter + 1: the reference's
    // "first invalid iteration is i + 1" (:404-408)
    *regs = R;
    return i;
}

// perturbation_nonholomorphic_FP_loop (FP_loop.pyx:1828-1979)
extern "C" int64_t fsh_orbit_bs(const char *seed_x, const char *seed_y, int64_t prec,
                                int64_t max_iter, int32_t kind, double M, int32_t need_xr,
                                double *orbit, fsh_registers **regs) {
    if (!seed_x || !seed_y || !orbit || !regs || bad_prec(prec) || max_iter < 0 || kind < 1 ||
        kind > 5)
        return FSH_ERR_ARG;
    *regs = nullptr;
    fsh_registers *R = new (std::nothrow) fsh_registers();
    if (!R) return FSH_ERR_NOMEM;
    Fr x(prec), y(prec), a(prec), b(prec);
    BSWork w(prec);
    if (mpfr_set_str(a, seed_x, 10, RN) != 0 || mpfr_set_str(b, seed_y, 10, RN) != 0) {
        delete R;
        return FSH_ERR_ARG;
    }
    mpfr_set_si(x, 0, RN);
    mpfr_set_si(y, 0, RN);
    orbit[0] = 0.;
    orbit[1] = 0.;
    Partials P(prec);
    Fr x2(2 * prec + 8), y2(2 * prec + 8);
    int64_t i;
    double abs_i = 0.;
    for (i = 1; i <= max_iter; i++) {
        iter_bs(kind, x, y, a, b, w);
        double xd = mpfr_get_d(x, RN), yd = mpfr_get_d(y, RN);
        orbit[2 * i] = xd;
        orbit[2 * i + 1] = yd;
        abs_i = std::hypot(xd, yd);
        if (abs_i > M) break;
        if (need_xr && (std::fabs(xd) < XR_TSHOLD || std::fabs(yd) < XR_TSHOLD))
            push(R, 0, i, x, y);
        if (abs_i <= P.curr) {
            mpfr_sqr(x2, x, RN);
            mpfr_sqr(y2, y, RN);
            mpfr_add(P.cand, x2, y2, RN);
            if (P.smaller()) {
                push(R, 1, i, x, y);
                P.take(xd, yd);
            }
        }
    }
    *regs = R;
    return i;
}

// ---------------------------------------------------------------------------
// ball method
// ---------------------------------------------------------------------------
// perturbation_mandelbrotN_select_ball_method (FP_loop.pyx:631-760)
extern "C" int64_t fsh_ball_mn(const char *seed_x, const char *seed_y, int64_t prec,
                               const char *seed_px, uint32_t exponent, int64_t maxiter,
                               double M_divergence) {
    if (!seed_x || !seed_y || !seed_px || bad_prec(prec) || exponent < 2) return FSH_ERR_ARG;
    Cx c(prec), z(prec), dz(prec), tmp(prec), r(prec);
    Fr ar(54), x(prec), y(prec), pix(prec), inv_pix(prec);
    if (mpfr_set_str(x, seed_x, 10, RN) != 0 || mpfr_set_str(y, seed_y, 10, RN) != 0 ||
        mpfr_set_str(pix, seed_px, 10, RN) != 0)
        return FSH_ERR_ARG;
    mpc_set_fr_fr(c, x, y, RN);
    mpfr_ui_div(inv_pix, 1, pix, RN);
    mpc_set_si_si(z, 0, 0, RN);
    mpc_set_si_si(dz, 0, 0, RN);
    mpc_set_si_si(tmp, 0, 0, RN);
    mpc_set_si_si(r, 0, 0, RN);
    for (int64_t i = 1; i <= maxiter; i++) {
        iter_deriv_mn(exponent, 0, z, dz, tmp);
        iter_mn(exponent, z, c, tmp);
        mpc_div(r, z, dz, RN);
        mpc_mul_fr(r, r, inv_pix, RN);
        double xd = mpfr_get_d(z.re(), RN), yd = mpfr_get_d(z.im(), RN);
        if (std::hypot(xd, yd) > M_divergence) return 0;
        mpc_abs(ar, r, RN);
        if (mpfr_cmp_d(ar, 1.) < 0) return i;
    }
    return 0;
}

// perturbation_nonholomorphic_ball_method (FP_loop.pyx:2357-2563)
extern "C" int64_t fsh_ball_bs(const char *seed_x, const char *seed_y, int64_t prec,
                               const char *seed_px, int32_t kind, int64_t maxiter,
                               double M_divergence) {
    if (!seed_x || !seed_y || !seed_px || bad_prec(prec) || kind < 1 || kind > 5)
        return FSH_ERR_ARG;
    Fr x(prec), y(prec), a(prec), b(prec), dxa(prec), dxb(prec), dya(prec), dyb(prec),
        delta(prec), rx(prec), ry(prec), pix(prec), inv_pix(prec), t(prec), low(54);
    BSWork w(prec);
    if (mpfr_set_str(a, seed_x, 10, RN) != 0 || mpfr_set_str(b, seed_y, 10, RN) != 0 ||
        mpfr_set_str(pix, seed_px, 10, RN) != 0)
        return FSH_ERR_ARG;
    mpfr_set_si(x, 0, RN); mpfr_set_si(y, 0, RN);
    mpfr_set_si(dxa, 0, RN); mpfr_set_si(dxb, 0, RN);
    mpfr_set_si(dya, 0, RN); mpfr_set_si(dyb, 0, RN);
    mpfr_ui_div(inv_pix, 1, pix, RN);
    for (int64_t i = 1; i <= maxiter; i++) {
        iter_jac_bs(kind, 0, x, y, dxa, dxb, dya, dyb, w);
        iter_bs(kind, x, y, a, b, w);
        matsolve(rx, ry, dxa, dxb, dya, dyb, x, y, delta, t);
        mpfr_mul(rx, rx, inv_pix, RN);
        mpfr_mul(ry, ry, inv_pix, RN);
        double xd = mpfr_get_d(x, RN), yd = mpfr_get_d(y, RN);
        if (std::hypot(xd, yd) > M_divergence) return 0;
        mpfr_abs(low, rx, RN);
        int cx = mpfr_cmp_d(low, 1.);
        mpfr_abs(low, ry, RN);
        int cy = mpfr_cmp_d(low, 1.);
        if (cx < 0 && cy < 0) {
            double rxd = mpfr_get_d(rx, RN), ryd = mpfr_get_d(ry, RN);
            if (std::hypot(rxd, ryd) < 1.) return i;
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Newton
// ---------------------------------------------------------------------------
// perturbation_mandelbrot_find_nucleus (FP_loop.pyx:900-1116): Newton on
// f^order(0) / prod_{i | order, i < order} f^i(0)
extern "C" int fsh_nucleus_m2(const char *seed_x, const char *seed_y, int64_t prec,
                              int64_t order, int64_t max_newton, const char *seed_eps_cv,
                              const char *seed_eps_valid, char *out_x, char *out_y,
                              int64_t out_len, int64_t *exp_x, int64_t *exp_y) {
    if (!seed_x || !seed_y || !seed_eps_cv || !seed_eps_valid || !out_x || !out_y || !exp_x ||
        !exp_y || bad_prec(prec) || order < 1 || max_newton < 0)
        return FSH_ERR_ARG;
    Cx c(prec), zr(prec), dzrdc(prec), h(prec), dh(prec), f(prec), df(prec), t1(prec), t2(prec);
    Fr x(prec), y(prec), abs_diff(54), eps(54);
    if (mpfr_set_str(x, seed_x, 10, RN) != 0 || mpfr_set_str(y, seed_y, 10, RN) != 0 ||
        mpfr_set_str(eps, seed_eps_cv, 10, RN) != 0)
        return FSH_ERR_ARG;
    mpc_set_fr_fr(c, x, y, RN);
    mpfr_mul_si(eps, eps, 64, RN);
    bool newton_cv = false;
    for (int64_t k = 0; k < max_newton; k++) {
        mpc_set_si_si(zr, 0, 0, RN);
        mpc_set_si_si(dzrdc, 0, 0, RN);
        mpc_set_si_si(h, 1, 0, RN);
        mpc_set_si_si(dh, 0, 0, RN);
        for (int64_t i = 1; i <= order; i++) {
            mpc_mul_si(t1, dzrdc, 2, RN);
            mpc_mul(t2, t1, zr, RN);
            mpc_add_ui(dzrdc, t2, 1, RN);
            mpc_sqr(t1, zr, RN);
            mpc_add(zr, t1, c, RN);
            if (i < order && order % i == 0) {
                mpc_mul(t1, h, zr, RN);
                mpc_swap(t1, h);
                mpc_div(t1, dzrdc, zr, RN);
                mpc_add(t2, t1, dh, RN);
                mpc_swap(t2, dh);
            }
        }
        mpc_div(f, zr, h, RN);
        mpc_mul(t1, zr, dh, RN);
        mpc_sub(t2, dzrdc, t1, RN);
        mpc_div(df, t2, h, RN);
        mpc_div(t1, f, df, RN);
        mpc_sub(t2, c, t1, RN);
        mpc_swap(t2, c);
        mpc_abs(abs_diff, t1, RN);
        if (mpfr_greaterequal_p(eps, abs_diff)) {
            mpc_abs(abs_diff, zr, RN);
            if (mpfr_set_str(eps, seed_eps_valid, 10, RN) != 0) return FSH_ERR_ARG;
            newton_cv = mpfr_greaterequal_p(eps, abs_diff) != 0;
            break;
        }
    }
    int rc = write_hex(c.re(), out_x, out_len, exp_x);
    if (rc == FSH_OK) rc = write_hex(c.im(), out_y, out_len, exp_y);
    return rc == FSH_OK ? (newton_cv ? 1 : 0) : rc;
}

// perturbation_mandelbrotN_select_find_any_nucleus (FP_loop.pyx:1159-1340)
extern "C" int fsh_any_nucleus_mn(const char *seed_x, const char *seed_y, int64_t prec,
                                  uint32_t exponent, int64_t order, int64_t max_newton,
                                  const char *seed_eps_cv, const char *seed_eps_valid,
                                  char *out_x, char *out_y, int64_t out_len, int64_t *exp_x,
                                  int64_t *exp_y) {
    if (!seed_x || !seed_y || !seed_eps_cv || !seed_eps_valid || !out_x || !out_y || !exp_x ||
        !exp_y || bad_prec(prec) || exponent < 2 || order < 1 || max_newton < 0)
        return FSH_ERR_ARG;
    Cx c(prec), zr(prec), dzrdc(prec), t1(prec);
    Fr x(prec), y(prec), abs_diff(54), eps(54);
    if (mpfr_set_str(x, seed_x, 10, RN) != 0 || mpfr_set_str(y, seed_y, 10, RN) != 0 ||
        mpfr_set_str(eps, seed_eps_cv, 10, RN) != 0)
        return FSH_ERR_ARG;
    mpc_set_fr_fr(c, x, y, RN);
    mpfr_mul_si(eps, eps, 64, RN);
    bool newton_cv = false;
    for (int64_t k = 0; k < max_newton; k++) {
        mpc_set_si_si(zr, 0, 0, RN);
        mpc_set_si_si(dzrdc, 0, 0, RN);
        for (int64_t i = 1; i <= order; i++) {
            iter_deriv_mn(exponent, 0, zr, dzrdc, t1);
            iter_mn(exponent, zr, c, t1);
        }
        mpc_div(t1, zr, dzrdc, RN);
        mpc_sub(c, c, t1, RN);
        mpc_abs(abs_diff, t1, RN);
        if (mpfr_greaterequal_p(eps, abs_diff)) {
            mpc_abs(abs_diff, zr, RN);
            if (mpfr_set_str(eps, seed_eps_valid, 10, RN) != 0) return FSH_ERR_ARG;
            newton_cv = mpfr_greaterequal_p(eps, abs_diff) != 0;
            break;
        }
    }
    int rc = write_hex(c.re(), out_x, out_len, exp_x);
    if (rc == FSH_OK) rc = write_hex(c.im(), out_y, out_len, exp_y);
    return rc == FSH_OK ? (newton_cv ? 1 : 0) : rc;
}

// perturbation_nonholomorphic_find_any_nucleus (FP_loop.pyx:2564-2756)
extern "C" int fsh_any_nucleus_bs(const char *seed_x, const char *seed_y, int64_t prec,
                                  int32_t kind, int64_t order, int64_t max_newton,
                                  const char *seed_eps_cv, const char *seed_eps_valid,
                                  char *out_x, char *out_y, int64_t out_len, int64_t *exp_x,
                                  int64_t *exp_y) {
    if (!seed_x || !seed_y || !seed_eps_cv || !seed_eps_valid || !out_x || !out_y || !exp_x ||
        !exp_y || bad_prec(prec) || kind < 1 || kind > 5 || order < 1 || max_newton < 0)
        return FSH_ERR_ARG;
    Fr x(prec), y(prec), a(prec), b(prec), da(prec), db(prec), dxa(prec), dxb(prec), dya(prec),
        dyb(prec), delta(prec), t(prec), eps(54), abs_diff(54);
    BSWork w(prec);
    if (mpfr_set_str(a, seed_x, 10, RN) != 0 || mpfr_set_str(b, seed_y, 10, RN) != 0 ||
        mpfr_set_str(eps, seed_eps_cv, 10, RN) != 0)
        return FSH_ERR_ARG;
    mpfr_mul_si(eps, eps, 64, RN);
    bool newton_cv = false;
    for (int64_t k = 0; k < max_newton; k++) {
        mpfr_set_si(x, 0, RN); mpfr_set_si(y, 0, RN);
        mpfr_set_si(dxa, 0, RN); mpfr_set_si(dxb, 0, RN);
        mpfr_set_si(dya, 0, RN); mpfr_set_si(dyb, 0, RN);
        for (int64_t i = 1; i <= order; i++) {
            iter_jac_bs(kind, 0, x, y, dxa, dxb, dya, dyb, w);
            iter_bs(kind, x, y, a, b, w);
        }
        matsolve(da, db, dxa, dxb, dya, dyb, x, y, delta, t);
        mpfr_sub(a, a, da, RN);
        mpfr_sub(b, b, db, RN);
        mpfr_hypot(abs_diff, da, db, RN);
        if (mpfr_greaterequal_p(eps, abs_diff)) {
            mpfr_hypot(abs_diff, x, y, RN);
            if (mpfr_set_str(eps, seed_eps_valid, 10, RN) != 0) return FSH_ERR_ARG;
            newton_cv = mpfr_greaterequal_p(eps, abs_diff) != 0;
            break;
        }
    }
    int rc = write_hex(a, out_x, out_len, exp_x);
    if (rc == FSH_OK) rc = write_hex(b, out_y, out_len, exp_y);
    return rc == FSH_OK ? (newton_cv ? 1 : 0) : rc;
}

// ---------------------------------------------------------------------------
// size estimates
// ---------------------------------------------------------------------------
// perturbation_mandelbrotN_select_nucleus_size_estimate (FP_loop.pyx:487-604)
extern "C" int fsh_size_mn(const char *seed_x, const char *seed_y, int64_t prec,
                           uint32_t exponent, int64_t order, double *out, int64_t *eout) {
    if (!seed_x || !seed_y || !out || !eout || bad_prec(prec) || exponent < 2 || order < 1)
        return FSH_ERR_ARG;
    Cx z(prec), c(prec), l(prec), b(prec), t(prec), t2(prec);
    Fr x(prec), y(prec);
    if (mpfr_set_str(x, seed_x, 10, RN) != 0 || mpfr_set_str(y, seed_y, 10, RN) != 0)
        return FSH_ERR_ARG;
    mpc_set_fr_fr(c, x, y, RN);
    mpc_set_si_si(z, 0, 0, RN);
    mpc_set_si_si(l, 1, 0, RN);
    mpc_set_si_si(b, 1, 0, RN);
    for (int64_t i = 1; i < order; i++) {
        iter_mn(exponent, z, c, t);
        iter_deriv_mn(exponent, 1, z, l, t);
        mpc_ui_div(t, 1, l, RN);
        mpc_add(t2, b, t, RN);
        mpc_swap(t2, b);
    }
    if (exponent == 2) mpc_sqr(t, l, RN);
    else mpc_pow_d(t, l, exponent / (exponent - 1.), RN);
    mpc_mul(t2, b, t, RN);
    mpc_ui_div(t, 1, t2, RN);
    long ex = 0, ey = 0;
    out[0] = mpfr_get_d_2exp(&ex, t.re(), RN);
    out[1] = mpfr_get_d_2exp(&ey, t.im(), RN);
    eout[0] = ex;
    eout[1] = ey;
    return FSH_OK;
}

// perturbation_nonholomorphic_nucleus_size_estimate (FP_loop.pyx:1982-2100)
extern "C" int fsh_size_bs(const char *seed_x, const char *seed_y, int64_t prec, int32_t kind,
                           int64_t order, double *out, int64_t *eout, double *skew) {
    if (!seed_x || !seed_y || !out || !eout || !skew || bad_prec(prec) || kind < 1 || kind > 5 ||
        order < 1)
        return FSH_ERR_ARG;
    Fr x(prec), y(prec), a(prec), b(prec), dxx(prec), dxy(prec), dyx(prec), dyy(prec),
        delta(prec), bxx(prec), bxy(prec), byx(prec), byy(prec), t(prec), dbeta(prec);
    BSWork w(prec);
    if (mpfr_set_str(a, seed_x, 10, RN) != 0 || mpfr_set_str(b, seed_y, 10, RN) != 0)
        return FSH_ERR_ARG;
    mpfr_set_si(x, 0, RN); mpfr_set_si(y, 0, RN);
    mpfr_set_si(dxx, 1, RN); mpfr_set_si(dxy, 0, RN);
    mpfr_set_si(dyx, 0, RN); mpfr_set_si(dyy, 1, RN);
    mpfr_set_si(bxx, 1, RN); mpfr_set_si(bxy, 0, RN);
    mpfr_set_si(byx, 0, RN); mpfr_set_si(byy, 1, RN);
    for (int64_t i = 1; i < order; i++) {
        iter_bs(kind, x, y, a, b, w);
        iter_jac_bs(kind, 1, x, y, dxx, dxy, dyx, dyy, w);
        det(delta, dxx, dxy, dyx, dyy, t);
        mpfr_ui_div(delta, 1, delta, RN);
        mpfr_mul(t, delta, dyy, RN); mpfr_add(bxx, bxx, t, RN);
        mpfr_mul(t, delta, dxy, RN); mpfr_sub(bxy, bxy, t, RN);
        mpfr_mul(t, delta, dyx, RN); mpfr_sub(byx, byx, t, RN);
        mpfr_mul(t, delta, dxx, RN); mpfr_add(byy, byy, t, RN);
    }
    det(delta, dxx, dxy, dyx, dyy, t);
    mpfr_sqr(delta, delta, RN);
    det(dbeta, bxx, bxy, byx, byy, t);
    mpfr_mul(delta, dbeta, delta, RN);
    mpfr_abs(t, delta, RN);
    mpfr_rec_sqrt(delta, t, RN);
    long e = 0;
    out[0] = mpfr_get_d_2exp(&e, delta, RN);
    eout[0] = e;
    mpfr_rec_sqrt(t, dbeta, RN);
    mpfr_mul(bxx, bxx, t, RN); mpfr_mul(bxy, bxy, t, RN);
    mpfr_mul(byx, byx, t, RN); mpfr_mul(byy, byy, t, RN);
    skew[0] = mpfr_get_d(byy, RN);
    skew[1] = mpfr_get_d(bxy, RN);
    skew[2] = mpfr_get_d(byx, RN);
    skew[3] = mpfr_get_d(bxx, RN);
    return FSH_OK;
}
