// fsg_perturb_fe32.cu -- power-2 Mandelbrot perturbation loop with deltas held
// as FP32 mantissa + int32 exponent.
//
// Control flow of the reference's numba_iterate (perturbation.py:1065-1400):
// BLA attempt every 8 iterations, full step, max_iter / interior / escape
// tests, rebase on reference divergence and Zhuoran's dynamic rebase.
//
// Representation: dz = u * 2^E, dz/dc = v * 2^F, dz/dz = q * 2^G with float2
// mantissas renormalised lazily (when max(|x|, |y|) leaves [2^-30, 2^30]) and
// dc = cm * 2^Ec (cm normalised).  cu = cm * 2^(Ec - E) is kept with E.
//
// Two step kinds:
//   * FP32 step, whenever Z_w and dz are normal floats (2^-100 .. 2^100, the
//     plain value of dz above 2^-126 unless |dz| < 2^-26 |Z|): in dz's frame
//     u' = u (2 Z + dz) + cu and v' = 2 (Z + dz) v + 2^k D u (k = De + E - F);
//     while |dz| < 2^-26 |Z| (one exponent compare) the dz terms are below
//     FP32 resolution and the step is u' = 2 Z u + cu.  Consecutive FP32 steps
//     run until the next event (BLA attempt, max_iter, divergence rebase, wrap)
//     or a test FP32 cannot decide;
//   * exact step otherwise (Z tiny or zero, dz out of float range): every
//     operation in fe arithmetic (fsg_num.cuh).
// Tests: escape and the componentwise rebase test in FP32 with a margin for
// the rounding of Z and dz; within the margin, the reference's exact form --
// the componentwise test on the double values (with to_standard()'s
// underflow), then, following the Xrange branch, the extended
// |Z + dz|^2 <= |dz|^2 confirmation.
// The BLA validity test |dz| < r is |u|^2 < r^2 2^(-2E) in FP32 with the
// exponent gap clamped (to_standard(dz), which the reference compares, is 0
// only below every r > 0), against the FP64 radius rounded down with a
// margin that covers the test's rounding: never a step beyond the radius.
// Runs of consecutive BLA steps (each on the largest admissible stage) are
// applied as one composite step where the composite's radius admits dz
// (fsg_ref.cu, k_fe_bla_chain), and so are runs of FP32 steps between BLA
// attempt points in the |dz| < 2^-26 |Z| regime, where a tabulated bound
// shows that every step of the run stays there (fsg_ref.cu, k_fe_runs): the
// same iterations, the same decisions, one step.
#include "fsg_internal.cuh"

// 2^k as a float for k in [-126, 127]; 0 below; k > 127 is clamped (callers
// keep k small)
__device__ __forceinline__ float p2f(int k) {
    k = min(max(k, -127), 127);
    return __int_as_float((k + 127) << 23);
}
// unbiased exponent of a positive normal float; -127 for 0 / subnormals
__device__ __forceinline__ int fexp(float m) { return ((__float_as_int(m) >> 23) & 0xff) - 127; }

__device__ __forceinline__ fe ld_fe(const int4 *p, int i) {
    int4 v = __ldg(&p[i]);
    return fe_make(__int_as_float(v.x), __int_as_float(v.y), v.z);
}

struct Lane {
    float ux, uy; int E;          // dz
    float vx, vy; int F;          // dz/dc
    float qx, qy; int G;          // dz/dz
    float cux, cuy;               // dc * 2^-E
};

__device__ __forceinline__ void set_cu(Lane &s, float cmx, float cmy, int Ec) {
    float sc = p2f(Ec - s.E);
    s.cux = cmx * sc; s.cuy = cmy * sc;
}

// lazy renormalisation of dz (keeps E >= Ec - 100 so that cu stays finite)
__device__ __forceinline__ void renorm_u(Lane &s, float cmx, float cmy, int Ec) {
    float m = fmaxf(fabsf(s.ux), fabsf(s.uy));
    if (m >= 0x1p-30f && m <= 0x1p30f) return;
    int En;
    if (m < 0x1p-126f) { s.ux = 0.f; s.uy = 0.f; En = Ec; }
    else {
        En = max(s.E + fexp(m), Ec - 100);
        float sc = p2f(s.E - En);
        s.ux *= sc; s.uy *= sc;
    }
    s.E = En;
    set_cu(s, cmx, cmy, Ec);
}

__device__ __forceinline__ void renorm_v(float &x, float &y, int &e) {
    float m = fmaxf(fabsf(x), fabsf(y));
    if (m >= 0x1p-30f && m <= 0x1p30f) return;
    if (m < 0x1p-126f) { x = 0.f; y = 0.f; e = FE_ZERO_E; return; }
    int k = fexp(m);
    float sc = p2f(-k);
    x *= sc; y *= sc; e += k;
}

// magnitude exponent of dz (FE_ZERO_E for 0)
__device__ __forceinline__ int mag_u(const Lane &s) {
    float m = fmaxf(fabsf(s.ux), fabsf(s.uy));
    return (m == 0.f) ? FE_ZERO_E : s.E + fexp(m);
}

__device__ __forceinline__ fe as_fe(float x, float y, int e) {
    return (x == 0.f && y == 0.f) ? fe_zero() : fe_norm(fe_make(x, y, e));
}
// dz from an fe value (cu is set when a fast run starts)
__device__ __forceinline__ void from_fe_u(Lane &s, fe d, float cmx, float cmy, int Ec) {
    if (d.e == FE_ZERO_E || (d.x == 0.f && d.y == 0.f)) { s.ux = 0.f; s.uy = 0.f; s.E = Ec; }
    else {
        s.E = max(d.e, Ec - 100);
        float sc = p2f(d.e - s.E);
        s.ux = d.x * sc; s.uy = d.y * sc;
    }
}
__device__ __forceinline__ void store_fe(float &x, float &y, int &e, fe d) {
    if (d.e == FE_ZERO_E || (d.x == 0.f && d.y == 0.f)) { x = 0.f; y = 0.f; e = FE_ZERO_E; }
    else { x = d.x; y = d.y; e = d.e; }
}

// biased exponent of max(|ux|, |uy|) (0 for 0 and subnormals)
__device__ __forceinline__ int mag_b(const Lane &s) {
    return __float_as_int(fmaxf(fabsf(s.ux), fabsf(s.uy))) >> 23;
}

// Fast update of a derivative delta d = x 2^e against the reference
// derivative Dv = {x, y, e} (e = FE_ZERO_E for 0, and for dzndc right after
// a dynamic rebase), 2 Z = (Zx, Zy):
//   d' = 2 (Z d + D dz)  as  x' = 2Z x + 2^(kd+1) D u,  kd = De + E - e
// (the dz d term is below FP32 resolution when |dz| < 2^-26 |Z|).  d = 0 is
// held with e = FE_ZERO_E, which sends kd above 100 and rescales d onto the
// new term.
__device__ __forceinline__ void deriv_fast(float &x, float &y, int &e, int4 Dv, float Zx, float Zy,
                                           const Lane &s) {
    const float dx = __int_as_float(Dv.x), dy = __int_as_float(Dv.y);
    int kd = Dv.z + s.E - e;
    if (kd > 100) {
        int en = Dv.z + s.E - 30;
        float sc = p2f(e - en);
        x *= sc; y *= sc; e = en; kd = 30;
    }
    // 2^(kd + 1), 0 below 2^-126 (kd <= 100 here)
    const float sk = __int_as_float((max(kd + 1, -127) + 127) << 23);
    const float dxs = dx * sk, dys = dy * sk;
    const float nx = fmaf(Zx, x, fmaf(-Zy, y, fmaf(dxs, s.ux, -dys * s.uy)));
    const float ny = fmaf(Zx, y, fmaf(Zy, x, fmaf(dxs, s.uy, dys * s.ux)));
    x = nx; y = ny;
    renorm_v(x, y, e);
}

// (x^2 + y^2) 2^(2e) < tm 2^te: the float sum of squares against the
// threshold eps^2 = tm 2^te, held as tm in [1, 2] (rounded up from the double:
// no float lies strictly between the two) and an int exponent; decided
// exactly on exponents and mantissas, as fe_abs2_lt's double compare is
__device__ __forceinline__ bool abs2_below(float x, float y, int e, float tm, int te) {
    float m2 = fmaf(x, x, y * y);
    if (m2 == 0.f) return true;
    int em = fexp(m2);
    if (em == -127) { m2 *= 0x1p64f; em = fexp(m2) - 64; }       // subnormal sum
    const float mm = __int_as_float((__float_as_int(m2) & 0x007fffff) | 0x3f800000);
    const int L = em + 2 * e;
    return L < te || (L == te && mm < tm);
}

// |q 2^G + Q|^2 < eps^2: both terms aligned on the larger exponent e
__device__ __forceinline__ bool stationary_fast(float qx, float qy, int G, int4 Q, float tm,
                                                int te) {
    const int e = max(G, Q.z);
    const float a = __int_as_float((max(G - e, -127) + 127) << 23);
    const float b = __int_as_float((max(Q.z - e, -127) + 127) << 23);
    const float x = fmaf(qx, a, __int_as_float(Q.x) * b), y = fmaf(qy, a, __int_as_float(Q.y) * b);
    return abs2_below(x, y, e, tm, te);
}

// The operands of a rare double test pass through an empty volatile asm
// inside the test's branch: the compiler cannot evaluate the double
// arithmetic that depends on them ahead of the branch.
__device__ __forceinline__ void opaque(float &a, float &b, int &c, int &d) {
    asm volatile("" : "+f"(a), "+f"(b), "+r"(c), "+r"(d));
}

// |dz| < r for a BLA header H = {r mantissa bits, r exponent, A exponent,
// B exponent}, as |u|^2 < rm^2 2^(2 (re - E)) in FP32.  u is normalised
// (|u| in [2^-30, 2^31) or 0), so exponent gaps beyond +-126 are decided by
// the clamp alone; r = 0 (rm = 0) admits nothing, dz = 0 any r > 0 -- the
// reference's strict 0 < r.  The table's rm is the FP64 radius rounded down
// with a 2^-20 margin (fsg_ref.cu, k_fe_bla): the test passes only where
// |dz| < r holds exactly, so no step goes beyond the FP64 radius; within
// 2^-19 of it (about 1 lookup in 10^5) the step is declined and the
// iterations run as full steps.  (An exact decision at those near-ties, in
// float-float or in double, cost 7 % of the headline: rare code in the
// lookup lengthened the loop.)
__device__ __forceinline__ bool bla_ok(const Lane &s, int4 H) {
    const int d = min(max(2 * (H.y - s.E), -126), 126);
    const float rm = __int_as_float(H.x);
    return fmaf(s.ux, s.ux, s.uy * s.uy) < (rm * rm) * __int_as_float((d + 127) << 23);
}

// ref_BLA_get (perturbation.py:2116-2170): the largest stage from
// 3 + ctz(w >> 3) (capped at stages - 1) down to 3 whose step is below
// first_invalid - w and whose radius admits dz.  The first candidate of each
// start index (header, payload and step) is tabulated when the reference is
// built.  Radii of one start index never grow with the stage (a parent's r is
// min(r of its first child, ...), :2023-2024), so when stage 3 refuses, every
// stage does: after the first candidate the search tests stage 3, then the
// stages between.
__device__ __forceinline__ int bla_find(const int4 *__restrict__ T, const int4 *__restrict__ FF,
                                        const int *__restrict__ FS, const Lane &s, int w,
                                        int4 &H, int4 &P) {
    const int it = w >> FSG_STG_COMPRESSED;
    const int st = __ldg(&FS[it]);
    H = __ldg(&FF[2 * it]);
    P = __ldg(&FF[2 * it + 1]);
    if (st == 0) return 0;
    const int i0 = 2 * it;
    // BLA_index(i, stg) = 2 i + 2^stg - 1 over the stored stages (stg - 3)
    if (bla_ok(s, H)) return st;
    if (st == 8) return 0;
    const int4 H3 = __ldg(&T[2 * i0]);
    if (!bla_ok(s, H3)) return 0;
    for (int stg = 30 - __clz(st); stg > FSG_STG_COMPRESSED; stg--) {
        const int idx = i0 + (1 << (stg - FSG_STG_COMPRESSED)) - 1;
        H = __ldg(&T[2 * idx]);
        if (bla_ok(s, H)) { P = __ldg(&T[2 * idx + 1]); return 1 << stg; }
    }
    H = H3; P = __ldg(&T[2 * i0 + 1]);
    return 1 << FSG_STG_COMPRESSED;
}

// The componentwise dynamic-rebase test on the double values (the
// reference's std values, to_standard() underflow included), taken only when
// the FP32 test is within its rounding of a tie, or for values outside the
// float range.
static __device__ __forceinline__ int rebase_test_double(fe dz, const double2 *Zn, int w) {
    const double2 dd = fe_to_d(dz);
    const double2 Zd = __ldg(&Zn[w]);
    const double2 ZZd = cadd(dd, Zd);
    return (fabs(ZZd.x) <= fabs(dd.x)) && (fabs(ZZd.y) <= fabs(dd.y));
}

// rebase bookkeeping shared by the three rebase kinds: dzndc += dZndc_w,
// dzndz += dZndz_w (wrapped slot at n = order) unless nullified
__device__ __forceinline__ void rebase_derivs(Lane &s, const RefDev &R, int w, int n, int order,
                                              bool dzndc_on, bool dzndz_on, bool &nullify) {
    if (dzndc_on)
        store_fe(s.vx, s.vy, s.F, fe_norm(fe_add(as_fe(s.vx, s.vy, s.F), ld_fe(R.dZndc_f, w))));
    if (dzndz_on) {
        if (!nullify)
            store_fe(s.qx, s.qy, s.G,
                     fe_norm(fe_add(as_fe(s.qx, s.qy, s.G),
                                    ld_fe(R.dZndz_f, (n == order) ? R.len : w))));
        nullify = true;
    }
}

// One pixel; returns its iteration count and adds its executed full steps,
// BLA steps and rebases to the (per-pixel, 32-bit) counters.
template <bool INTERIOR>
__device__ __forceinline__ int pixel_fe32(const TileDev &T, const CalcDev &C, long long ip,
                                          unsigned &nfull, unsigned &nbla, unsigned &nreb) {
    const RefDev &R = *T.ref;
    const long long np = (long long)T.nx * T.ny;
    const bool dzndz_on = INTERIOR, dzndc_on = C.calc_dzndc;
    // the fast interior test needs eps^2 as a normal float
    // eps^2 = tm 2^te for the integer-exponent interior test (any finite
    // eps^2 > 0; else the double test)
    const bool eps_fast = C.eps2 > 0. && C.eps2 < INFINITY;
    int te = 0;
    const float tm = eps_fast ? __double2float_ru(2. * frexp(C.eps2, &te)) : 0.f;
    te -= 1;
    const int xrsem = C.xrsem, max_iter = C.max_iter;
    const int order = R.order, div_iter = R.div_iter, first_invalid = R.first_invalid;
    const bool bla_on = C.bla && R.bla_first != nullptr;
    // escape test on the table's 2 Z: |2 Z|^2 > 4 M^2
    const float M2f = (float)C.M2, M2f4 = 4.f * M2f;
    const int4 *__restrict__ Zp = R.Zp;
    const int4 *__restrict__ dZndc_f = R.dZndc_f;
    const int4 *__restrict__ dZndz_f = R.dZndz_f;
    const int4 *__restrict__ bla_f = R.bla_f;
    const int4 *__restrict__ bla_first = R.bla_first;
    const int *__restrict__ bla_first_step = R.bla_first_step;
    const int4 *__restrict__ fe_runs = R.fe_runs;
    const int4 *__restrict__ bla_chain = R.bla_chain;
    const int2 *__restrict__ bla_chain_step = R.bla_chain_step;
    // c from the pixel (perturbation.py:2214-2230) in Xrange, then fe
    double2 pp = fsg_pixel(T, ip);
    double x1 = T.lin[0] * pp.x + T.lin[1] * pp.y;
    double y1 = T.lin[2] * pp.x + T.lin[3] * pp.y;
    xf dxr; dxr.m = T.dx_m; dxr.e = T.dx_e;
    xc c_xr = xr_add(xf_mul_c(dxr, cx(x1, y1)), xc_make(T.drift_re, T.drift_im, T.drift_e));
    const fe dcf = fe_from_xc(c_xr);
    const bool dc_zero = (dcf.e == FE_ZERO_E);
    const float cmx = dc_zero ? 0.f : dcf.x, cmy = dc_zero ? 0.f : dcf.y;
    const int Ec = dc_zero ? 0 : dcf.e;

    Lane s;
    s.ux = 0.f; s.uy = 0.f; s.E = Ec;
    s.vx = 0.f; s.vy = 0.f; s.F = FE_ZERO_E;
    s.qx = 0.f; s.qy = 0.f; s.G = FE_ZERO_E;
    s.cux = cmx; s.cuy = cmy;
    int w = 0, n = 0; signed char stop = -1;
    bool nullify = false, dyn = true;
    int4 Zc = __ldg(&Zp[0]);

    for (;;) {
        // ---------------- BLA step (perturbation.py:1121-1154) -------------
        // (w < first_invalid here: w = 0, or the tests that let the loop
        // continue saw w < div_iter - 1, or a BLA jump stopped short of it)
        if (bla_on && (w & 7) == 0 && w < first_invalid) {
            int4 H, P;
            int step = bla_find(bla_f, bla_first, bla_first_step, s, w, H, P);
            // when the first candidate is taken, the run of first candidates
            // from here, composed (its radius is at most 0.9 of the first
            // candidate's: the margin covers the FP32 test's rounding)
            if (step != 0 && step == __ldg(&bla_first_step[w >> FSG_STG_COMPRESSED])) {
                const int2 cs = __ldg(&bla_chain_step[w >> FSG_STG_COMPRESSED]);
                if (cs.y >= 2) {
                    const int4 Hc = __ldg(&bla_chain[2 * (w >> FSG_STG_COMPRESSED)]);
                    if (bla_ok(s, Hc)) {
                        H = Hc;
                        P = __ldg(&bla_chain[2 * (w >> FSG_STG_COMPRESSED) + 1]);
                        step = cs.x;
                    }
                }
            }
            if (step != 0) {
                const float Ax = __int_as_float(P.x), Ay = __int_as_float(P.y);
                const float Bx = __int_as_float(P.z), By = __int_as_float(P.w);
                // dz' = A dz + B dc on the exponent En = max(E + Ae, Ec + Be - 60,
                // Ec - 100): A dz scaled by 2^(E + Ae - En) <= 1, B dc by
                // 2^(Ec + Be - En) <= 2^60 (terms below 2^-127 of the scale vanish)
                const int Ea = s.E + H.z, Eb = Ec + H.w;
                const int En = max(max(Ea, Eb - 60), Ec - 100);
                const float sa = __int_as_float((max(Ea - En, -127) + 127) << 23);
                const float sb = __int_as_float((max(Eb - En, -127) + 127) << 23);
                const float bx = (Bx * cmx - By * cmy) * sb, by = (Bx * cmy + By * cmx) * sb;
                const float nx = fmaf(Ax * s.ux - Ay * s.uy, sa, bx);
                const float ny = fmaf(Ax * s.uy + Ay * s.ux, sa, by);
                s.ux = nx; s.uy = ny; s.E = En;
                if ((unsigned)(mag_b(s) - 97) > 60u) renorm_u(s, cmx, cmy, Ec);
                if (dzndc_on) {
                    float vx = Ax * s.vx - Ay * s.vy, vy = Ax * s.vy + Ay * s.vx;
                    s.vx = vx; s.vy = vy; s.F += H.z;
                    renorm_v(s.vx, s.vy, s.F);
                }
                if (dzndz_on) {
                    float qx = Ax * s.qx - Ay * s.qy, qy = Ax * s.qy + Ay * s.qx;
                    s.qx = qx; s.qy = qy; s.G += H.z;
                    renorm_v(s.qx, s.qy, s.G);
                }
                n += step;
                w += step;               // step < first_invalid - w <= order - w: no wrap
                Zc = __ldg(&Zp[w]);
                nbla++;
                continue;
            }
        }
        // ---------------- full step (perturbation.py:1158-1214) ------------
        // A run of FP32 steps when Z_w is a normal float (2^-100 .. 2^100) and
        // |dz| < 2^100: dz' = dz (dz + 2 Z) + dc in dz's frame,
        // u' = u (2 Z + dz) + cu, and the derivatives with 2 (Z + dz) -- for
        // |dz| < 2^-26 |Z| the dz terms vanish below FP32 resolution.
        // (u = 0 counts as 2^(E - 127).)  Below E = -126 the plain value of
        // dz flushes to 0, which is exact only in the |dz| < 2^-26 |Z| regime.
        const int md0 = s.E + mag_b(s) - 127;     // exponent of |dz|inf
        const int4 *Rr = fe_runs + 5 * (size_t)w;
        int4 T4 = make_int4(0, 0, 0, 0), T3 = T4;
        // (the table is read only where its bound can hold: |dz| below the
        // fast-step limit at w already)
        if (!INTERIOR && fe_runs != nullptr && !dyn && (w & 7) != 0 && Zc.z != FE_ZERO_E
            && Zc.z > md0) {
            T4 = __ldg(&Rr[4]);
            T3 = __ldg(&Rr[3]);
        }
        // A composed run (fsg_ref.cu, k_fe_runs): the fast steps from w to the
        // next multiple of 8 in one, where the table's bound shows that every
        // one of them is in the |dz| < 2^-26 |Z| regime (|U0| a + |c| b < 1/2,
        // each term bounded by 2 max(|x|, |y|) 2^e < 2^-2), so that no rebase
        // test could fire, and the orbit's |2 Z|^2 stays below 4 M^2 (the run's
        // escape tests); the run must also fit before the orbit's end, the
        // reference's divergence and max_iter, as a stepwise run would.  Only
        // runs that start between BLA attempt points are composed (the run
        // after the orbit's critical point); on escape-dominated views most
        // runs start at a declined attempt, and lanes of one warp split between
        // the two forms would run both.  The choice depends on the pixel alone.
        if (T4.y != 0 && w + T4.y <= order && w + T4.y <= div_iter - 1 && n + T4.y <= max_iter
            && __int_as_float(T4.x) <= M2f4 * (1.f - 0x1p-20f)
            && fexp(__int_as_float(T3.x) * fmaxf(fabsf(s.ux), fabsf(s.uy))) + T3.y + s.E <= -3
            && fexp(__int_as_float(T3.z) * fmaxf(fabsf(cmx), fabsf(cmy))) + T3.w + Ec <= -3) {
            const int kt = T4.y;
            const int4 T0 = __ldg(&Rr[0]), T1 = __ldg(&Rr[1]);
            const float Px = __int_as_float(T0.x), Py = __int_as_float(T0.y);
            const float Qx = __int_as_float(T1.x), Qy = __int_as_float(T1.y);
            if (dzndc_on) {
                // V = P V0 + R U0 + S c on the largest term's exponent (the
                // others scaled by at most 1; below 2^-127 of it they vanish)
                const int4 T2 = __ldg(&Rr[2]);
                const float Rx = __int_as_float(T1.z), Ry = __int_as_float(T1.w);
                const float Sx = __int_as_float(T2.z), Sy = __int_as_float(T2.w);
                const int e1 = (s.F == FE_ZERO_E) ? FE_ZERO_E : s.F + T0.z;
                const int e2 = (T2.x == FE_ZERO_E) ? FE_ZERO_E : s.E + T2.x;
                const int e3 = (T2.y == FE_ZERO_E || dc_zero) ? FE_ZERO_E : Ec + T2.y;
                const int Fn = max(max(e1, e2), e3);
                if (Fn > FE_ZERO_E / 2) {
                    const float s1 = p2f(max(e1 - Fn, -127)), s2 = p2f(max(e2 - Fn, -127));
                    const float s3 = p2f(max(e3 - Fn, -127));
                    const float ax = (Px * s.vx - Py * s.vy) * s1, ay = (Px * s.vy + Py * s.vx) * s1;
                    const float bx = (Rx * s.ux - Ry * s.uy) * s2, by = (Rx * s.uy + Ry * s.ux) * s2;
                    const float cx_ = (Sx * cmx - Sy * cmy) * s3, cy_ = (Sx * cmy + Sy * cmx) * s3;
                    s.vx = ax + bx + cx_;
                    s.vy = ay + by + cy_;
                    s.F = Fn;
                    renorm_v(s.vx, s.vy, s.F);
                }
            }
            // U = P U0 + Q c, as a BLA step applies A dz + B dc
            const int Ea = s.E + T0.z, Eb = Ec + T0.w;
            const int En = max(max(Ea, Eb - 60), Ec - 100);
            const float sa = __int_as_float((max(Ea - En, -127) + 127) << 23);
            const float sb = __int_as_float((max(Eb - En, -127) + 127) << 23);
            const float bx = (Qx * cmx - Qy * cmy) * sb, by = (Qx * cmy + Qy * cmx) * sb;
            const float nx = fmaf(Px * s.ux - Py * s.uy, sa, bx);
            const float ny = fmaf(Px * s.uy + Py * s.ux, sa, by);
            s.ux = nx; s.uy = ny; s.E = En;
            if ((unsigned)(mag_b(s) - 97) > 60u) renorm_u(s, cmx, cmy, Ec);
            n += kt;
            nbla++;
            w += kt;
            if (w >= order) w = 0;
            dyn = false;
        } else if (Zc.z != FE_ZERO_E && md0 <= 100 && (Zc.z >= md0 || s.E >= -126)) {
            // the run lasts up to the next event that needs the general
            // tests -- a BLA attempt (w % 8 == 0), max_iter, the reference's
            // divergence rebase, the orbit's wrap -- or until a step's tests
            // (escape, rebase) cannot be decided in FP32
            int k = order - w;
            if (bla_on) k = min(k, 8 - (w & 7));
            k = min(k, max(div_iter - 1 - w, 1));
            k = max(min(k, max_iter - n), 1);
            set_cu(s, cmx, cmy, Ec);
            float sE = p2f(s.E);
            int4 Dv = make_int4(0, 0, FE_ZERO_E, 0);
            if (dzndc_on && !dyn) Dv = __ldg(&dZndc_f[w]);
            // dzndz: the reference derivative is dZndz_0 once nullified, else
            // dZndz_w (n = order, the wrapped slot, is a wrap: an event)
            int4 Q0 = Dv, Qv = Dv;
            if (INTERIOR) {
                Q0 = __ldg(&dZndz_f[0]);
                Qv = nullify ? Q0 : __ldg(&dZndz_f[w]);
            }
            int j = 0;
            bool esc = false, stat = false;
            bool tiny = Zc.z >= md0;               // |dz| < 2^-26 |Z| at this step
            for (;;) {
                // next entries (w + 1 <= order <= len, inside the tables)
                const int4 Zn = __ldg(&Zp[w + 1]);
                int4 Dn = Dv, Qn = Qv;
                if (dzndc_on) Dn = __ldg(&dZndc_f[w + 1]);
                if (INTERIOR) Qn = nullify ? Q0 : __ldg(&dZndz_f[w + 1]);
                const float Zx = __int_as_float(Zc.x), Zy = __int_as_float(Zc.y);   // 2 Z
                if (tiny) {
                    // the dz terms are below FP32 resolution: u' = 2 Z u + cu
                    if (dzndc_on) deriv_fast(s.vx, s.vy, s.F, Dv, Zx, Zy, s);
                    if (INTERIOR) deriv_fast(s.qx, s.qy, s.G, Qv, Zx, Zy, s);
                    const float nx = fmaf(Zx, s.ux, fmaf(-Zy, s.uy, s.cux));
                    const float ny = fmaf(Zx, s.uy, fmaf(Zy, s.ux, s.cuy));
                    s.ux = nx; s.uy = ny;
                } else {
                    const float ex = s.ux * sE, ey = s.uy * sE;                      // dz
                    const float tx = Zx + ex, ty = Zy + ey;                          // 2 Z + dz
                    if (dzndc_on) deriv_fast(s.vx, s.vy, s.F, Dv, tx + ex, ty + ey, s);
                    if (INTERIOR) deriv_fast(s.qx, s.qy, s.G, Qv, tx + ex, ty + ey, s);
                    const float nx = fmaf(tx, s.ux, fmaf(-ty, s.uy, s.cux));
                    const float ny = fmaf(tx, s.uy, fmaf(ty, s.ux, s.cuy));
                    s.ux = nx; s.uy = ny;
                }
                j++; w++;
                if (j == k) break;
                Zc = Zn; Dv = Dn; Qv = Qn;
                if (INTERIOR) {
                    // (:1224-1246) against the next reference derivative
                    bool st = eps_fast ? stationary_fast(s.qx, s.qy, s.G, Qn, tm, te)
                                       : fe_abs2_lt(fe_add(as_fe(s.qx, s.qy, s.G),
                                                           fe_make(__int_as_float(Qn.x),
                                                                   __int_as_float(Qn.y), Qn.z)),
                                                    C.eps2);
                    if (st) { stat = true; break; }
                }
                int b = mag_b(s);
                if ((unsigned)(b - 97) > 60u) { renorm_u(s, cmx, cmy, Ec); b = mag_b(s); sE = p2f(s.E); }
                const int md = s.E + b - 127;
                const float Zx2 = __int_as_float(Zc.x), Zy2 = __int_as_float(Zc.y);
                tiny = Zc.z >= md;                 // false for FE_ZERO_E
                if (tiny) {
                    // |dz| < 2^-26 |Z|: ZZ = Z to FP32 resolution and
                    // |Z|inf >= 4 |dz|inf rules the rebase out
                    if (Zx2 * Zx2 + Zy2 * Zy2 > M2f4) { esc = true; break; }
                } else {
                    // Z out of the float range or 0, dz too large, or dz's
                    // plain value out of range: the next step in exact form
                    if (Zc.z == FE_ZERO_E || md > 100 || s.E < -126) break;
                    // escape (:1252-1279) and the componentwise rebase test
                    // (:1317-1320) in FP32: "no rebase" is certain when a
                    // component of |Z + dz| exceeds that of |dz| by more than
                    // 2^-20 of the magnitudes (Z carries 2^-24 of rounding);
                    // otherwise the general tests decide, in double at ties
                    const float fx = s.ux * sE, fy = s.uy * sE;
                    const float hx = fmaf(0.5f, Zx2, fx), hy = fmaf(0.5f, Zy2, fy);
                    if (hx * hx + hy * hy > M2f) { esc = true; break; }
                    const float tau = 0x1p-21f * (fabsf(Zx2) + fabsf(Zy2)) + 0x1p-20f * (fabsf(fx) + fabsf(fy));
                    if (!(fabsf(hx) - fabsf(fx) > tau || fabsf(hy) - fabsf(fy) > tau)) break;
                }
                dyn = false;
            }
            renorm_u(s, cmx, cmy, Ec);
            n += j; nfull += j;
            if (stat) { stop = 2; break; }
            if (esc) { stop = 1; break; }
            if (w >= order) w = 0;
        } else if ((Zc.w & 1) && !dzndz_on && dyn && 2 * md0 + 4 < Ec - 26) {
            // Z_w = 0 (the critical point, once per period of a cycle) with
            // |dz|^2 < 2^-27 |dc| and the reference derivative nullified
            // (dyn, after the rebase there): dz' = dz^2 + dc is dc to within
            // 2^-27 of its modulus (below the FP32 rounding of the value),
            // and dzndc' = 2 dz dzndc is one FP32 complex product on the
            // exponents' sum -- the fe step below, in FP32
            n += 1;
            nfull++;
            if (dzndc_on && s.F != FE_ZERO_E) {
                const float vx = s.ux * s.vx - s.uy * s.vy, vy = s.ux * s.vy + s.uy * s.vx;
                s.vx = vx; s.vy = vy; s.F = s.F + s.E + 1;
                renorm_v(s.vx, s.vy, s.F);
            }
            s.ux = cmx; s.uy = cmy; s.E = Ec;
            w += 1;
            if (w >= order) w = 0;
        } else {
            n += 1;
            nfull++;
            fe dz = as_fe(s.ux, s.uy, s.E);
            if ((Zc.w & 1) && !dzndz_on) {
                // Z_w = 0: dz' = dz^2 + dc, dzndc' = 2 dz (dzndc + D)
                if (dzndc_on) {
                    fe t = as_fe(s.vx, s.vy, s.F);
                    if (!dyn) t = fe_add(t, ld_fe(dZndc_f, w));
                    store_fe(s.vx, s.vy, s.F, fe_norm(fe_scale2(fe_mul(dz, t), 1)));
                }
                dz = fe_norm(fe_add(fe_mul(dz, dz), dcf));
            } else {
                // exact step in fe arithmetic
                fe Zw = ld_fe(R.Zf, w);
                if (dzndc_on) {
                    fe D = dyn ? fe_zero() : ld_fe(dZndc_f, w);
                    fe d = as_fe(s.vx, s.vy, s.F);
                    store_fe(s.vx, s.vy, s.F,
                             fe_norm(fe_scale2(fe_add(fe_mul(fe_add(Zw, dz), d), fe_mul(D, dz)), 1)));
                }
                if (dzndz_on) {
                    fe D = ld_fe(R.dZndz_f, nullify ? 0 : w);
                    fe q = as_fe(s.qx, s.qy, s.G);
                    store_fe(s.qx, s.qy, s.G,
                             fe_norm(fe_scale2(fe_add(fe_mul(fe_add(Zw, dz), q), fe_mul(D, dz)), 1)));
                }
                dz = fe_norm(fe_add(fe_mul(dz, fe_add(dz, fe_scale2(Zw, 1))), dcf));
            }
            from_fe_u(s, dz, cmx, cmy, Ec);
            w += 1;
            if (w >= order) w = 0;       // w < order before the increment
        }
        // ---------------- max_iter (:1218-1220) ----------------------------
        if (n >= max_iter) { stop = 0; break; }
        // ---------------- interior detection (:1224-1246) ------------------
        if (dzndz_on) {
            int k = nullify ? 0 : ((n == order) ? R.len : w);
            fe ZdZ = fe_add(as_fe(s.qx, s.qy, s.G), ld_fe(R.dZndz_f, k));
            if (eps_fast ? abs2_below(ZdZ.x, ZdZ.y, ZdZ.e, tm, te) : fe_abs2_lt(ZdZ, C.eps2)) {
                stop = 2;
                break;
            }
        }
        Zc = __ldg(&Zp[w]);
        if (w < div_iter - 1) {
            if (Zc.z >= s.E + mag_b(s) - 127) {
                // fast tests: |dz| < 2^-26 |Z_next|, no rebase possible
                const float Zx = __int_as_float(Zc.x), Zy = __int_as_float(Zc.y);
                if (Zx * Zx + Zy * Zy > M2f4) { stop = 1; break; }
                dyn = false;
                continue;
            }
            if (Zc.w & 1) {
                // Z_w exactly 0 (the critical point, flagged in the table):
                // ZZ = dz escapes iff |dz|^2 > M^2; otherwise the
                // componentwise test |dz| <= |dz| and the Xrange confirmation
                // hold, and the dynamic rebase leaves dz unchanged
                const float2 df = fe_to_f(as_fe(s.ux, s.uy, s.E));
                if (df.x * df.x + df.y * df.y > M2f) { stop = 1; break; }
                dyn = true;
                rebase_derivs(s, R, w, n, order, dzndc_on, dzndz_on, nullify);
                w = 0; nreb++;
                Zc = __ldg(&Zp[0]);
                continue;
            }
        }
        // ---------------- exact tests ---------------------------------------
        fe Zn = ld_fe(R.Zf, w);
        fe dz = as_fe(s.ux, s.uy, s.E);
        float2 zf = fe_to_f(Zn), df = fe_to_f(dz);
        float XX = zf.x + df.x, YY = zf.y + df.y;
        if (XX * XX + YY * YY > M2f) { stop = 1; break; }
        if (w >= div_iter - 1) {        // rebase when the reference diverges
            from_fe_u(s, fe_norm(fe_add(Zn, dz)), cmx, cmy, Ec);
            rebase_derivs(s, R, w, n, order, dzndc_on, dzndz_on, nullify);
            w = 0; nreb++;
            Zc = __ldg(&Zp[0]);
            continue;
        }
        // dynamic rebase (:1317-1320): integer pre-rejection (|Z|inf >=
        // 4 |dz|inf), then the componentwise test in FP32 when both values
        // are normal floats, in double (the reference's std values) when the
        // FP32 test lies within its rounding of a tie
        dyn = false;
        if (Zn.e < dz.e + 2) {
            int dec = 2;                                  // 0 no, 1 yes, 2 undecided
            if (Zn.e > -100 && Zn.e < 100 && dz.e > -100 && dz.e < 100) {
                const float tau = 0x1p-21f * (fabsf(zf.x) + fabsf(zf.y))
                                  + 0x1p-20f * (fabsf(df.x) + fabsf(df.y));
                const float ax = fabsf(XX) - fabsf(df.x), ay = fabsf(YY) - fabsf(df.y);
                if (ax > tau || ay > tau) dec = 0;
                else if (ax < -tau && ay < -tau) dec = 1;
            }
            if (dec == 2) {
                fe d = dz;
                int wv = w;
                opaque(d.x, d.y, d.e, wv);
                dec = rebase_test_double(d, R.Zn, wv);
            }
            dyn = dec == 1;
            if (dyn) {
                fe ZZ = fe_add(dz, Zn);
                bool ok = true;
                if (xrsem) {
                    fe a = fe_norm(ZZ);
                    int k = a.e - dz.e;
                    float l = a.x * a.x + a.y * a.y, r = dz.x * dz.x + dz.y * dz.y;
                    if (a.e == FE_ZERO_E) ok = true;
                    else if (k >= 2) ok = false;
                    else if (k <= -2) ok = true;
                    else ok = (k == 1 ? l * 4.f : (k == -1 ? l * 0.25f : l)) <= r;
                }
                if (ok) {
                    from_fe_u(s, fe_norm(ZZ), cmx, cmy, Ec);
                    rebase_derivs(s, R, w, n, order, dzndc_on, dzndz_on, nullify);
                    w = 0; nreb++;
                    Zc = __ldg(&Zp[0]);
                    continue;
                }
            }
        }
    }
    // end of iterations (:1375-1385): the read-out sums in double (Xrange),
    // from the double forms of the orbit and of the reference derivative
    fe dzf = as_fe(s.ux, s.uy, s.E);
    double2 zn = cadd(fe_to_d(dzf), __ldg(&R.Zn[w]));
    double2 dzc = cx(0., 0.);
    // dzndc in the tile's unit: the reference's scale times 2^dzs
    if (dzndc_on) {
        const xc v = (s.F == FE_ZERO_E || (s.vx == 0.f && s.vy == 0.f))
                         ? xc_zero() : xc_make((double)s.vx, (double)s.vy, s.F);
        const xc D = R.dZndc_xm ? xc_make(__ldg(&R.dZndc_xm[w]).x, __ldg(&R.dZndc_xm[w]).y,
                                          __ldg(&R.dZndc_xe[w]))
                                : xr_from(__ldg(&R.dZndc[w]));
        xc t = xr_add(v, D);
        t.e += T.dzs;
        dzc = xr_to_std(t);
    }
    double2 *Z = (double2 *)T.Z;
    Z[ip] = zn;
    if (dzndz_on) Z[T.i_dzndz * np + ip] = xrsem ? cx(0., 0.) : fe_to_d(as_fe(s.qx, s.qy, s.G));
    if (dzndc_on && T.proj) dzc = rmul(fsg_dzndc_modifier(T, ip), dzc);
    if (dzndc_on) Z[T.i_dzndc * np + ip] = dzc;
    if (T.U) T.U[ip] = w;
    T.stop_iter[ip] = n;
    T.stop_reason[ip] = stop;
    fsg_epilogue(T, C, ip, zn, hypot(dzc.x, dzc.y), n);
    return n;
}

// 128-thread blocks, 7 per SM: 72 registers a thread without spills, 28 warps
// an SM (the register file's limit at 72); with interior detection 6 per SM
// (80 registers)
#define FE32_BLOCK 128
template <bool INTERIOR>
// Shared memory, sized at launch (the unified L1 keeps the rest for the orbit
// and BLA tables): per-thread statistics (iterations, full steps, BLA steps,
// rebases; 64-bit accumulators would hold 8 registers in the loop), then the
// pixel offsets of the launch's tiles.
__global__ void __launch_bounds__(FE32_BLOCK, INTERIOR ? 6 : 7) k_perturb_m2_fe32(WorkDev W, CalcDev C) {
    extern __shared__ unsigned long long fe32_smem[];
    unsigned long long *acc = fe32_smem + threadIdx.x;         // acc[k * blockDim.x]
    long long *s_start = (long long *)(fe32_smem + 4 * blockDim.x);
    const int nb = blockDim.x;
    for (int k = 0; k < 4; k++) acc[k * nb] = 0ULL;
    fsg_load_starts(W, s_start);
    int t; long long ip;
    while (true) {
        if (*W.cancel) { *W.status = 1; break; }
        if (!fsg_claim(W, s_start, t, ip)) break;
        unsigned nfull = 0, nbla = 0, nreb = 0;
        const int n = pixel_fe32<INTERIOR>(W.tiles[t], C, ip, nfull, nbla, nreb);
        fsg_account(W, (unsigned long long)n);
        acc[0] += (unsigned long long)n;
        acc[nb] += nfull;
        acc[2 * nb] += nbla;
        acc[3 * nb] += nreb;
    }
    fsg_flush_stats(W, acc[0], acc[nb], acc[2 * nb], acc[3 * nb]);
}

void fsg_launch_perturb_fe32(const WorkDev &W, const CalcDev &C, int grid, int block,
                             cudaStream_t s) {
    const int b = (block > 0 && block <= FE32_BLOCK) ? block : FE32_BLOCK;
    const size_t smem = sizeof(unsigned long long) * (4 * (size_t)b + W.ntiles + 1);
    if (C.interior)
        k_perturb_m2_fe32<true><<<fsg_auto_grid(k_perturb_m2_fe32<true>, grid, b,
                                                W.total - W.base, smem), b, smem, s>>>(W, C);
    else
        k_perturb_m2_fe32<false><<<fsg_auto_grid(k_perturb_m2_fe32<false>, grid, b,
                                                 W.total - W.base, smem), b, smem, s>>>(W, C);
}
