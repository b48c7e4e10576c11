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
//   * fast step, when |dz|_inf < 2^-26 |Z|_inf (almost every step of a deep
//     zoom): dz^2 and dz * dzndc are below FP32 resolution against 2 Z dz and
//     Z dzndc, so  u' = 2 Z u + cu  and  v' = 2 (Z v + 2^k D u)  with
//     k = De + E - F -- plain FP32 FMAs on the orbit's float copy;
//   * exact step otherwise (Z tiny or zero, rebases, escapes): every operation
//     in fe arithmetic (fsg_num.cuh), and the reference's tests in their exact
//     form: the componentwise rebase test on the double values (with
//     to_standard()'s underflow), then -- following the Xrange branch -- the
//     extended |Z + dz|^2 <= |dz|^2 confirmation.
// The BLA validity test |dz| < r compares exponents first and mantissas only
// on near ties, which is exact with respect to the reference's comparison of
// to_standard(dz) (it underflows to 0 only below every r > 0).
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

// |dz| < r for dz = u 2^E with magnitude exponent L (of max(|ux|, |uy|) 2^E),
// r given as (mantissa in [1, 2), exponent)
__device__ __forceinline__ bool lt_r(float ux, float uy, int E, int L, float rm, int re) {
    int k = re - L;
    if (k >= 2) return true;
    if (k <= -2) return false;
    // compare u^2 2^(2E) against rm^2 2^(2 re): scale u by 2^-(L - E)
    float s = p2f(E - L);
    float x = ux * s, y = uy * s;
    float r2 = rm * rm;
    r2 = (k == 1) ? r2 * 4.f : ((k == -1) ? r2 * 0.25f : r2);
    return x * x + y * y < r2;
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
__device__ __forceinline__ void from_fe_u(Lane &s, fe d, float cmx, float cmy, int Ec) {
    if (d.e == FE_ZERO_E || (d.x == 0.f && d.y == 0.f)) { s.ux = 0.f; s.uy = 0.f; s.E = Ec; }
    else {
        s.E = max(d.e, Ec - 100);
        float sc = p2f(d.e - s.E);
        s.ux = d.x * sc; s.uy = d.y * sc;
    }
    set_cu(s, cmx, cmy, Ec);
}
__device__ __forceinline__ void store_fe(float &x, float &y, int &e, fe d) {
    if (d.e == FE_ZERO_E || (d.x == 0.f && d.y == 0.f)) { x = 0.f; y = 0.f; e = FE_ZERO_E; }
    else { x = d.x; y = d.y; e = d.e; }
}

__device__ __forceinline__ int bla_lookup_fast(const RefDev &R, const Lane &s, int L, int w,
                                               int &ib) {
    int it = w >> FSG_STG_COMPRESSED;
    int stages = FSG_STG_COMPRESSED;
    for (int k = FSG_STG_COMPRESSED; k < R.stages; k++) {
        stages = k;
        if (it & 1) break;
        it >>= 1;
    }
    int invalid_step = R.first_invalid - w;
    for (int stg = stages; stg >= FSG_STG_COMPRESSED; stg--) {
        int step = 1 << stg;
        if (step >= invalid_step) continue;
        int idx = 2 * (w >> FSG_STG_COMPRESSED) + ((1 << (stg - FSG_STG_COMPRESSED)) - 1);
        float rm = __int_as_float(__ldg(&R.bla_f_A[idx].w));
        int re = __ldg(&R.bla_f_B[idx].w);
        bool ok = (L == FE_ZERO_E) ? (re != FE_ZERO_E) : lt_r(s.ux, s.uy, s.E, L, rm, re);
        if (ok) { ib = idx; return step; }
    }
    return 0;
}

__device__ __forceinline__ void pixel_fe32(const TileDev &T, const CalcDev &C, long long ip,
                                           unsigned long long &nfull, unsigned long long &nbla,
                                           unsigned long long &nreb, unsigned long long &itsum) {
    const RefDev &R = *T.ref;
    const long long np = (long long)T.nx * T.ny;
    const int dzndz_on = C.interior, dzndc_on = C.calc_dzndc, xrsem = C.xrsem;
    const int order = R.order, div_iter = R.div_iter, w_wrapped = R.len;
    const float M2f = (float)C.M2;
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
    set_cu(s, cmx, cmy, Ec);
    int w = 0, n = 0; signed char stop = -1;
    bool nullify = false, dyn = true;
    int4 Zc = __ldg(&R.Zp[0]);

    for (;;) {
        // ---------------- BLA step (perturbation.py:1121-1154) -------------
        if (C.bla && (w & 7) == 0) {
            int ib;
            int L = mag_u(s);
            int step = bla_lookup_fast(R, s, L, w, ib);
            if (step != 0) {
                int4 Av = __ldg(&R.bla_f_A[ib]), Bv = __ldg(&R.bla_f_B[ib]);
                float Ax = __int_as_float(Av.x), Ay = __int_as_float(Av.y);
                float Bx = __int_as_float(Bv.x), By = __int_as_float(Bv.y);
                // dz' = A dz + B dc, on the scale of the larger term
                int ea = (L == FE_ZERO_E) ? FE_ZERO_E : L + Av.z;
                int eb = dc_zero ? FE_ZERO_E : Ec + Bv.z;
                int En = max(ea, eb);
                if (En == FE_ZERO_E) En = Ec;
                float sa = p2f(s.E + Av.z - En), sb = p2f(Ec + Bv.z - En);
                float bx = Bx * cmx - By * cmy, by = Bx * cmy + By * cmx;
                float nx = (Ax * s.ux - Ay * s.uy) * sa + bx * sb;
                float ny = (Ax * s.uy + Ay * s.ux) * sa + by * sb;
                s.ux = nx; s.uy = ny; s.E = max(En, Ec - 100);
                if (s.E != En) { float sc = p2f(En - s.E); s.ux *= sc; s.uy *= sc; }
                set_cu(s, cmx, cmy, Ec);
                renorm_u(s, cmx, cmy, Ec);
                if (dzndc_on) {
                    float vx = Ax * s.vx - Ay * s.vy, vy = Ax * s.vy + Ay * s.vx;
                    s.vx = vx; s.vy = vy; s.F += Av.z;
                    renorm_v(s.vx, s.vy, s.F);
                }
                if (dzndz_on) {
                    float qx = Ax * s.qx - Ay * s.qy, qy = Ax * s.qy + Ay * s.qx;
                    s.qx = qx; s.qy = qy; s.G += Av.z;
                    renorm_v(s.qx, s.qy, s.G);
                }
                n += step;
                w = (w + step) % order;
                Zc = __ldg(&R.Zp[w]);
                nbla++;
                continue;
            }
        }
        // ---------------- full step (perturbation.py:1158-1214) ------------
        n += 1;
        nfull++;
        const int Ldz = mag_u(s);
        if (!dzndz_on && Zc.z != FE_ZERO_E && Zc.z >= Ldz + 26) {
            // fast step: |dz| < 2^-26 |Z|
            float Zx = __int_as_float(Zc.x), Zy = __int_as_float(Zc.y);
            if (dzndc_on) {
                float dx = 0.f, dy = 0.f; int De = 0;
                if (!dyn) {
                    int4 Dv = __ldg(&R.dZndc_f[w]);
                    dx = __int_as_float(Dv.x); dy = __int_as_float(Dv.y); De = Dv.z;
                    if (De == FE_ZERO_E) { dx = 0.f; dy = 0.f; De = 0; }
                }
                bool dzero = (dx == 0.f && dy == 0.f) || Ldz == FE_ZERO_E;
                if (s.vx == 0.f && s.vy == 0.f) s.F = dzero ? 0 : De + s.E;
                int kd = De + s.E - s.F;
                if (!dzero && kd > 100) {          // the D dz term dominates: rescale v
                    int Fn = De + s.E - 30;
                    float sc = p2f(s.F - Fn);
                    s.vx *= sc; s.vy *= sc; s.F = Fn; kd = 30;
                }
                float sk = dzero ? 0.f : p2f(kd);
                float ax = dx * s.ux - dy * s.uy, ay = dx * s.uy + dy * s.ux;
                float vx = 2.f * (Zx * s.vx - Zy * s.vy + sk * ax);
                float vy = 2.f * (Zx * s.vy + Zy * s.vx + sk * ay);
                s.vx = vx; s.vy = vy;
                renorm_v(s.vx, s.vy, s.F);
            }
            float nx = 2.f * (Zx * s.ux - Zy * s.uy) + s.cux;
            float ny = 2.f * (Zx * s.uy + Zy * s.ux) + s.cuy;
            s.ux = nx; s.uy = ny;
            renorm_u(s, cmx, cmy, Ec);
        } else {
            // exact step in fe arithmetic
            fe Zw = ld_fe(R.Zf, w);
            fe dz = as_fe(s.ux, s.uy, s.E);
            if (dzndc_on) {
                fe D = dyn ? fe_zero() : ld_fe(R.dZndc_f, w);
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
            from_fe_u(s, dz, cmx, cmy, Ec);
        }
        w += 1;
        if (w >= order) w = w % order;
        // ---------------- max_iter (:1218-1220) ----------------------------
        if (n >= C.max_iter) { stop = 0; break; }
        // ---------------- interior detection (:1224-1246) ------------------
        if (dzndz_on) {
            int k = nullify ? 0 : ((n == order) ? w_wrapped : w);
            fe ZdZ = fe_add(as_fe(s.qx, s.qy, s.G), ld_fe(R.dZndz_f, k));
            if (fe_abs2_lt(ZdZ, C.eps2)) { stop = 2; break; }
        }
        Zc = __ldg(&R.Zp[w]);
        const int Ln = mag_u(s);
        if (Zc.z != FE_ZERO_E && Zc.z >= Ln + 26 && w < div_iter - 1) {
            // fast tests: |dz| < 2^-26 |Z_next|, no rebase possible
            float Zx = __int_as_float(Zc.x), Zy = __int_as_float(Zc.y);
            if (Zx * Zx + Zy * Zy > M2f) { stop = 1; break; }
            dyn = false;
            continue;
        }
        // ---------------- exact tests ---------------------------------------
        fe Zn = ld_fe(R.Zf, w);
        fe dz = as_fe(s.ux, s.uy, s.E);
        float2 zf = fe_to_f(Zn), df = fe_to_f(dz);
        float XX = zf.x + df.x, YY = zf.y + df.y;
        if (XX * XX + YY * YY > M2f) { stop = 1; break; }
        if (w >= div_iter - 1) {        // rebase when the reference diverges
            from_fe_u(s, fe_norm(fe_add(Zn, dz)), cmx, cmy, Ec);
            if (dzndc_on)
                store_fe(s.vx, s.vy, s.F,
                         fe_norm(fe_add(as_fe(s.vx, s.vy, s.F), ld_fe(R.dZndc_f, w))));
            if (dzndz_on) {
                if (!nullify)
                    store_fe(s.qx, s.qy, s.G,
                             fe_norm(fe_add(as_fe(s.qx, s.qy, s.G),
                                            ld_fe(R.dZndz_f, (n == order) ? w_wrapped : w))));
                nullify = true;
            }
            w = 0; nreb++;
            Zc = __ldg(&R.Zp[0]);
            continue;
        }
        // dynamic rebase: integer pre-rejection, then the double-range test
        dyn = false;
        if (Zn.e < dz.e + 2) {
            double2 dd = fe_to_d(dz);
            double2 Zd = __ldg(&R.Zn[w]);
            double2 ZZd = cadd(dd, Zd);
            dyn = (fabs(ZZd.x) <= fabs(dd.x)) && (fabs(ZZd.y) <= fabs(dd.y));
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
                    if (dzndc_on)
                        store_fe(s.vx, s.vy, s.F,
                                 fe_norm(fe_add(as_fe(s.vx, s.vy, s.F), ld_fe(R.dZndc_f, w))));
                    if (dzndz_on) {
                        if (!nullify)
                            store_fe(s.qx, s.qy, s.G,
                                     fe_norm(fe_add(as_fe(s.qx, s.qy, s.G),
                                                    ld_fe(R.dZndz_f, (n == order) ? w_wrapped : w))));
                        nullify = true;
                    }
                    w = 0; nreb++;
                    Zc = __ldg(&R.Zp[0]);
                    continue;
                }
            }
        }
    }
    // end of iterations (:1375-1385)
    fe dzf = as_fe(s.ux, s.uy, s.E);
    double2 zn = cadd(fe_to_d(dzf), __ldg(&R.Zn[w]));
    double2 dzc = cx(0., 0.);
    if (dzndc_on) dzc = fe_to_d(fe_add(as_fe(s.vx, s.vy, s.F), ld_fe(R.dZndc_f, w)));
    double2 *Z = (double2 *)T.Z;
    Z[ip] = zn;
    if (dzndz_on) Z[T.i_dzndz * np + ip] = xrsem ? cx(0., 0.) : fe_to_d(as_fe(s.qx, s.qy, s.G));
    if (dzndc_on) Z[T.i_dzndc * np + ip] = dzc;
    if (T.U) T.U[ip] = w;
    T.stop_iter[ip] = n;
    T.stop_reason[ip] = stop;
    fsg_epilogue(T, C, ip, zn, hypot(dzc.x, dzc.y), n);
    itsum += (unsigned long long)n;
}

__global__ void __launch_bounds__(256) k_perturb_m2_fe32(WorkDev W, CalcDev C) {
    __shared__ long long s_start[FSG_MAX_TILES_PER_LAUNCH + 1];
    fsg_load_starts(W, s_start);
    unsigned long long nfull = 0, nbla = 0, nreb = 0, itsum = 0;
    int t; long long ip;
    while (true) {
        if (*W.cancel) { *W.status = 1; break; }
        if (!fsg_claim(W, s_start, t, ip)) break;
        pixel_fe32(W.tiles[t], C, ip, nfull, nbla, nreb, itsum);
    }
    fsg_flush_stats(W, itsum, nfull, nbla, nreb);
}

void fsg_launch_perturb_fe32(const WorkDev &W, const CalcDev &C, int grid, int block,
                             cudaStream_t s) {
    k_perturb_m2_fe32<<<fsg_auto_grid(k_perturb_m2_fe32, grid, block, W.total), block, 0, s>>>(W, C);
}
