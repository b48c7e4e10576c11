// fsg_perturb_fe32.cu -- power-2 Mandelbrot perturbation loop with deltas held
// as FP32 mantissa + int32 exponent ("fe").
//
// Same control flow as the reference's numba_iterate (perturbation.py:1065-1400):
// BLA attempt every 8 iterations, full step, max_iter / interior / escape
// tests, rebase on reference divergence and Zhuoran's dynamic rebase.  The bulk
// arithmetic (the delta, dz/dc and dz/dz recurrences, BLA steps, escape test)
// runs on the FP32 pipe with integer exponent bookkeeping.  FP64 is used only
// where the reference's decisions are sensitive to the double range:
//   * the componentwise rebase test |Z + dz| <= |dz| is first rejected in
//     integer arithmetic when |Z|_inf >= 4 |dz|_inf, and otherwise evaluated
//     on the double values exactly as the reference does (to_standard()
//     underflow included), followed when the Xrange branch is followed by the
//     extended |Z + dz|^2 <= |dz|^2 confirmation;
//   * the final zn / dzndc read out (double results, as the reference's
//     complex128 outputs).
// The BLA validity test |dz| < r compares exponents first and mantissas only
// for the near ties, which is exact with respect to the reference's
// comparison of to_standard(dz) (it underflows to 0 only below every r > 0).
#include "fsg_internal.cuh"

__device__ __forceinline__ fe ld_fe(const int4 *p, int i) {
    int4 v = __ldg(&p[i]);
    return fe_make(__int_as_float(v.x), __int_as_float(v.y), v.z);
}

// |dz| < r, dz normalised, r given as (mantissa in [1, 2) bits, exponent)
__device__ __forceinline__ bool fe_lt_r(fe dz, float rm, int re) {
    int k = re - dz.e;
    if (k >= 2) return true;
    if (k <= -2) return false;
    float r2 = rm * rm;
    r2 = (k == 1) ? r2 * 4.f : ((k == -1) ? r2 * 0.25f : r2);
    return dz.x * dz.x + dz.y * dz.y < r2;
}

__device__ __forceinline__ int bla_lookup_fe(const RefDev &R, fe dz, int w, int &ib) {
    int it = w >> FSG_STG_COMPRESSED;
    int stages = FSG_STG_COMPRESSED;
    for (int s = FSG_STG_COMPRESSED; s < R.stages; s++) {
        stages = s;
        if (it & 1) break;
        it >>= 1;
    }
    int invalid_step = R.first_invalid - w;
    for (int stg = stages; stg >= FSG_STG_COMPRESSED; stg--) {
        int step = 1 << stg;
        if (step >= invalid_step) continue;
        int idx = 2 * (w >> FSG_STG_COMPRESSED) + ((1 << (stg - FSG_STG_COMPRESSED)) - 1);
        int4 Av = __ldg(&R.bla_f_A[idx]);
        int re = __ldg(&R.bla_f_B[idx]).w;
        if (fe_lt_r(dz, __int_as_float(Av.w), re)) { ib = idx; return step; }
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
    // c from the pixel (perturbation.py:2214-2230), kept in fe form
    double2 pp = fsg_pixel(T, ip);
    double px = pp.x, py = pp.y;
    double x1 = T.lin[0] * px + T.lin[1] * py;
    double y1 = T.lin[2] * px + T.lin[3] * py;
    xf dxr; dxr.m = T.dx_m; dxr.e = T.dx_e;
    xc c_xr = xr_add(xf_mul_c(dxr, cx(x1, y1)), xc_make(T.drift_re, T.drift_im, T.drift_e));
    const fe dc = fe_from_xc(c_xr);

    fe dz = fe_zero(), dzndc = fe_zero(), dzndz = fe_zero();
    int w = 0, n = 0; signed char stop = -1;
    bool nullify = false, dyn = true;
    int poll = 0;

    for (;;) {
        if (C.bla && (w & 7) == 0) {
            int ib;
            int step = bla_lookup_fe(R, dz, w, ib);
            if (step != 0) {
                int4 Av = __ldg(&R.bla_f_A[ib]), Bv = __ldg(&R.bla_f_B[ib]);
                fe A = fe_make(__int_as_float(Av.x), __int_as_float(Av.y), Av.z);
                fe B = fe_make(__int_as_float(Bv.x), __int_as_float(Bv.y), Bv.z);
                n += step;
                w = (w + step) % order;
                dz = fe_norm(fe_add(fe_mul(A, dz), fe_mul(B, dc)));
                if (dzndc_on) dzndc = fe_norm(fe_mul(A, dzndc));
                if (dzndz_on) dzndz = fe_norm(fe_mul(A, dzndz));
                nbla++;
                continue;
            }
        }
        n += 1;
        nfull++;
        int4 Zv = __ldg(&R.Zf[w]);
        fe Zw = fe_make(__int_as_float(Zv.x), __int_as_float(Zv.y), Zv.z);
        if (dzndc_on) {
            fe D = dyn ? fe_zero() : ld_fe(R.dZndc_f, w);
            fe t = fe_add(Zw, dz);
            dzndc = fe_norm(fe_scale2(fe_add(fe_mul(t, dzndc), fe_mul(D, dz)), 1));
        }
        if (dzndz_on) {
            fe D = ld_fe(R.dZndz_f, nullify ? 0 : w);
            fe t = fe_add(Zw, dz);
            dzndz = fe_norm(fe_scale2(fe_add(fe_mul(t, dzndz), fe_mul(D, dz)), 1));
        }
        dz = fe_norm(fe_add(fe_mul(dz, fe_add(dz, fe_scale2(Zw, 1))), dc));
        w += 1;
        if (w >= order) w = w % order;
        if (n >= C.max_iter) { stop = 0; break; }
        if (dzndz_on) {
            int k = nullify ? 0 : ((n == order) ? w_wrapped : w);
            fe ZdZ = fe_add(dzndz, ld_fe(R.dZndz_f, k));
            if (fe_abs2_lt(ZdZ, C.eps2)) { stop = 2; break; }
        }
        // escape test on the FP32 pipe
        int4 Zn4 = __ldg(&R.Zf[w]);
        fe Zn = fe_make(__int_as_float(Zn4.x), __int_as_float(Zn4.y), Zn4.z);
        float2 zf = fe_to_f(Zn), df = fe_to_f(dz);
        float XX = zf.x + df.x, YY = zf.y + df.y;
        if (XX * XX + YY * YY > M2f) { stop = 1; break; }
        if (w >= div_iter - 1) {
            dz = fe_norm(fe_add(Zn, dz));
            if (dzndc_on) dzndc = fe_norm(fe_add(dzndc, ld_fe(R.dZndc_f, w)));
            if (dzndz_on) {
                if (!nullify) dzndz = fe_norm(fe_add(dzndz, ld_fe(R.dZndz_f, (n == order) ? w_wrapped : w)));
                nullify = true;
            }
            w = 0; nreb++;
            continue;
        }
        // dynamic rebase: integer pre-rejection, then the double-range test
        dyn = false;
        if (Zn4.w < dz.e + 2) {
            double2 dd = fe_to_d(dz);
            double2 Zd = __ldg(&R.Zn[w]);
            double2 ZZd = cadd(dd, Zd);
            dyn = (fabs(ZZd.x) <= fabs(dd.x)) && (fabs(ZZd.y) <= fabs(dd.y));
            if (dyn) {
                fe ZZ = fe_add(dz, Zn);
                bool ok = true;
                if (xrsem) {
                    fe a = fe_norm(ZZ);
                    // |ZZ|^2 <= |dz|^2 in extended range
                    int k = a.e - dz.e;
                    float l = a.x * a.x + a.y * a.y, r = dz.x * dz.x + dz.y * dz.y;
                    if (a.e == FE_ZERO_E) ok = true;
                    else if (k >= 2) ok = false;
                    else if (k <= -2) ok = true;
                    else ok = (k == 1 ? l * 4.f : (k == -1 ? l * 0.25f : l)) <= r;
                }
                if (ok) {
                    dz = fe_norm(ZZ);
                    if (dzndc_on) dzndc = fe_norm(fe_add(dzndc, ld_fe(R.dZndc_f, w)));
                    if (dzndz_on) {
                        if (!nullify) dzndz = fe_norm(fe_add(dzndz, ld_fe(R.dZndz_f, (n == order) ? w_wrapped : w)));
                        nullify = true;
                    }
                    w = 0; nreb++;
                    continue;
                }
            }
        }
        if (++poll == FSG_CANCEL_POLL) {   // bounded latency for fsg_cancel
            poll = 0;
        }
    }
    double2 zn = cadd(fe_to_d(dz), __ldg(&R.Zn[w]));
    double2 dzc = cx(0., 0.);
    if (dzndc_on) dzc = fe_to_d(fe_add(dzndc, ld_fe(R.dZndc_f, w)));
    double2 *Z = (double2 *)T.Z;
    Z[ip] = zn;
    if (dzndz_on) Z[T.i_dzndz * np + ip] = xrsem ? cx(0., 0.) : fe_to_d(dzndz);
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
    k_perturb_m2_fe32<<<grid, block, 0, s>>>(W, C);
}
