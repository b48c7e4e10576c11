// fsg_perturb.cu -- perturbation loops in the reference's two delta forms.
//
// Power-2 Mandelbrot: perturbation.py:988-1400 (numba_cycles_perturb,
// numba_initialize, numba_iterate) with the closures of
// models/mandelbrot_M2.py:591-627 (MN = false) or, for the power-n model,
// models/mandelbrot_Mn.py:626-733 (MN = true, fsg_mn.cuh).  XR = false is the branch with
// xr_detect_activated False (double deltas), XR = true the Xrange branch
// (double mantissa + int32 exponent, numba_xr.py semantics).
// Burning Ship family: perturbation.py:1406-1811 with the closures of
// models/burning_ship.py:19-60, 535-859 (double deltas).
//
// Built with -fmad=false so that every operation rounds once in the order of
// the reference source.  One thread iterates one pixel at a time and claims
// the next pixel from the launch's work counter as soon as it finishes.
#include "fsg_internal.cuh"

#include "fsg_bs.cuh"

__device__ __forceinline__ xc ldx(const double2 *m, const int *e, int i) {
    double2 v = __ldg(&m[i]);
    return xc_make(v.x, v.y, __ldg(&e[i]));
}

template <bool XR, bool MN, bool ORB>
__device__ __forceinline__ void pixel_m2(const TileDev &T, const CalcDev &C, long long ip,
                                         unsigned long long &nfull, unsigned long long &nbla,
                                         unsigned long long &nreb, unsigned long long &itsum) {
    const RefDev &R = *T.ref;
    const long long np = (long long)T.nx * T.ny;
    const int dzndz_on = C.interior, dzndc_on = C.calc_dzndc;
    const int order = R.order, div_iter = R.div_iter, w_wrapped = R.len;
    const int nexp = R.nexp;
    const double *Cb = R.binom;
    // perturbation.py:2214-2230 ref_path_c_from_pix, 2666-2672 lin_proj_impl
    double2 pp = fsg_pixel(T, ip);
    double px = pp.x, py = pp.y;
    double x1 = T.lin[0] * px + T.lin[1] * py;
    double y1 = T.lin[2] * px + T.lin[3] * py;
    xf dxr; dxr.m = T.dx_m; dxr.e = T.dx_e;
    xc c_xr = xr_add(xf_mul_c(dxr, cx(x1, y1)), xc_make(T.drift_re, T.drift_im, T.drift_e));
    double2 c = xr_to_std(c_xr);

    // numba_initialize :1055-1060 (the per-tile Xrange dzndz carry-over of the
    // reference is erased by the first full step, so it starts at zero here)
    double2 zn = cx(0., 0.), dzndc = cx(0., 0.), dzndz = cx(0., 0.);
    xc xzn = xc_zero(), xdzndc = xc_zero(), xdzndz = xc_zero();
    int w = 0, n = 0; signed char stop = -1;
    bool nullify = false, dyn = true;
    const xc xzero = xc_zero();
    // calc_orbit snapshots :1096-1101
    const int bs = ORB ? C.backshift : 0;
    OrbitSnap<double2> S;
    if (ORB) S.init(bs, zn);

    for (;;) {
        // BLA step :1121-1154
        if (C.bla && R.bla_len > 0 && (w & 7) == 0) {
            int ib;
            const int step = bla_possible(R, w) ? bla_lookup_z(R, zn, w, ib) : 0;
            if (step != 0) {
                double2 A = __ldg(&R.Mbla[2 * ib]), B = __ldg(&R.Mbla[2 * ib + 1]);
                n += step;
                w = (w + step) % order;
                if (XR) {
                    xzn = xr_add(xr_mul_s(A, xzn), xr_mul_s(B, c_xr));
                    zn = xr_to_std(xzn);
                    if (dzndc_on) xdzndc = xr_mul_s(A, xdzndc);
                    if (dzndz_on) xdzndz = xr_mul_s(A, xdzndz);
                } else {
                    zn = cadd(cmul(A, zn), cmul(B, c));
                    if (dzndc_on) dzndc = cmul(A, dzndc);
                    if (dzndz_on) dzndz = cmul(A, dzndz);
                }
                nbla++;
                continue;
            }
        }
        // full perturbation step :1158-1214
        n += 1;
        nfull++;
        double2 ref_zn = __ldg(&R.Zn[w]);
        xc ref_zn_xr;
        if (XR) {
            int slot = R.n_xr ? __ldg(&R.xr_slot[w]) : -1;
            ref_zn_xr = (slot >= 0) ? ldx(R.xr_m, R.xr_e, slot) : xr_from(ref_zn);
        }
        if (dzndc_on) {
            if (XR) {
                xc rd = dyn ? xzero : ldx(R.dZndc_xm, R.dZndc_xe, w);
                xdzndc = MN ? mn_p_deriv_x(nexp, Cb, xzn, xdzndc, ref_zn_xr, rd)
                            : xr_mul_2(xr_add(xr_mul(xr_add(ref_zn_xr, xzn), xdzndc), xr_mul(rd, xzn)));
            } else {
                double2 rd = dyn ? cx(0., 0.) : __ldg(&R.dZndc[w]);
                dzndc = MN ? mn_p_deriv(nexp, Cb, zn, dzndc, ref_zn, rd)
                           : rmul2(cadd(cmul(cadd(ref_zn, zn), dzndc), cmul(rd, zn)));
            }
        }
        if (dzndz_on) {
            int k = nullify ? 0 : w;
            if (XR) {
                xc rd = ldx(R.dZndz_xm, R.dZndz_xe, k);
                xdzndz = MN ? mn_p_deriv_x(nexp, Cb, xzn, xdzndz, ref_zn_xr, rd)
                            : xr_mul_2(xr_add(xr_mul(xr_add(ref_zn_xr, xzn), xdzndz), xr_mul(rd, xzn)));
            } else {
                double2 rd = __ldg(&R.dZndz[k]);
                dzndz = MN ? mn_p_deriv(nexp, Cb, zn, dzndz, ref_zn, rd)
                           : rmul2(cadd(cmul(cadd(ref_zn, zn), dzndz), cmul(rd, zn)));
            }
        }
        if (XR) {
            xzn = MN ? mn_p_zn_x(nexp, Cb, xzn, ref_zn_xr, c_xr)
                     : xr_add(xr_mul(xzn, xr_add(xzn, xr_mul_2(ref_zn_xr))), c_xr);
            zn = xr_to_std(xzn);
        } else {
            zn = MN ? mn_p_zn(nexp, Cb, zn, ref_zn, c) : cadd(cmul(zn, cadd(zn, rmul2(ref_zn))), c);
        }
        w += 1;
        if (w >= order) w = w % order;
        // max_iter :1218-1220
        if (n >= C.max_iter) { stop = 0; break; }
        // interior detection :1224-1246
        if (dzndz_on) {
            int k = nullify ? 0 : ((n == order) ? w_wrapped : w);
            bool stat;
            if (XR) {
                xc ZdZ = xr_add(xdzndz, ldx(R.dZndz_xm, R.dZndz_xe, k));
                stat = xf_sq_lt_s(xr_abs2(ZdZ), C.eps2);
            } else {
                double2 ZdZ = cadd(dzndz, __ldg(&R.dZndz[k]));
                stat = d_sq_lt(ZdZ.x * ZdZ.x + ZdZ.y * ZdZ.y, C.eps2);
            }
            if (stat) { stop = 2; break; }
        }
        // divergence :1252-1279
        double2 ref_next = __ldg(&R.Zn[w]);
        double2 ZZ = cadd(zn, ref_next);
        if (ORB) S.take(n, bs, ZZ);                                   // :1265-1273
        if (d_sq_gt(ZZ.x * ZZ.x + ZZ.y * ZZ.y, C.M2)) { stop = 1; break; }
        // rebase when the reference diverges :1283-1313
        if (w >= div_iter - 1) {
            zn = ZZ;
            if (XR) {
                xzn = xr_from(ZZ);
                if (dzndc_on) xdzndc = xr_add(xdzndc, ldx(R.dZndc_xm, R.dZndc_xe, w));
                if (dzndz_on) {
                    if (!nullify) {
                        int k = (n == order) ? w_wrapped : w;
                        xdzndz = xr_add(xdzndz, ldx(R.dZndz_xm, R.dZndz_xe, k));
                    }
                    nullify = true;
                }
            } else {
                if (dzndc_on) dzndc = cadd(dzndc, __ldg(&R.dZndc[w]));
                if (dzndz_on) {
                    if (!nullify) dzndz = cadd(dzndz, __ldg(&R.dZndz[(n == order) ? w_wrapped : w]));
                    nullify = true;
                }
            }
            w = 0; nreb++;
            continue;
        }
        // dynamic rebase :1317-1372, componentwise test
        dyn = d_abs_le(ZZ.x, zn.x) && d_abs_le(ZZ.y, zn.y);
        if (dyn) {
            if (XR) {
                int slot = R.n_xr ? __ldg(&R.xr_slot[w]) : -1;
                xc ZZx = (slot >= 0) ? xr_add(xzn, ldx(R.xr_m, R.xr_e, slot)) : xr_add_s(xzn, ref_next);
                if (xf_le(xr_abs2(ZZx), xr_abs2(xzn))) {
                    xzn = ZZx;
                    zn = xr_to_std(ZZx);
                    if (dzndc_on) xdzndc = xr_add(xdzndc, ldx(R.dZndc_xm, R.dZndc_xe, w));
                    if (dzndz_on) {
                        if (!nullify) {
                            int k = (n == order) ? w_wrapped : w;
                            xdzndz = xr_add(xdzndz, ldx(R.dZndz_xm, R.dZndz_xe, k));
                        }
                        nullify = true;
                    }
                    w = 0; nreb++;
                    continue;
                }
            } else {
                zn = ZZ;
                if (dzndc_on) dzndc = cadd(dzndc, __ldg(&R.dZndc[w]));
                if (dzndz_on) {
                    if (!nullify) dzndz = cadd(dzndz, __ldg(&R.dZndz[(n == order) ? w_wrapped : w]));
                    nullify = true;
                }
                w = 0; nreb++;
                continue;
            }
        }
    }
    // end of iterations :1375-1385
    // dzndc in the tile's unit: the reference's scale times 2^dzs
    if (XR) {
        zn = cadd(xr_to_std(xzn), __ldg(&R.Zn[w]));
        if (dzndc_on) {
            xc t = xr_add(xdzndc, ldx(R.dZndc_xm, R.dZndc_xe, w));
            t.e += T.dzs;
            dzndc = xr_to_std(t);
        }
        dzndz = cx(0., 0.);   // the Xrange branch never writes back Z[dzndz]
    } else {
        zn = cadd(zn, __ldg(&R.Zn[w]));
        if (dzndc_on) {
            dzndc = cadd(dzndc, __ldg(&R.dZndc[w]));
            if (T.dzs != 0) dzndc = cx(ldexp_d(dzndc.x, T.dzs), ldexp_d(dzndc.y, T.dzs));
        }
    }
    double2 *Z = (double2 *)T.Z;
    if (ORB) {
        // :1389-1396, the orbit point n - backshift from the full c
        double2 CC = cadd(c, __ldg(&R.Zn[1]));
        double2 zo = S.z2;
        for (int i2 = S.i2; i2 < n - bs; i2++)
            zo = MN ? cadd(mn_ipow(zo, nexp), CC) : cadd(csq(zo), CC);
        Z[(long long)T.i_orb * np + ip] = zo;
    }
    Z[ip] = zn;
    if (dzndz_on) Z[T.i_dzndz * np + ip] = dzndz;
    // Expmap: derivatives times exp(Re(ht pix) + h_moy) (perturbation.py:1387-1388)
    if (dzndc_on && T.proj) dzndc = rmul(fsg_dzndc_modifier(T, ip), dzndc);
    if (dzndc_on) Z[T.i_dzndc * np + ip] = dzndc;
    if (T.U) T.U[ip] = w;
    T.stop_iter[ip] = n;
    T.stop_reason[ip] = stop;
    fsg_epilogue(T, C, ip, zn, hypot(dzndc.x, dzndc.y), n);
    itsum += (unsigned long long)n;
}

template <bool XR, bool MN, bool ORB>
__global__ void __launch_bounds__(256) k_perturb_m2(WorkDev W, CalcDev C) {
    extern __shared__ long long s_start[];          // [W.ntiles + 1], sized at launch
    fsg_load_starts(W, s_start);
    unsigned long long nfull = 0, nbla = 0, nreb = 0, itsum = 0;
    int t; long long ip;
    while (true) {
        if (*W.cancel) { *W.status = 1; break; }
        if (!fsg_claim(W, s_start, t, ip)) break;
        const unsigned long long before = itsum;
        pixel_m2<XR, MN, ORB>(W.tiles[t], C, ip, nfull, nbla, nreb, itsum);
        fsg_account(W, itsum - before);
    }
    fsg_flush_stats(W, itsum, nfull, nbla, nreb);
}

// Burning Ship family, double deltas: fsg_bs.cuh instantiated on double
// (compiled here, without FMA contraction)
template __global__ void k_perturb_bs<double, 0>(WorkDev W, CalcDev C);
// ... and on float64 Xrange records: the reference's Xrange branch
template __global__ void k_perturb_bs<xf, 0>(WorkDev W, CalcDev C);

template <bool XR, bool MN, bool ORB>
static void launch_m2(const WorkDev &W, const CalcDev &C, int grid, int block, cudaStream_t s) {
    const size_t sm = fsg_starts_smem(W);
    k_perturb_m2<XR, MN, ORB><<<fsg_auto_grid(k_perturb_m2<XR, MN, ORB>, grid, block,
                                              W.total - W.base, sm), block, sm, s>>>(W, C);
}

template <bool ORB>
static void launch_m2_orb(const WorkDev &W, const CalcDev &C, int grid, int block,
                          cudaStream_t s) {
    if (C.nexp != 0 && C.mode == 1) launch_m2<true, true, ORB>(W, C, grid, block, s);
    else if (C.nexp != 0) launch_m2<false, true, ORB>(W, C, grid, block, s);
    else if (C.mode == 1) launch_m2<true, false, ORB>(W, C, grid, block, s);
    else launch_m2<false, false, ORB>(W, C, grid, block, s);
}

void fsg_launch_perturb(const WorkDev &W, const CalcDev &C, int grid, int block, cudaStream_t s) {
    const size_t sm = fsg_starts_smem(W);
    if (C.flavor != 0 && C.mode == 1)
        k_perturb_bs<xf, 0><<<fsg_auto_grid(k_perturb_bs<xf, 0>, grid, block, W.total - W.base, sm),
                              block, sm, s>>>(W, C);
    else if (C.flavor != 0)
        k_perturb_bs<double, 0><<<fsg_auto_grid(k_perturb_bs<double, 0>, grid, block,
                                                W.total - W.base, sm), block, sm, s>>>(W, C);
    else if (C.backshift > 0)
        launch_m2_orb<true>(W, C, grid, block, s);
    else
        launch_m2_orb<false>(W, C, grid, block, s);
}
