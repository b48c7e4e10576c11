// fsg_std.cu -- standard (non-perturbation) escape-time loops, FP64.
//
// Power-2 Mandelbrot: core.py:2935-3004 numba_cycles / numba_iterate and
// models/mandelbrot_M2.py:309-334 iterate_once; power-n Mandelbrot:
// models/mandelbrot_Mn.py:317-355.  Burning Ship family:
// core.py:3007-3056 numba_iterate_BS and models/burning_ship.py:350-434.
// The reference compiles these without fastmath, so this file is built with
// -fmad=false: each operation rounds once, in the order of the reference.
#include "fsg_internal.cuh"

__device__ __forceinline__ double sgn(double x) { return x < 0. ? -1. : 1.; }

// core.py:3161-3194 c_from_pix, Cartesian projection
__device__ __forceinline__ double2 std_c(const TileDev &T, long long ip) {
    double2 pp = fsg_pixel(T, ip);
    double px = pp.x, py = pp.y;
    double x1 = T.lin[0] * px + T.lin[1] * py;
    double y1 = T.lin[2] * px + T.lin[3] * py;
    return cadd(cx(T.cre, T.cim), rmul(T.dx, cx(x1, y1)));
}

// OPT: the optional outputs d2zndc2 (mandelbrot_M2.py:316-317) and the orbit
// point n - backshift (core.py:2965-3004)
#define FSG_STD_CHUNK 16        // steps between two block-level compaction checks

template <bool OPT>
__global__ void __launch_bounds__(256) k_std_m2(WorkDev W, CalcDev C) {
    __shared__ long long s_start[FSG_MAX_TILES_PER_LAUNCH + 1];
    // pixel states moved by the compaction (one slot per thread)
    __shared__ double2 s_c[256], s_zn[256], s_dzndz[256], s_dzndc[256];
    __shared__ double2 s_d2[OPT ? 256 : 1];
    __shared__ OrbitSnap<double2> s_S[OPT ? 256 : 1];
    __shared__ long long s_ip[256];
    __shared__ int s_t[256], s_n[256];
    __shared__ int s_cnt;
    fsg_load_starts(W, s_start);
    unsigned long long it_sum = 0, steps = 0;
    const int bs = OPT ? C.backshift : 0;
    const bool d2_on = OPT && C.d2;
    // One pass of the inner loop is one step of the lane's pixel; a lane
    // whose pixel stops stores it and takes the next one within the pass.
    // Every FSG_STD_CHUNK steps the block counts its live pixels: once the
    // queue is empty and at most 3/4 of the threads hold one, the states move
    // (bit for bit) to the block's first threads, so that the long pixels of
    // the tail run in full warps -- a warp's FP64 instruction costs the pipe
    // the same with 2 active lanes as with 32.  The interruption flag is
    // polled per pixel, like numba_cycles (core.py:2959-2960).
    int t = 0; long long ip = 0;
    double2 c = cx(0., 0.), zn = c, dzndz = c, dzndc = c, d2 = c;
    OrbitSnap<double2> S;
    int n = 0;
    bool have = !fsg_cancelled(W) && fsg_claim(W, s_start, t, ip);
    bool drained = !have;
    if (have) { c = std_c(W.tiles[t], ip); if (OPT) S.init(bs, zn); }
    for (;;) {
        for (int k = 0; k < FSG_STD_CHUNK && have; k++) {
            n += 1;
            signed char reason = -1;
            bool stop = true;
            if (n >= C.max_iter) {
                reason = 0;
            } else {
                if (d2_on) d2 = rmul2(cadd(cmul(d2, zn), csq(dzndc)));
                dzndc = caddr(cmul(rmul2(dzndc), zn), 1.);
                dzndz = cmul(rmul2(dzndz), zn);
                zn = cadd(csq(zn), c);
                if (n == 1) dzndz = cx(1., 0.);
                if (d_sq_gt(zn.x * zn.x + zn.y * zn.y, C.M2)) reason = 1;
                else if (d_sq_lt(dzndz.x * dzndz.x + dzndz.y * dzndz.y, C.eps2)) reason = 2;
                else stop = false;
            }
            if (OPT && bs > 0) S.take(n, bs, zn);
            if (stop) {
                const TileDev &T = W.tiles[t];
                const long long np = (long long)T.nx * T.ny;
                double2 *Z = (double2 *)T.Z;
                Z[ip] = zn; Z[np + ip] = dzndz; Z[2 * np + ip] = dzndc;
                if (d2_on) Z[3 * np + ip] = d2;
                if (OPT && bs > 0) {
                    double2 zo = S.z2;
                    for (int i2 = S.i2; i2 < n - bs; i2++) zo = cadd(csq(zo), c);   // M2_iterate
                    Z[(long long)T.i_orb * np + ip] = zo;
                }
                T.stop_iter[ip] = n; T.stop_reason[ip] = reason;
                it_sum += (unsigned long long)n; fsg_account(W, (unsigned long long)n); steps += (unsigned long long)(n - 1);
                have = !fsg_cancelled(W) && fsg_claim(W, s_start, t, ip);
                if (have) {
                    c = std_c(W.tiles[t], ip);
                    zn = cx(0., 0.); dzndz = zn; dzndc = zn; d2 = zn; n = 0;
                    if (OPT) S.init(bs, zn);
                } else {
                    drained = true;
                }
            }
        }
        const int live = __syncthreads_count(have);
        if (live == 0) break;
        if (__syncthreads_or(drained) && 4 * live <= 3 * (int)blockDim.x) {
            if (threadIdx.x == 0) s_cnt = 0;
            __syncthreads();
            if (have) {
                const int j = atomicAdd(&s_cnt, 1);
                s_c[j] = c; s_zn[j] = zn; s_dzndz[j] = dzndz; s_dzndc[j] = dzndc;
                s_ip[j] = ip; s_t[j] = t; s_n[j] = n;
                if (OPT) { s_d2[j] = d2; s_S[j] = S; }
            }
            __syncthreads();
            have = (int)threadIdx.x < live;
            if (have) {
                const int j = threadIdx.x;
                c = s_c[j]; zn = s_zn[j]; dzndz = s_dzndz[j]; dzndc = s_dzndc[j];
                ip = s_ip[j]; t = s_t[j]; n = s_n[j];
                if (OPT) { d2 = s_d2[j]; S = s_S[j]; }
            }
            __syncthreads();
        }
    }
    fsg_flush_stats(W, it_sum, steps, 0ULL, 0ULL);
}

// Move the block's live pixel states (one per thread with have set, live in
// all) to its first threads, bit for bit.  Called by every thread of the block.
template <class P>
__device__ __forceinline__ void fsg_block_compact(P *s_px, int *s_cnt, int live, bool &have,
                                                  P &px) {
    if (threadIdx.x == 0) *s_cnt = 0;
    __syncthreads();
    if (have) s_px[atomicAdd(s_cnt, 1)] = px;
    __syncthreads();
    have = (int)threadIdx.x < live;
    if (have) px = s_px[threadIdx.x];
    __syncthreads();
}

// Power-n Mandelbrot: models/mandelbrot_Mn.py:317-355 iterate_once
// (calc_d2zndc2 False): z^(n-1) once per step, z^n = z^(n-1) z.
// a power-n standard pixel's state, for the block compaction
struct StdMnPx {
    double2 c, zn, dzndz, dzndc, d2;
    OrbitSnap<double2> S;
    long long ip; int t, n;
};

template <bool OPT>
__global__ void __launch_bounds__(256) k_std_mn(WorkDev W, CalcDev C) {
    __shared__ long long s_start[FSG_MAX_TILES_PER_LAUNCH + 1];
    __shared__ StdMnPx s_px[256];
    __shared__ int s_cnt;
    fsg_load_starts(W, s_start);
    unsigned long long it_sum = 0, steps = 0;
    const int nexp = C.nexp;
    const double deg = (double)nexp;
    const int bs = OPT ? C.backshift : 0;
    const bool d2_on = OPT && C.d2;
    // lanes step together; a stopped pixel is stored and the next one taken
    // within the pass, and the block compacts its live pixels once the queue
    // is empty (k_std_m2)
    int t = 0; long long ip = 0;
    double2 c = cx(0., 0.), zn = c, dzndz = c, dzndc = c, d2 = c;
    OrbitSnap<double2> S;
    int n = 0;
    bool have = !fsg_cancelled(W) && fsg_claim(W, s_start, t, ip);
    if (have) { c = std_c(W.tiles[t], ip); if (OPT) S.init(bs, zn); }
    bool drained = !have;
    for (;;) {
        for (int k = 0; k < FSG_STD_CHUNK && have; k++) {
            n += 1;
            signed char reason = -1;
            bool stop = true;
            if (n >= C.max_iter) {
                reason = 0;
            } else {
                double2 zm1, zm;
                if (d2_on) {
                    // mandelbrot_Mn.py:325-333; the reference's recurrence
                    // multiplies by dzndz where d/dc of n z^(n-1) dzndc has dzndc
                    double2 zm2 = mn_ipow(zn, nexp - 2);
                    zm1 = cmul(zm2, zn);
                    zm = cmul(zm1, zn);
                    d2 = rmul(deg, cadd(cmul(d2, zm1),
                                        cmul(cmul(rmul((double)(nexp - 1), dzndz), dzndc), zm2)));
                } else {
                    zm1 = mn_ipow(zn, nexp - 1);
                    zm = cmul(zm1, zn);
                }
                dzndc = caddr(cmul(rmul(deg, dzndc), zm1), 1.);
                dzndz = cmul(rmul(deg, dzndz), zm1);
                zn = cadd(zm, c);
                if (n == 1) dzndz = cx(1., 0.);
                if (d_sq_gt(zn.x * zn.x + zn.y * zn.y, C.M2)) reason = 1;
                else if (d_sq_lt(dzndz.x * dzndz.x + dzndz.y * dzndz.y, C.eps2)) reason = 2;
                else stop = false;
            }
            if (OPT && bs > 0) S.take(n, bs, zn);
            if (stop) {
                const TileDev &T = W.tiles[t];
                const long long np = (long long)T.nx * T.ny;
                double2 *Z = (double2 *)T.Z;
                Z[ip] = zn; Z[np + ip] = dzndz; Z[2 * np + ip] = dzndc;
                if (d2_on) Z[3 * np + ip] = d2;
                if (OPT && bs > 0) {
                    double2 zo = S.z2;
                    for (int i2 = S.i2; i2 < n - bs; i2++) zo = cadd(mn_ipow(zo, nexp), c);   // Mn_iterate
                    Z[(long long)T.i_orb * np + ip] = zo;
                }
                T.stop_iter[ip] = n; T.stop_reason[ip] = reason;
                it_sum += (unsigned long long)n; fsg_account(W, (unsigned long long)n); steps += (unsigned long long)(n - 1);
                have = !fsg_cancelled(W) && fsg_claim(W, s_start, t, ip);
            drained |= !have;
                if (have) {
                    c = std_c(W.tiles[t], ip);
                    zn = cx(0., 0.); dzndz = zn; dzndc = zn; d2 = zn; n = 0;
                    if (OPT) S.init(bs, zn);
                }
            }
        }
        const int live = __syncthreads_count(have);
        if (live == 0) break;
        if (__syncthreads_or(drained) && 4 * live <= 3 * (int)blockDim.x) {
            StdMnPx px;
            px.c = c; px.zn = zn; px.dzndz = dzndz; px.dzndc = dzndc; px.d2 = d2; px.S = S;
            px.ip = ip; px.t = t; px.n = n;
            fsg_block_compact(s_px, &s_cnt, live, have, px);
            c = px.c; zn = px.zn; dzndz = px.dzndz; dzndc = px.dzndc; d2 = px.d2; S = px.S;
            ip = px.ip; t = px.t; n = px.n;
        }
    }
    fsg_flush_stats(W, it_sum, steps, 0ULL, 0ULL);
}

// OPT: the orbit point n - backshift (core.py:3007-3056)
// a Burning Ship standard pixel's state, for the block compaction
struct StdBSPx {
    double a, b, X, Y, dXdA, dXdB, dYdA, dYdB;
    OrbitSnap<double2> S;
    long long ip; int t, n;
};

template <bool OPT>
__global__ void __launch_bounds__(256) k_std_bs(WorkDev W, CalcDev C) {
    __shared__ long long s_start[FSG_MAX_TILES_PER_LAUNCH + 1];
    __shared__ StdBSPx s_px[256];
    __shared__ int s_cnt;
    fsg_load_starts(W, s_start);
    unsigned long long it_sum = 0, steps = 0;
    const int flavor = C.flavor;
    const int bs = OPT ? C.backshift : 0;
    // lanes step together; a stopped pixel is stored and the next one taken
    // within the pass, and the block compacts its live pixels once the queue
    // is empty (k_std_m2)
    int t = 0; long long ip = 0;
    double a = 0., b = 0.;
    double X = 0., Y = 0., dXdA = 0., dXdB = 0., dYdA = 0., dYdB = 0.;
    OrbitSnap<double2> S;
    int n = 0;
    bool have = !fsg_cancelled(W) && fsg_claim(W, s_start, t, ip);
    if (have) {
        const double2 c = std_c(W.tiles[t], ip);
        a = c.x; b = c.y;
        if (OPT) S.init(bs, cx(0., 0.));
    }
    bool drained = !have;
    for (;;) {
        for (int k = 0; k < FSG_STD_CHUNK && have; k++) {
            n += 1;
            signed char reason = -1;
            bool stop = true;
            if (n >= C.max_iter) {
                reason = 0;
                if (OPT && bs > 0) S.take(n, bs, cx(X, Y));
            } else {
                double nX, nY, nXa, nXb, nYa, nYb;
                if (flavor == 1) {
                    nX = X * X - Y * Y + a;
                    nY = 2. * fabs(X * Y) - b;
                    nXa = 2. * (X * dXdA - Y * dYdA) + 1.;
                    nXb = 2. * (X * dXdB - Y * dYdB);
                    nYa = 2. * (fabs(X) * sgn(Y) * dYdA + sgn(X) * dXdA * fabs(Y));
                    nYb = 2. * (fabs(X) * sgn(Y) * dYdB + sgn(X) * dXdB * fabs(Y)) - 1.;
                } else if (flavor == 2) {
                    nX = X * X - Y * Y + a;
                    nY = 2. * X * fabs(Y) - b;
                    nXa = 2. * (X * dXdA - Y * dYdA) + 1.;
                    nXb = 2. * (X * dXdB - Y * dYdB);
                    nYa = 2. * (X * sgn(Y) * dYdA + dXdA * fabs(Y));
                    nYb = 2. * (X * sgn(Y) * dYdB + dXdB * fabs(Y)) - 1.;
                } else if (flavor == 3) {
                    nX = X * X - Y * fabs(Y) + a;
                    nY = 2. * X * Y - b;
                    nXa = 2. * (X * dXdA - fabs(Y) * dYdA) + 1.;
                    nXb = 2. * (X * dXdB - fabs(Y) * dYdB);
                    nYa = 2. * (dXdA * Y + X * dYdA);
                    nYb = 2. * (dXdB * Y + X * dYdB) - 1.;
                } else if (flavor == 4) {
                    double q = X * X - Y * Y;
                    nX = fabs(q) + a;
                    nY = 2. * X * Y - b;
                    nXa = 2. * sgn(q) * (X * dXdA - Y * dYdA);
                    nXb = 2. * sgn(q) * (X * dXdB - Y * dYdB);
                    nYa = 2. * (dXdA * Y + X * dYdA);
                    nYb = 2. * (dXdB * Y + X * dYdB) - 1.;
                } else {
                    double q = X * X - Y * Y;
                    nX = fabs(q) + a;
                    nY = 2. * fabs(X * Y) - b;
                    nXa = 2. * sgn(q) * (X * dXdA - Y * dYdA);
                    nXb = 2. * sgn(q) * (X * dXdB - Y * dYdB);
                    nYa = 2. * (fabs(X) * sgn(Y) * dYdA + sgn(X) * dXdA * fabs(Y));
                    nYb = 2. * (fabs(X) * sgn(Y) * dYdB + sgn(X) * dXdB * fabs(Y)) - 1.;
                }
                X = nX; Y = nY; dXdA = nXa; dXdB = nXb; dYdA = nYa; dYdB = nYb;
                bool esc = d_sq_gt(X * X + Y * Y, C.M2);
                if (OPT && bs > 0) S.take(n, bs, cx(X, Y));
                if (esc) reason = 1;
                else stop = false;
            }
            if (!stop) continue;
            const TileDev &T = W.tiles[t];
            const long long np = (long long)T.nx * T.ny;
            double *Z = (double *)T.Z;
            Z[ip] = X; Z[np + ip] = Y; Z[2 * np + ip] = dXdA; Z[3 * np + ip] = dXdB;
            Z[4 * np + ip] = dYdA; Z[5 * np + ip] = dYdB;
            if (OPT && bs > 0) {
                double xo = S.z2.x, yo = S.z2.y;
                for (int i2 = S.i2; i2 < n - bs; i2++) {
                    double nx_, ny_;
                    bs_map(flavor, xo, yo, a, b, nx_, ny_);
                    xo = nx_; yo = ny_;
                }
                Z[(long long)T.i_orb * np + ip] = xo;
                Z[(long long)(T.i_orb + 1) * np + ip] = yo;
            }
            T.stop_iter[ip] = n; T.stop_reason[ip] = reason;
            it_sum += (unsigned long long)n; fsg_account(W, (unsigned long long)n); steps += (unsigned long long)(n - 1);
            have = !fsg_cancelled(W) && fsg_claim(W, s_start, t, ip);
            drained |= !have;
            if (have) {
                const double2 c = std_c(W.tiles[t], ip);
                a = c.x; b = c.y;
                X = 0.; Y = 0.; dXdA = 0.; dXdB = 0.; dYdA = 0.; dYdB = 0.; n = 0;
                if (OPT) S.init(bs, cx(0., 0.));
            }
        }
        const int live = __syncthreads_count(have);
        if (live == 0) break;
        if (__syncthreads_or(drained) && 4 * live <= 3 * (int)blockDim.x) {
            StdBSPx px;
            px.a = a; px.b = b; px.X = X; px.Y = Y; px.dXdA = dXdA; px.dXdB = dXdB;
            px.dYdA = dYdA; px.dYdB = dYdB; px.S = S; px.ip = ip; px.t = t; px.n = n;
            fsg_block_compact(s_px, &s_cnt, live, have, px);
            a = px.a; b = px.b; X = px.X; Y = px.Y; dXdA = px.dXdA; dXdB = px.dXdB;
            dYdA = px.dYdA; dYdB = px.dYdB; S = px.S; ip = px.ip; t = px.t; n = px.n;
        }
    }
    fsg_flush_stats(W, it_sum, steps, 0ULL, 0ULL);
}

// Potential and distance estimate of every pixel of the launch, from the
// values the iteration kernel stored (zn, dzndc or the Jacobian, stop_iter):
// the same formulas on the same values as an in-loop epilogue, run here so
// that the lanes of a warp take them together.  Within the iteration kernel a
// pixel escapes after ~25 iterations on average and its FP64 logarithms ran
// while the other lanes of its warp waited (8.8 of 32 lanes active).
template <bool BS>
__global__ void __launch_bounds__(256) k_std_epilogue(WorkDev W, CalcDev C) {
    __shared__ long long s_start[FSG_MAX_TILES_PER_LAUNCH + 1];
    fsg_load_starts(W, s_start);
    for (long long g = W.base + blockIdx.x * (long long)blockDim.x + threadIdx.x; g < W.total;
         g += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = W.ntiles - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_start[mid] <= g) lo = mid; else hi = mid - 1;
        }
        const TileDev &T = W.tiles[lo];
        if (T.pot == nullptr && T.dem == nullptr) continue;
        const long long ip = g - s_start[lo], np = (long long)T.nx * T.ny;
        const int n = T.stop_iter[ip];
        if (BS) {
            const double *Z = (const double *)T.Z;
            const double dXdA = Z[2 * np + ip], dXdB = Z[3 * np + ip];
            const double dYdA = Z[4 * np + ip], dYdB = Z[5 * np + ip];
            const double absd = 0.5 * (hypot(dXdA + dYdB, dXdB - dYdA) +
                                       hypot(dXdA - dYdB, dXdB + dYdA));
            fsg_epilogue(T, C, ip, cx(Z[ip], Z[np + ip]), absd, n);
        } else {
            const double2 *Z = (const double2 *)T.Z;
            const double2 d = Z[2 * np + ip];
            fsg_epilogue(T, C, ip, Z[ip], hypot(d.x, d.y), n);
        }
    }
}

template <bool OPT>
static void launch_std(const WorkDev &W, const CalcDev &C, int grid, int block, cudaStream_t s) {
    if (C.flavor == 0 && C.nexp != 0)
        k_std_mn<OPT><<<fsg_auto_grid(k_std_mn<OPT>, grid, block, W.total - W.base), block, 0, s>>>(W, C);
    else if (C.flavor == 0)
        k_std_m2<OPT><<<fsg_auto_grid(k_std_m2<OPT>, grid, block, W.total - W.base), block, 0, s>>>(W, C);
    else
        k_std_bs<OPT><<<fsg_auto_grid(k_std_bs<OPT>, grid, block, W.total - W.base), block, 0, s>>>(W, C);
    if (C.flavor == 0)
        k_std_epilogue<false><<<fsg_auto_grid(k_std_epilogue<false>, 0, 256, W.total - W.base), 256, 0, s>>>(
            W, C);
    else
        k_std_epilogue<true><<<fsg_auto_grid(k_std_epilogue<true>, 0, 256, W.total - W.base), 256, 0, s>>>(
            W, C);
}

void fsg_launch_std(const WorkDev &W, const CalcDev &C, int grid, int block, cudaStream_t s) {
    if (C.backshift > 0 || C.d2) launch_std<true>(W, C, grid, block, s);
    else launch_std<false>(W, C, grid, block, s);
}
