// fsg_postproc.cu -- post-processing of the raw outputs on the device:
// orbit-averaged field lines and the DEM normal map.
//
//   k_fieldlines <- Fieldlines_pp (postproc.py:409-530) with
//                   Fieldlines_pp_infinity (:1038-1091) and
//                   Fieldlines_pp_infinity_BS (:1094-1160), Catmull-Rom
//                   weights cm_H0..cm_H3 (:1021-1035)
//   k_normal     <- DEM_normal_pp (postproc.py:533-628) with
//                   apply_unskew_1d (core.py:3147-3158)
//
// Both read the arrays Fractal.calc_raw stores (zn or zn_orbit, dzndc,
// d2zndc2, the Jacobian of the Burning Ship family) and the context of
// Continuous_iter_pp (nu_frac, n).  The transcendental functions are CUDA's
// (sin, cos, atan2, log, hypot): results agree with numpy's to a few ulps.
#include "fsg_internal.cuh"

namespace {

// Catmull-Rom spline weights, postproc.py:1021-1035 (x ** 2 as x * x)
__device__ __forceinline__ double cm_h0(double x) { return 0.5 * x * (-x + x * x); }
__device__ __forceinline__ double cm_h1(double x) { return 0.5 * x * (1. + 4. * x - 3. * (x * x)); }
__device__ __forceinline__ double cm_h2(double x) { return 1. + 0.5 * x * (-5. * x + 3. * (x * x)); }
__device__ __forceinline__ double cm_h3(double x) { return 0.5 * x * (-1. + 2. * x - x * x); }

// the model's map: M2_iterate (mandelbrot_M2.py:14-15), Mn_iterate
// (mandelbrot_Mn.py:13-17, numpy's integer power), BS_iterate
// (burning_ship.py:82-123)
__device__ __forceinline__ double2 fl_map(int model, double2 z, double2 c) {
    if (model == 0) return cadd(csq(z), c);
    if (model > 0) return cadd(mn_ipow(z, model), c);
    double nx, ny;
    bs_map(-model, z.x, z.y, c.x, c.y, nx, ny);
    return cx(nx, ny);
}

}  // namespace

// Fieldlines_pp_infinity(_BS): the angles of n_iter + 3 orbit points from the
// stored start point (beyond |z| > M_cutoff the point is put back on the
// circle of radius M_cutoff and iterated with c = 0), weighted by the
// Catmull-Rom polynomials of the fractional escape count
__global__ void __launch_bounds__(256) k_fieldlines(FieldlinesDev A) {
    const double M_cutoff = 100000.;
    double ang[FSG_FIELDLINES_MAX_ITER + 3];
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < A.npix;
         j += (long long)gridDim.x * blockDim.x) {
        double2 c = A.c[j];
        double2 z = A.z[j];
        ang[0] = atan2(z.y, z.x);
        for (int i = 0; i < A.n_iter + 2; i++) {
            if (hypot(z.x, z.y) > M_cutoff) {
                z = cx(cos(ang[i]) * M_cutoff, sin(ang[i]) * M_cutoff);
                z = fl_map(A.model, z, cx(0., 0.));
            } else {
                z = fl_map(A.model, z, c);
            }
            ang[i + 1] = atan2(z.y, z.x);
        }
        double d = -A.nu_frac[j];
        // a backshift beyond the escape count: constant weights
        if (A.is_backward && A.backshift > A.n[j]) d = 1.;
        const double a0 = cm_h0(d), a1 = cm_h1(d), a2 = cm_h2(d), a3 = cm_h3(d);
        double val = 0.;
        for (int i = 0; i < A.n_iter; i++) {
            const double ph = A.phi[i];
            val += A.k[i] * (a0 * sin(ang[i] + ph) + a1 * sin(ang[i + 1] + ph)
                             + a2 * sin(ang[i + 2] + ph) + a3 * sin(ang[i + 3] + ph));
        }
        A.out[j] = val;
    }
}

namespace {
// numpy's complex division (Smith's algorithm, npy_math_complex)
__device__ __forceinline__ double2 cdiv_np(double2 a, double2 b) {
    const double abs_br = fabs(b.x), abs_bi = fabs(b.y);
    if (abs_br >= abs_bi) {
        if (abs_br == 0. && abs_bi == 0.) return cx(a.x / abs_br, a.y / abs_bi);
        const double rat = b.y / b.x, scl = 1.0 / (b.x + b.y * rat);
        return cx((a.x + a.y * rat) * scl, (a.y - a.x * rat) * scl);
    }
    const double rat = b.x / b.y, scl = 1.0 / (b.y + b.x * rat);
    return cx((a.x * rat + a.y) * scl, (a.y * rat - a.x) * scl);
}
__device__ __forceinline__ double2 conj_(double2 a) { return cx(a.x, -a.y); }
}  // namespace

// DEM_normal_pp: kind 0 "potential" (z / dzndc), 1 "Milnor"
// (z dzndc ((1 + log|z|) conj(dzndc^2) - log|z| conj(z d2zndc2))),
// 2 "potential" of the Burning Ship family (J^T z); optional unskew, unit
// length
__global__ void __launch_bounds__(256) k_normal(NormalDev A) {
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < A.npix;
         j += (long long)gridDim.x * blockDim.x) {
        const double2 zn = A.zn[j];
        double2 nv;
        if (A.kind == 0) {
            nv = cdiv_np(zn, A.dzndc[j]);
        } else if (A.kind == 1) {
            const double2 dc = A.dzndc[j], d2 = A.d2[j];
            const double lo = log(hypot(zn.x, zn.y));
            const double2 t1 = rmul(1. + lo, conj_(csq(dc)));
            const double2 t2 = rmul(lo, conj_(cmul(zn, d2)));
            nv = cmul(cmul(zn, dc), cx(t1.x - t2.x, t1.y - t2.y));
        } else {
            const long long np = A.npix;
            const double dXdA = A.jac[j], dXdB = A.jac[np + j];
            const double dYdA = A.jac[2 * np + j], dYdB = A.jac[3 * np + j];
            nv = cx(dXdA * zn.x + dYdA * zn.y, dXdB * zn.x + dYdB * zn.y);
        }
        if (A.has_skew) {
            // product by the transposed skew matrix (contravariant)
            const double x = nv.x, y = nv.y;
            nv = cx(A.skew[0] * x + A.skew[2] * y, A.skew[1] * x + A.skew[3] * y);
        }
        const double r = hypot(nv.x, nv.y);
        A.out[j] = cx(nv.x / r, nv.y / r);
    }
}

static int pp_grid(long long n) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long need = (n + 255) / 256;
    long long g = (long long)sms * 8;
    return (int)(need < g ? (need > 0 ? need : 1) : g);
}

void fsg_launch_fieldlines(const FieldlinesDev &A, cudaStream_t s) {
    k_fieldlines<<<pp_grid(A.npix), 256, 0, s>>>(A);
}

void fsg_launch_normal(const NormalDev &A, cudaStream_t s) {
    k_normal<<<pp_grid(A.npix), 256, 0, s>>>(A);
}
