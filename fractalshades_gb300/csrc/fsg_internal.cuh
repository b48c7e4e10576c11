// fsg_internal.cuh -- device-side descriptors shared by the kernel translation
// units and the C-ABI layer.  Everything here lives in device memory.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "fsg_num.cuh"
#include "fsg_mn.cuh"

#define FSG_MAX_TILES_PER_LAUNCH 1024
#define FSG_STG_COMPRESSED 3          // settings.py:40 BLA_compression
#define FSG_CANCEL_POLL 65536         // steps between two reads of the cancel flag

// Reference orbit + derived tables (perturbation.py:317-375, 431-562)
struct RefDev {
    int len, div_iter, order, first_invalid;   // order clamped to INT32_MAX when none
    int flavor;                                 // 0 = M2, 1..5 BS
    int nexp;                                   // 0: power-2 closures; n: power-n model
    double binom[FSG_MN_MAX_EXP + 1];           // C(nexp, k) as float64
    int n_xr;
    const double2 *Zn;          // [len + 1], Zn[len] = 0 (read when w reaches len)
    const int *xr_slot;         // [len + 1]: -1 or index in the side table
    const double2 *xr_m;        // [n_xr] Xrange mantissas (M2: complex; BS: as doubles,
                                // [n_xr] x then [n_xr] y)
    const int *xr_e;            // [n_xr] (M2) or [2 n_xr] x then y (BS) exponents
    // derivative paths, standard form
    const double2 *dZndc;       // [len + 1]
    const double2 *dZndz;       // [len + 2] (slot len = wrapped value)
    // derivative paths, Xrange form
    const double2 *dZndc_xm; const int *dZndc_xe;
    const double2 *dZndz_xm; const int *dZndz_xe;
    // BS Jacobian paths
    const double *dXa, *dXb, *dYa, *dYb;        // [len + 1]
    const double *bs_xpm; const int *bs_xpe;    // Xrange branch: [4][len + 1] dXa, dXb, dYa,
                                                // dYb as float64 Xrange records
    // BLA tree (compressed, perturbation.py:1819-1881)
    const double2 *Mbla;        // M2: [bla_len][2] (A, B)
    const double *Mbla_bs;      // BS: [bla_len][8]
    const double *rbla;         // [bla_len]
    int stages, bla_len;
    // FE32 tables: int4 {x bits, y bits, exponent, aux}
    const int4 *Zf;             // [len + 1]; aux = exponent of max(|x|,|y|) or FE_ZERO_E
    const int4 *Zp;             // [len + 1] plain floats {2 Z.x bits, 2 Z.y bits,
                                // (exponent of max(|Z.x|,|Z.y|)) - 26 or FE_ZERO_E
                                // outside [2^-100, 2^100], 1 if Z is exactly 0}
    const int4 *dZndc_f;        // [len + 1]
    const int4 *dZndz_f;        // [len + 2]
    const int4 *bla_f;          // [2 bla_len] per entry i: [2i] = {r mantissa bits
                                // (rounded down with a 2^-20 margin), r exponent,
                                // A exponent, B exponent},
                                // [2i + 1] = {A.x, A.y, B.x, B.y} float bits
    const int4 *bla_first;      // [2 bla_nit] per start index it = w / 8, the first
                                // stage ref_BLA_get tries there: its bla_f record
    const int *bla_first_step;  // [bla_nit] that stage's step, 0 when none is tried
    const int4 *bla_chain;      // [2 bla_nit] per start index, the composite of the run of
                                // first candidates from there (header and payload as bla_f)
    const int2 *bla_chain_step; // [bla_nit] {iterations of that run, its BLA steps}, {0, 0}
                                // when none is stored
    int bla_nit;                // (len >> 3) + 1
    const int4 *fe_runs;        // [5 (len + 1)] per position w, the composed map of the
                                // fast steps from w to the next multiple of 8 (fsg_ref.cu,
                                // k_fe_runs): {P.x, P.y, P exponent, Q exponent},
                                // {Q.x, Q.y, R.x, R.y}, {R exponent, S exponent, S.x, S.y},
                                // {a mantissa, a exponent, b mantissa, b exponent},
                                // {max |2 Z|^2 bits, steps or 0 when not composable, 0, 0}
    // Burning Ship FP32+exp tables: reals as {mantissa bits, exponent} pairs
    const int4 *bs_Zf;          // [len + 1] {X, Y} (Xrange side-table values where present)
    const int4 *bs_hf;          // [2 (len + 1)] {dXa, dXb}, {dYa, dYb}
    const int4 *bs_blaf;        // [4 bla_len] the 8 BLA coefficients, two per int4
    const int2 *bs_rf;          // [bla_len] the BLA radii {mantissa bits, exponent}
    const float4 *bs_fa;        // [len + 1] frame step: {X, Y, exponent of X, of Y}
    const int4 *bs_fz;          // [len + 1] frame step: {flags, Hessian exponent g,
                                // no-rebase bound Tw, exponent of max(|X|, |Y|)}
    const float4 *bs_fh;        // [len + 1] frame step: {dXa, dXb, dYa, dYb} * 2^-g
};

struct TileDev {
    const RefDev *ref;
    const double *xs, *ys;
    const double2 *pix;                        // optional explicit positions
    int nx, ny;
    double lin[4];
    double cre, cim, dx;                       // standard loop
    double dx_m; int dx_e;                     // perturbation
    double drift_re, drift_im; int drift_e;
    double drifty_m; int drifty_e;
    void *Z; int nZ, i_dzndz, i_dzndc;
    int *U; signed char *stop_reason; int *stop_iter;
    double *pot, *dem;
    int dzs;                                   // dzndc scale 2^dzs over the reference's
    int i_orb;                                 // Z row of the orbit point
    int proj;                                  // 0 Cartesian, 1 Expmap
    double ph, pht_re, pht_im;                 // Expmap: exp(ph + pht * pix)
};

// The Burning Ship map of flavor 1..5 (burning_ship.py:82-123 BS_iterate,
// x ** 2 as x * x): the orbit replay of calc_orbit
__device__ __forceinline__ void bs_map(int flavor, double X, double Y, double a, double b,
                                       double &nX, double &nY) {
    if (flavor == 1) { nX = X * X - Y * Y + a; nY = 2. * fabs(X * Y) - b; }
    else if (flavor == 2) { nX = X * X - Y * Y + a; nY = 2. * X * fabs(Y) - b; }
    else if (flavor == 3) { nX = X * X - Y * fabs(Y) + a; nY = 2. * X * Y - b; }
    else if (flavor == 4) { nX = fabs(X * X - Y * Y) + a; nY = 2. * X * Y - b; }
    else { nX = fabs(X * X - Y * Y) + a; nY = 2. * fabs(X * Y) - b; }
}

// Orbit snapshots of calc_orbit (core.py:2965-3004, perturbation.py:1096-1101,
// 1265-1273): when n // backshift grows, the last two snapshots shift; at
// exit the older one is iterated forward to n - backshift.  "n // backshift
// grew" is tested as n >= next (no division per step).
template <class V>
struct OrbitSnap {
    int next, i1, i2;
    V z1, z2;
    __device__ __forceinline__ void init(int backshift, V z0) {
        next = backshift; i1 = 0; i2 = 0; z1 = z0; z2 = z0;
    }
    __device__ __forceinline__ void take(int n, int backshift, V z) {
        if (n >= next) {
            next = (n / backshift + 1) * backshift;
            i2 = i1; z2 = z1; i1 = n; z1 = z;
        }
    }
};

struct CalcDev {
    int max_iter;
    double M2, eps2, logM;
    int mode, calc_dzndc, interior, bla, flavor, xrsem;
    int nexp;                                  // 0: power-2 model; n: power-n model
    double logd;                               // log of the degree (potential)
    int backshift;                             // > 0: orbit point n - backshift
    int d2;                                    // standard loop: d2zndc2 in row 3
};

// Work distribution of one launch: a device counter hands out pixel indices
// of the concatenated tiles.
struct WorkDev {
    const TileDev *tiles;
    const long long *start;          // [ntiles + 1] prefix sums of pixel counts
    int ntiles;
    long long base;                  // claims [base, total): the pixels of the concatenated
    long long total;                 // tiles (one launch, or one segment of a streamed call),
    const unsigned *order;           // or, with order, the pixels order[base .. total)
    unsigned long long *counter;
    unsigned long long *stats;       // [4]: pixel_iters, full_steps, bla_steps, rebases
    volatile int *cancel;            // mapped host flag
    int *status;                     // device status word (1 = interrupted, 2 = budget)
    unsigned long long budget;       // iteration budget of the launch (0: none)
    unsigned long long *used;        // iterations of the pixels finished so far
};

// Claim the next pixel: returns false when the work is exhausted, or when
// the pixels finished so far have used the launch's iteration budget (the
// status word then reads 2; pixels already claimed run to their end, the
// others are left as they were for the caller to submit again).
__device__ __forceinline__ bool fsg_claim(const WorkDev &W, const long long *s_start,
                                          int &t, long long &ip) {
    if (W.budget && *(volatile unsigned long long *)W.used >= W.budget) {
        *W.status = 2;
        return false;
    }
    long long g = W.base + (long long)atomicAdd(W.counter, 1ULL);
    if (g >= W.total) return false;
    if (W.order) g = (long long)W.order[g];
    int lo = 0, hi = W.ntiles - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (s_start[mid] <= (long long)g) lo = mid; else hi = mid - 1;
    }
    t = lo;
    ip = g - s_start[lo];
    return true;
}

// a finished pixel's iterations, counted against the launch's budget
__device__ __forceinline__ void fsg_account(const WorkDev &W, unsigned long long n) {
    if (W.budget) atomicAdd(W.used, n);
}

// the host's interruption flag: sets the launch status and stops claiming
__device__ __forceinline__ bool fsg_cancelled(const WorkDev &W) {
    if (*W.cancel) { *W.status = 1; return true; }
    return false;
}

// shared memory of a kernel's tile offsets, sized at launch (dynamic)
inline size_t fsg_starts_smem(const WorkDev &W) { return sizeof(long long) * (W.ntiles + 1); }

__device__ __forceinline__ void fsg_load_starts(const WorkDev &W, long long *s_start) {
    for (int i = threadIdx.x; i <= W.ntiles; i += blockDim.x) s_start[i] = W.start[i];
    __syncthreads();
}

// Warp-reduced statistics (one atomic per warp per counter)
__device__ __forceinline__ void fsg_flush_stats(const WorkDev &W, unsigned long long a,
                                                unsigned long long b, unsigned long long c,
                                                unsigned long long d) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
        d += __shfl_down_sync(0xffffffffu, d, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&W.stats[0], a); atomicAdd(&W.stats[1], b);
        atomicAdd(&W.stats[2], c); atomicAdd(&W.stats[3], d);
    }
}

// Screen position of pixel ip of a tile
__device__ __forceinline__ double2 fsg_pixel_raw(const TileDev &T, long long ip) {
    if (T.pix) return __ldg(&T.pix[ip]);
    int ix = (int)(ip % T.nx), iy = (int)(ip / T.nx);
    return make_double2(__ldg(&T.xs[ix]), __ldg(&T.ys[iy]));
}

// Re(pht * pix): the h coordinate of an Expmap pixel (projection.py:306-314)
__device__ __forceinline__ double fsg_proj_h(const TileDev &T, double2 p) {
    return T.pht_re * p.x - T.pht_im * p.y;
}

// Expmap.f (projection.py:363-373): exp(h_moy + ht * pix).  Not inlined:
// its transcendental functions stay out of the iteration kernels' register
// allocation (called once per pixel)
static __device__ __noinline__ double2 fsg_expmap(double ph, double hr, double hi, double2 p) {
    const double zr = ph + (hr * p.x - hi * p.y);
    const double zi = hr * p.y + hi * p.x;
    const double e = exp(zr);
    return make_double2(e * cos(zi), e * sin(zi));
}
static __device__ __noinline__ double fsg_exp_nl(double x) { return exp(x); }

// The projected screen position (Cartesian: pix)
__device__ __forceinline__ double2 fsg_pixel(const TileDev &T, long long ip) {
    double2 p = fsg_pixel_raw(T, ip);
    if (T.proj == 0) return p;
    return fsg_expmap(T.ph, T.pht_re, T.pht_im, p);
}

// Expmap's derivative modifier of the perturbation loops
// (projection.py:455-473): exp(Re(ht * pix) + h_moy)
__device__ __forceinline__ double fsg_dzndc_modifier(const TileDev &T, long long ip) {
    return fsg_exp_nl(fsg_proj_h(T, fsg_pixel_raw(T, ip)) + T.ph);
}

// Potential (postproc.py:352-406 with Continuous_iter_pp_infinity :1001-1009,
// d = the degree, a_d = 1) and distance estimate (postproc.py:684-731).
__device__ __forceinline__ void fsg_epilogue(const TileDev &T, const CalcDev &C, long long ip,
                                             double2 zn, double absd, int n) {
    if (T.pot == nullptr && T.dem == nullptr) return;
    double az = hypot(zn.x, zn.y);
    if (T.pot) {
        double nu_frac = -(log(log(az) / C.logM) / C.logd);
        double x = -nu_frac;
        double q = floor(x);
        T.pot[ip] = ((double)n - q) - (x - q);
    }
    if (T.dem) {
        // |get_dzndc| = |dzndc| |df| with Expmap's |df| = exp(Re(ht * pix))
        if (T.proj) absd *= fsg_exp_nl(fsg_proj_h(T, fsg_pixel_raw(T, ip)));
        T.dem[ip] = az * log(az) / absd;
    }
}


// Persistent grid for a kernel: every SM filled to its occupancy limit,
// capped by the number of blocks the work needs.  grid > 0 is kept as given.
template <class K>
inline int fsg_auto_grid(K kernel, int grid, int block, long long total, size_t smem = 0) {
    // grid > 0: as given; 0: one wave at the occupancy limit; -k: at most k
    // CTAs per SM
    if (grid > 0) return grid;
    int dev = 0, sms = 1, per = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, smem) != cudaSuccess
        || per < 1)
        per = 1;
    if (grid < 0 && -grid < per) per = -grid;
    long long need = (total + block - 1) / block;
    long long g = (long long)sms * per;
    if (need < g) g = need > 0 ? need : 1;
    return (int)g;
}

#ifndef FSG_FIELDLINES_MAX_ITER
#define FSG_FIELDLINES_MAX_ITER 64
#endif
// Post-processing arguments (fsg_postproc.cu), device pointers
struct FieldlinesDev {
    long long npix;
    int model, is_backward, backshift, n_iter;
    const double2 *c, *z;
    const double *nu_frac;
    const int *n;
    const double *k, *phi;
    double *out;
};
struct NormalDev {
    long long npix;
    int kind, has_skew;
    double skew[4];
    const double2 *zn, *dzndc, *d2;
    const double *jac;          // Burning Ship: [4][npix] dxnda, dxndb, dynda, dyndb
    double2 *out;
};
void fsg_launch_fieldlines(const FieldlinesDev &A, cudaStream_t s);
void fsg_launch_normal(const NormalDev &A, cudaStream_t s);

// Kernel launchers (one per translation unit); grid 0 = one persistent wave
// at full occupancy
void fsg_launch_std(const WorkDev &W, const CalcDev &C, int grid, int block, cudaStream_t s);
void fsg_launch_perturb(const WorkDev &W, const CalcDev &C, int grid, int block, cudaStream_t s);
void fsg_launch_perturb_bs_fe32(const WorkDev &W, const CalcDev &C, int grid, int block,
                                cudaStream_t s);
void fsg_launch_perturb_fe32(const WorkDev &W, const CalcDev &C, int grid, int block,
                             cudaStream_t s);
// Reference tables
struct RefHost;   // defined in fsg_ref.cu
