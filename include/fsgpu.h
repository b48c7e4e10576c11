/*
 * fsgpu.h -- C-ABI of the GB300 escape-time / perturbation kernels.
 *
 * Drop-in boundary for Fractalshades' per-pixel iteration hot path.  Each entry
 * point replaces one reference interface (paths relative to src/fractalshades/):
 *
 *   fsg_std_tiles      <- Fractal.numba_cycle_call -> numba_cycles
 *                         (core.py:2022-2027, 2935-3056) for the standard
 *                         Mandelbrot / Burning Ship loops
 *   fsg_ref_create     <- PerturbationFractal.get_cycle_indep_args
 *                         (perturbation.py:431-562): uploads the reference
 *                         orbit and builds on the GPU the derivative paths
 *                         (numba_dZndc_path :2282, numba_dZndz_path :2466,
 *                         numba_dZndc_path_BS :2339) and the BLA tree
 *                         (numba_make_BLA :1819, numba_make_BLA_BS :1884)
 *   fsg_perturb_tiles  <- PerturbationFractal.numba_cycle_call ->
 *                         numba_cycles_perturb(_BS) (perturbation.py:414-428,
 *                         988-1811), plus the potential / distance estimate of
 *                         postproc.py:352-406, 684-731, 1001-1009 fused in the
 *                         kernel epilogue
 *   fsg_cancel         <- Fractal.raise_interruption (core.py:2011) polled by
 *                         the kernels like _interrupted (perturbation.py:1042)
 *
 * Conventions: plain pointers and sizes only; complex arrays are interleaved
 * (re, im) doubles (numpy complex128); Z is laid out [nZ][npix], pixels of a
 * tile in row-major order with x fastest (the ravel of the reference's
 * meshgrid, core.py:1820).  Every function returns FSG_OK or an error code and
 * never throws; fsg_last_error() gives the message.
 */
#ifndef FSGPU_H
#define FSGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSG_OK 0
#define FSG_INTERRUPTED 1      /* USER_INTERRUPTED (perturbation.py:984)      */
#define FSG_BUDGET 2           /* the launch's fsg_calc.iter_budget was used   */
#define FSG_ERR_ARG (-1)
#define FSG_ERR_CUDA (-2)
#define FSG_ERR_NOMEM (-3)
#define FSG_ERR_NODEV (-4)
#define FSG_ERR_LIMIT (-5)     /* a size beyond a stated maximum              */

/* delta arithmetic of the perturbation kernels */
#define FSG_MODE_FP64 0  /* double deltas: the reference with xr_detect_activated False   */
#define FSG_MODE_XR64 1  /* Xrange deltas, double mantissa + int32 exponent: the reference
                            with xr_detect_activated True (dx < settings.xrange_zoom_level) */
#define FSG_MODE_FE32 2  /* float mantissa + int32 exponent deltas (fast form)           */

#define FSG_MN_MAX_EXP 32  /* largest exponent of the power-n model                      */
#define FSG_MAX_ITER_LIMIT 0x3fffffff  /* largest max_iter, 2^30 - 1: n + a BLA step stays
                                        * inside int32 */

/* where the tile buffers live */
#define FSG_HOST 0       /* host pointers: page-locked arrays read and written in
                            place, pageable ones staged by the library            */
#define FSG_DEVICE 1     /* device pointers: asynchronous on the context stream     */

typedef struct fsg_ctx fsg_ctx;
typedef struct fsg_ref fsg_ref;

/* Reference orbit and the tables derived from it (perturbation.py:317-375,
 * 431-562).  All pointers are host pointers. */
typedef struct {
    const double *Zn;         /* complex128 [len]: FP64 orbit, Zn[0] = 0        */
    int64_t len;              /* ref_orbit_len                                   */
    int64_t div_iter;         /* ref_div_iter (first invalid iteration)          */
    int64_t order;            /* ref_order (cycle length), <= 0 when none        */
    int32_t n_xr;             /* sparse Xrange side table (ref_index_xr, ref_xr) */
    const int32_t *xr_idx;    /* [n_xr], increasing                              */
    const double *xr_m;       /* M2: complex128 mantissas [n_xr]; BS: [n_xr] x
                                 then [n_xr] y float64 mantissas                 */
    const int32_t *xr_e;      /* M2: [n_xr]; BS: [2 * n_xr] (x then y)           */
    int32_t flavor;           /* 0 = power-2 Mandelbrot, 1..5 Burning Ship       */
    int32_t xr_paths;         /* derivative paths in Xrange form                 */
    int32_t calc_dzndc;       /* build dZndc (M2) / the Jacobian paths (BS)      */
    int32_t calc_dzndz;       /* build dZndz (M2, interior detection)            */
    double scale_m;           /* dx * projection.scale as a float64 Xrange       */
    int32_t scale_e;
    int32_t bla;              /* build the BLA tree (empty below 8 orbit points,
                                 where no BLA step is valid: a calculation with
                                 bla on then takes full steps only, as the
                                 reference's ref_BLA_get does)                */
    double kc;                /* to_standard(kc) (perturbation.py:1830)          */
    double bla_eps;
    int32_t nexp;             /* flavor 0 only: 0 = the power-2 model
                                 (models/mandelbrot_M2.py), n in 2 ..
                                 FSG_MN_MAX_EXP = the power-n model
                                 (models/mandelbrot_Mn.py, exponent n): the
                                 paths and BLA use df/dz = n z^(n-1)         */
} fsg_ref_desc;

/* Calculation options (the calc_std_div keyword arguments). */
typedef struct {
    int64_t max_iter;
    double M_divergence;
    double epsilon_stationnary;
    int32_t mode;             /* FSG_MODE_*                                      */
    int32_t calc_dzndc;       /* M2: dzndc; BS: calc_hessian                     */
    int32_t interior;         /* M2 interior_detect (dzndz)                      */
    int32_t bla;              /* BLA_activated: every tile's reference must have
                                 been created with fsg_ref_desc.bla            */
    int32_t flavor;           /* 0 = M2, 1..5 Burning Ship                       */
    int32_t xr_semantics;     /* FE32 only: follow the Xrange branch's rebase
                                 confirmation (reference xr_detect_activated)    */
    int32_t nexp;             /* flavor 0 only: 0 = power-2 model, n in 2 ..
                                 FSG_MN_MAX_EXP = power-n model (standard loop
                                 of models/mandelbrot_Mn.py:317-355, perturbation
                                 closures :626-733, potential with d = n); a
                                 perturbation tile's reference must have been
                                 created with the same nexp.  FP64 and XR64
                                 only (FSG_MODE_FE32 is the power-2 form)     */
    int32_t backshift;        /* > 0: calc_orbit -- store the orbit point at
                                 iteration stop_iter - backshift in the tile's
                                 row i_znorbit (core.py:2965-3056,
                                 perturbation.py:1096-1101, 1265-1273,
                                 1389-1396, 1641-1651, 1778-1787); 0: off.
                                 Standard loops and FP64 / XR64 perturbation  */
    int32_t calc_d2zndc2;     /* standard power-2 / power-n loops: the second
                                 derivative d2zndc2 in Z row 3
                                 (mandelbrot_M2.py:316-317,
                                 mandelbrot_Mn.py:325-333)                    */
    int32_t block;            /* launch shape (chosen by the autotuner,
                                 fractalshades_gb300/tune.py): threads per
                                 CTA, 0 = the kernel's default (256; 128 for
                                 the FE32 power-2 kernel), else a multiple of
                                 32 up to that default                        */
    int32_t ctas_per_sm;      /* resident CTAs per SM of the persistent grid,
                                 0 = the occupancy limit, else at most that
                                 many (the allocation-free entry point keeps
                                 its fixed shape)                             */
    int64_t iter_budget;      /* 0: none.  Else the launch stops claiming pixels
                                 once the pixels it finished have used this many
                                 iterations: pixels already claimed run to their
                                 end, the others keep their stop_reason (-1 for
                                 the reference's fresh arrays, core.py:2070-2073;
                                 host-buffer calls copy -1 back for them), and the
                                 call returns FSG_BUDGET -- submit those pixels
                                 again to finish.  No counterpart in the
                                 reference (it runs a tile to its end)         */
    int32_t claim_order;      /* FSG_ORDER_PIXELS (0): pixels claimed in order;
                                 FSG_ORDER_LONGEST (1): a perturbation launch of
                                 2^18 pixels or more claims them longest first
                                 (see fsg_perturb_tiles).  Outputs are the same;
                                 longest first shortens the tail of views whose
                                 iteration counts spread over decades (a view
                                 straddling a minibrot's boundary: -10 %) and
                                 costs its pre-pass on uniform ones (+1.5 % on
                                 an all-interior one)                          */
} fsg_calc;

#define FSG_ORDER_PIXELS 0
#define FSG_ORDER_LONGEST 1

/* One tile: a rectangle of pixels with its own view and outputs. */
typedef struct {
    int32_t nx, ny;
    const double *xs;         /* [nx] screen fraction per column                 */
    const double *ys;         /* [ny] screen fraction per row (already negated and
                                 divided by xy_ratio, core.py:1820-1830)          */
    const double *pix;        /* optional complex128 [nx * ny] explicit pixel
                                 positions (the reference's c_pix, e.g. a subset
                                 or a jittered grid); when set, xs / ys are
                                 ignored and may be NULL                          */
    double lin_mat[4];        /* rotation / skew (core.py:1470-1484), row-major   */
    /* standard loop: c = center + dx * lin_mat . pix */
    double center_re, center_im, dx;
    /* perturbation: dc = dx_xr * lin_mat . pix + drift_xr */
    double dx_m; int32_t dx_e;
    double drift_re, drift_im; int32_t drift_e;   /* M2 complex drift; BS: driftx in
                                                     drift_re with drift_e      */
    double drifty_m; int32_t drifty_e;            /* BS: drifty                 */
    fsg_ref *ref;
    /* outputs, [nZ][nx*ny] etc.; potential / dem may be NULL */
    void *Z; int32_t nZ; int32_t i_dzndz; int32_t i_dzndc;
    int32_t *U; int8_t *stop_reason; int32_t *stop_iter;
    double *potential; double *dem;
    /* perturbation: the tile's derivative unit (M2 dzndc, BS Hessian) is
       the reference's derivative scale times 2^dzndc_scale_e (the
       derivative recurrences are linear in their scale, so one reference
       serves views of every width, and a reference of unit scale serves
       widths below the double range: the derivative outputs and DEM are
       scaled exactly); 0 for the reference's own scale.  Must be 0 for the
       standard loop.  No counterpart in the reference (one scale per
       reference, perturbation.py:461-468). */
    int32_t dzndc_scale_e;
    /* with fsg_calc.backshift > 0: the Z row of the orbit point (complex
       zn_orbit; Burning Ship: xn_orbit, then yn_orbit in the next row) */
    int32_t i_znorbit;
    /* projection of the screen position before lin_mat (projection.py):
       0 Cartesian (identity); 1 Expmap, pix -> exp(proj_h + proj_ht * pix)
       with proj_ht = proj_ht_re + i proj_ht_im (:363-373).  With Expmap the
       perturbation loops multiply the derivatives at exit by
       exp(Re(proj_ht * pix) + proj_h) (:455-473, perturbation.py:1387-1388,
       1772-1776) and the fused distance estimate divides by
       |df| = exp(Re(proj_ht * pix)) (postproc.py:184-205) */
    int32_t proj;
    double proj_h, proj_ht_re, proj_ht_im;
} fsg_tile;

/* Post-processing on the device (postproc.py).  Pointers are host or device
 * arrays as `where` says (FSG_HOST: the library stages the copies and
 * returns once the output is back in host memory). */
#define FSG_FIELDLINES_MAX_ITER 64

/* Fieldlines_pp (postproc.py:409-530, 1038-1160): the orbit-averaged angle
 * of n_iter + 3 orbit points from the stored start point, smoothed by the
 * Catmull-Rom weights of the fractional escape count. */
typedef struct {
    int64_t npix;
    int32_t model;            /* 0: z^2 + c; n >= 2: z^n + c; -1 .. -5: Burning
                                 Ship flavor 1 .. 5                              */
    const double *c;          /* complex128 [npix]: the pixel's c (get_std_cpt) */
    const double *z;          /* complex128 [npix]: zn_orbit (or zn); Burning
                                 Ship: (xn_orbit, yn_orbit) pairs               */
    const double *nu_frac;    /* float64 [npix]: Continuous_iter_pp's nu_frac   */
    const int32_t *n;         /* int32 [npix]: Continuous_iter_pp's n           */
    int32_t is_backward;      /* z is the orbit point n - backshift             */
    int32_t backshift;
    int32_t n_iter;           /* 1 .. FSG_FIELDLINES_MAX_ITER                   */
    const double *k;          /* float64 [n_iter]: weights                      */
    const double *phi;        /* float64 [n_iter]: phases                       */
    double *out;              /* float64 [npix]                                 */
} fsg_fieldlines;

/* DEM_normal_pp (postproc.py:533-628): the unit normal of the distance
 * estimate. */
typedef struct {
    int64_t npix;
    int32_t kind;             /* 0: "potential", zn / dzndc; 1: "Milnor";
                                 2: "potential" of the Burning Ship family     */
    const double *zn;         /* complex128 [npix] (Burning Ship: (xn, yn))     */
    const double *dzndc;      /* complex128 [npix]; Burning Ship: float64
                                 [4][npix] dxnda, dxndb, dynda, dyndb           */
    const double *d2zndc2;    /* complex128 [npix] (kind 1)                     */
    const double *skew;       /* NULL or float64 [2][2]: the view's skew, undone
                                 on the normal (core.py:3147-3158)              */
    double *out;              /* complex128 [npix]                              */
} fsg_normal;

int fsg_postproc_fieldlines(fsg_ctx *ctx, const fsg_fieldlines *args, int32_t where);
int fsg_postproc_normal(fsg_ctx *ctx, const fsg_normal *args, int32_t where);

/* Launch statistics of the last fsg_*_tiles call. */
typedef struct {
    double kernel_ms;          /* device time of the iteration kernel            */
    int64_t pixels;
    int64_t pixel_iters;       /* sum of stop_iter                               */
    int64_t full_steps;        /* executed perturbation / standard steps         */
    int64_t bla_steps;         /* executed BLA steps                             */
    int64_t rebases;
} fsg_stats;

const char *fsg_version(void);
int fsg_ctx_create(int device, fsg_ctx **out);
int fsg_ctx_destroy(fsg_ctx *ctx);
const char *fsg_last_error(const fsg_ctx *ctx);
/* Use an external CUDA stream (cudaStream_t as void*) instead of the
 * context's own; NULL restores the context's own stream (the legacy default
 * stream cannot be selected). */
int fsg_set_stream(fsg_ctx *ctx, void *stream);
int fsg_sync(fsg_ctx *ctx);

int fsg_ref_create(fsg_ctx *ctx, const fsg_ref_desc *desc, fsg_ref **out);
int fsg_ref_destroy(fsg_ctx *ctx, fsg_ref *ref);

/* A reference that shares the orbit, the Xrange side table, the derivative
   paths and their FP32 copies of `base` and owns a BLA tree of its own, built
   for kc / bla_eps: views of one centre at other widths need another kc (the
   BLA radii depend on it, nothing else does; the derivative scale is set per
   tile with fsg_tile.dzndc_scale_e).  FSG_ERR_ARG when base is itself derived;
   fsg_ref_destroy refuses a base while references derived from it live.
   Returns without waiting for the build: the BLA kernels run on ctx's stream
   and every later launch (on any context) or download that uses the derived
   reference waits for them on the device.
   No counterpart in the reference (one BLA tree per calculation,
   perturbation.py:1819-1881). */
int fsg_ref_derive_bla(fsg_ctx *ctx, fsg_ref *base, double kc, double bla_eps,
                       fsg_ref **out);
/* Copy tables back to the host (tests).  which: 0 dZndc (complex128 [len]) or
 * its Xrange form (mantissa complex128 [len] + exp int32 [len]), 1 dZndz
 * ([len + 1]), 2 BLA (M complex128 [bla_len][2], r float64 [bla_len]),
 * 3 BS Jacobian paths (4 x float64 [len]), 4 BS Jacobian paths as Xrange
 * records (out0 4 x float64 [len] mantissas, out1 4 x int32 [len] exponents;
 * references created with xr_paths).  Sizes via fsg_ref_info. */
int fsg_ref_info(const fsg_ref *ref, int64_t *len, int64_t *bla_len, int32_t *stages);
int fsg_ref_download(fsg_ctx *ctx, const fsg_ref *ref, int which, void *out0,
                     void *out1);

/* The iteration over the tiles (one launch of up to FSG_MAX_TILES_PER_LAUNCH
 * tiles).  With fsg_calc.claim_order = FSG_ORDER_LONGEST, a perturbation
 * launch of 2^18 pixels or more (without an iteration budget, buffers not
 * written in place) claims its pixels longest first: a pre-pass iterates one
 * pixel per 8 x 8 block with max_iter capped at max_iter / 8 (256 .. 4096),
 * then every pixel is claimed in decreasing order of its block's count;
 * outputs do not depend on the order.  With FSG_HOST buffers the call
 * returns once the outputs are in host memory:
 *   - page-locked buffers (cudaHostAlloc, cudaHostRegister; every array of
 *     every tile) are read and written in place by the kernels, as the
 *     reference's loop writes its arrays: fields a kernel does not produce,
 *     and pixels a budget leaves unrun, keep the caller's values;
 *   - pageable buffers are staged on the device: fields the kernels do not
 *     produce come back as zeros and unrun pixels with stop_reason -1; a
 *     perturbation call of at least 2^21 pixels runs as up to four launches
 *     over consecutive pixel ranges, each range's outputs copied back while
 *     the next computes (outputs identical to one launch).
 * Returns FSG_OK, FSG_BUDGET (fsg_calc.iter_budget reached), FSG_INTERRUPTED
 * (fsg_cancel: host buffers are left as they were when the cancel came before
 * the call; one that comes while the call runs may leave written the pixels,
 * or the staged ranges, finished before it -- the reference's loop writes its
 * arrays in place too, and discards an interrupted tile), or an error. */
int fsg_std_tiles(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles,
                  int32_t ntiles, int32_t where);
int fsg_perturb_tiles(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles,
                      int32_t ntiles, int32_t where);
int fsg_last_stats(const fsg_ctx *ctx, fsg_stats *out);

/* Measured FMA throughput of this GPU in TFLOP/s (fp64 = 0: FP32 pipe,
 * 1: FP64 pipe): the roofline denominator of the iteration kernels.  No
 * counterpart in the reference (a measurement helper). */
int fsg_peak_flops(fsg_ctx *ctx, int32_t fp64, double *tflops);

int fsg_cancel(fsg_ctx *ctx);
int fsg_clear_cancel(fsg_ctx *ctx);

/* Serving queue for interactive rendering.  No counterpart in the reference,
 * which renders one image at a time (its GUI runs one script,
 * gui/guimodel.py); the submit / poll pair is the asynchronous form of
 * fsg_std_tiles / fsg_perturb_tiles with host buffers, with the reference's
 * interruption contract (core.py:2545-2547).
 *   fsg_serve_open: `slots` launch streams of the context (each runs one
 *     request at a time, so up to `slots` requests overlap on the device) and
 *     an HBM budget for the requests' staged buffers (their inputs and
 *     outputs on the device: what fsg_perturb_tiles stages for host buffers);
 *   fsg_submit: queues a request of host-buffer tiles (at most
 *     FSG_MAX_TILES_PER_LAUNCH; all perturbation tiles, with references, or
 *     all standard tiles) and returns its ticket at once.  The caller keeps
 *     every buffer of the tiles, and the references, alive until fsg_poll
 *     reports the request finished.  A request is admitted when a slot is
 *     free and its staged bytes fit in what the budget has left (a request
 *     whose arrays are all page-locked stages nothing: the kernels read and
 *     write them in place, as fsg_perturb_tiles does); the next one
 *     in `order` waits for that (FSG_SERVE_FIFO: arrival order;
 *     FSG_SERVE_SHORTEST: smallest expected_work first, the caller's estimate,
 *     e.g. pixels x expected iterations; <= 0 means the pixel count;
 *     FSG_SERVE_HRRN: highest response ratio (wait + S) / S first, S =
 *     expected_work over the work rate of a slot measured on the finished
 *     requests -- short requests first, a long one once it has waited about
 *     its own service time; smallest expected_work first until a request
 *     has finished);
 *     FSG_ERR_LIMIT for a request larger than the whole budget;
 *   fsg_poll: FSG_PENDING while queued or running; once finished, the
 *     request's outcome (FSG_OK, FSG_BUDGET, FSG_INTERRUPTED with the
 *     caller's arrays untouched -- for staged requests; one written in place
 *     may hold the pixels finished before -- or an error code), its results in the
 *     caller's buffers, and the ticket released.  Polling also retires
 *     finished launches and admits queued requests: call it regularly;
 *   fsg_serve_close: waits for running requests, drops queued ones;
 *     fsg_ctx_destroy closes an open queue.
 * fsg_cancel interrupts running and later-admitted requests alike. */
#define FSG_SERVE_FIFO 0
#define FSG_SERVE_SHORTEST 1
#define FSG_SERVE_HRRN 2
#define FSG_PENDING 3          /* fsg_poll: the request is not finished yet    */
typedef struct {
    int64_t queued, running;
    int64_t reserved_bytes, peak_reserved_bytes, budget_bytes;
    int32_t slots;
} fsg_serve_stats;
int fsg_serve_open(fsg_ctx *ctx, int64_t hbm_budget_bytes, int32_t slots, int32_t order);
int fsg_submit(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
               double expected_work, int64_t *ticket);
int fsg_poll(fsg_ctx *ctx, int64_t ticket);
int fsg_serve_info(fsg_ctx *ctx, fsg_serve_stats *out);
int fsg_serve_close(fsg_ctx *ctx);

/* Allocation-free variant of fsg_std_tiles.  It has no counterpart in the
 * reference: it serves callers that cannot call cudaMalloc -- their device
 * memory is reserved up front by another allocator, or they cannot afford the
 * device synchronisation that cudaMalloc / cudaFree imply inside a frame loop.
 * It needs no context and allocates nothing: every pointer of every tile
 * (xs / ys or pix, Z, stop_reason, stop_iter, optional potential / dem) is a
 * device pointer, and the launch's work counter, statistics and tile
 * descriptors live in a file-scope __device__ array of the library, one per
 * device, held until the process exits.
 *   - at most FSG_NOALLOC_MAX_TILES tiles per call, else FSG_ERR_LIMIT;
 *   - asynchronous on `stream` (NULL: the legacy default stream); results are
 *     valid once the stream has completed;
 *   - every call shares the array (the counter and statistics are cleared at
 *     the start of each call): calls whose launches overlap on the GPU, from
 *     other streams or host threads, race on it;
 *   - the first call on a device resolves the array's address with that device
 *     current; make that first call before any stream capture;
 *   - the descriptors travel as the parameter of a small upload kernel on
 *     `stream`: the call makes no host-to-device copy and does not wait for
 *     the stream;
 *   - an error left pending by earlier CUDA work of the calling thread is
 *     consumed on entry (cudaGetLastError), so FSG_ERR_CUDA reports this
 *     call's own launches;
 *   - max_iter in 1 .. FSG_MAX_ITER_LIMIT, like fsg_std_tiles;
 *   - no iteration budget (fsg_calc.iter_budget must be 0, else FSG_ERR_ARG);
 *   - not cancellable (fsg_cancel does not apply). */
#define FSG_NOALLOC_MAX_TILES 64
int fsg_std_tiles_noalloc(const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
                          void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FSGPU_H */
