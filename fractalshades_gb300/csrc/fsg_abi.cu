// fsg_abi.cu -- the extern "C" boundary declared in include/fsgpu.h.
//
// Owns the CUDA context state (stream, work counter, statistics, cancel flag),
// the device copies of reference orbits with their derived tables, and the
// launch of the iteration kernels over batches of tiles.  No C++ exception
// crosses the boundary: every entry point returns a status code.
#include <climits>
#include <cstdio>
#include <cstring>
#include <map>
#include <algorithm>
#include <chrono>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "fsg_internal.cuh"
#include "../../include/fsgpu.h"

#define FSG_VERSION "fractalshades_gb300 0.1.0 (sm_103a)"

// launchers of fsg_ref.cu
void fsg_build_paths_m2(const RefDev *Rd, int len, double2 *dzndc, double2 *dzndc_xm, int *dzndc_xe,
                        double2 *dzndz, double2 *dzndz_xm, int *dzndz_xe, int div_iter, int xr_mode,
                        int want_dzndc, int want_dzndz, double scale_m, int scale_e,
                        cudaStream_t s);
void fsg_build_paths_bs(const RefDev *Rd, int len, double *dXa, double *dXb, double *dYa, double *dYb,
                        double scale, cudaStream_t s);
void fsg_build_paths_bs_xr(const RefDev *Rd, int len, double *pm, int *pe, double scale_m,
                           int scale_e, cudaStream_t s);
void fsg_build_bla(const RefDev *Rd, int flavor, int len, double2 *M2, double *Mbs, double *r,
                   int stages, double kc, double eps, cudaStream_t s);
void fsg_build_plain_orbit(const RefDev *Rd, int len, const int4 *Zf, int4 *Zp, cudaStream_t s);
void fsg_build_fe_runs(const RefDev *Rd, int len, const int4 *Zp, const int4 *Df, int4 *runs,
                       cudaStream_t s);
void fsg_build_fe_tables(const RefDev *Rd, int len, int4 *Zf, const double2 *dzndc,
                         const double2 *dzndc_xm, const int *dzndc_xe, int4 *dzndc_f,
                         const double2 *dzndz, const double2 *dzndz_xm, const int *dzndz_xe,
                         int4 *dzndz_f, const double2 *Mbla, const double *rbla, int bla_len,
                         int4 *bla_f, int bla_nit, int4 *bla_first, int *bla_first_step,
                         double kc, int4 *bla_chain, int2 *bla_chain_step,
                         cudaStream_t s);
void fsg_build_fe_bla(const RefDev *Rd, const double2 *Mbla, const double *rbla, int bla_len,
                      int4 *bla_f, int bla_nit, int4 *bla_first, int *bla_first_step,
                      double kc, int4 *bla_chain, int2 *bla_chain_step,
                      cudaStream_t s);
void fsg_build_bs_fr(const RefDev *Rd, int len, int4 *Zf, const double *dXa, const double *dXb,
                     const double *dYa, const double *dYb, int4 *hf, float4 *fa, int4 *fz,
                     float4 *fh, int div_iter, cudaStream_t s);
void fsg_build_bs_fr_bla(const double *Mbs, const double *rbla, int bla_len, int4 *blaf,
                         int2 *rf, cudaStream_t s);

double fsg_launch_fma_peak(int fp64, int sm_count, void *out, cudaStream_t s);

// launchers of fsg_lpt.cu (claim order, longest pixels first)
int fsg_lpt_blocks_count(const int *nx, const int *ny, int ntiles);
void fsg_lpt_prepare(const TileDev *tiles, const long long *start, int ntiles, int nblk,
                     int *blk_start, unsigned *hist, unsigned *rep, cudaStream_t s);
void fsg_lpt_order(const TileDev *tiles, const long long *start, int ntiles, int nblk,
                   const int *blk_start, unsigned *hist, const unsigned *rep,
                   unsigned char *bucket, unsigned *order, cudaStream_t s);

// Streamed copy-back of host-buffer calls (run_tiles): at most this many
// launch segments, each of at least this many pixels
#define FSG_COPY_SEGMENTS 4
#define FSG_COPY_SEGMENT_PIXELS (1LL << 20)
// Claim order longest pixels first (fsg_lpt.cu) for perturbation launches of
// at least this many pixels (and below 2^31: 32-bit pixel indices)
#define FSG_LPT_MIN_PIXELS (1LL << 18)

struct ServeState;   // the serving queue (fsg_serve_open), below

struct fsg_ctx {
    ServeState *serve = nullptr;
    int device = 0;
    int sm_count = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    volatile int *cancel_host = nullptr;   // pinned, mapped
    int *cancel_dev = nullptr;             // device alias of cancel_host
    int *status_dev = nullptr;
    unsigned long long *used_dev = nullptr;  // iterations counted against the budget
    unsigned long long *counter_dev = nullptr;
    unsigned long long *stats_dev = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_desc = nullptr;
    // streamed copy-back of host-buffer calls: a copy stream and one event
    // per launch segment
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_seg[FSG_COPY_SEGMENTS] = {};
    bool timed = false;
    int64_t last_pixels = 0;
    // tile descriptors: pinned staging + device copy
    TileDev *tiles_host = nullptr; long long *start_host = nullptr;
    TileDev *tiles_dev = nullptr; long long *start_dev = nullptr;
    // grow-only device scratch for host-buffer calls
    char *scratch = nullptr; size_t scratch_size = 0;
    // grow-only device scratch of the longest-first claim order
    char *lpt = nullptr; size_t lpt_size = 0;
};

struct fsg_ref {
    RefDev host;            // device pointers, host copy
    RefDev *dev = nullptr;  // device copy of the descriptor
    std::vector<void *> allocs;   // stream-ordered allocations (cudaMallocAsync)
    int64_t len = 0;
    int xr_paths = 0, flavor = 0, has_dzndc = 0, has_dzndz = 0;
    int nexp = 0;                 // 0: power-2 model, n: power-n model
    int bla_req = 0;              // built with a BLA tree (empty below 8 orbit points,
                                  // where no BLA step is ever valid)
    fsg_ref *base = nullptr;      // fsg_ref_derive_bla: owner of the shared tables
    int derived = 0;              // live references derived from this one
    cudaEvent_t ready = nullptr;  // derived references: recorded after the BLA build;
                                  // launches and downloads wait for it
};

namespace {

int set_err(fsg_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_err(fsg_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return FSG_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return set_err(c, e == cudaErrorMemoryAllocation ? FSG_ERR_NOMEM : FSG_ERR_CUDA, m);
}

#define CK(call, what)                                      \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_err(ctx, e_, what); \
    } while (0)

template <class T>
int ref_alloc(fsg_ctx *ctx, fsg_ref *r, T **p, size_t n) {
    void *q = nullptr;
    // stream-ordered: no device-wide synchronisation while other streams run
    cudaError_t e = cudaMallocAsync(&q, n * sizeof(T) + 16, ctx->stream);
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMalloc(reference table)");
    r->allocs.push_back(q);
    *p = (T *)q;
    return FSG_OK;
}

// threads per CTA of the kernel a calculation launches by default, and the
// largest its launch bounds allow
static int default_block(const fsg_calc *calc, int perturb) {
    return (perturb && calc->flavor == 0 && calc->nexp == 0 && calc->mode == FSG_MODE_FE32) ? 128
                                                                                             : 256;
}

void ref_release(fsg_ref *r, cudaStream_t s) {
    for (void *p : r->allocs) cudaFreeAsync(p, s);
    r->allocs.clear();
    if (r->dev) cudaFreeAsync(r->dev, s);
    r->dev = nullptr;
}

int ensure_scratch(fsg_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->scratch_size) return FSG_OK;
    if (ctx->scratch) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr; ctx->scratch_size = 0;
    }
    size_t sz = bytes + bytes / 4;
    CK(cudaMalloc((void **)&ctx->scratch, sz), "cudaMalloc(scratch)");
    ctx->scratch_size = sz;
    return FSG_OK;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

int check_tile(fsg_ctx *ctx, const fsg_tile &t, bool perturb, const fsg_calc *calc) {
    if (t.nx <= 0 || t.ny <= 0) return set_err(ctx, FSG_ERR_ARG, "tile with nx <= 0 or ny <= 0");
    if ((!t.pix && (!t.xs || !t.ys)) || !t.Z || !t.stop_reason || !t.stop_iter)
        return set_err(ctx, FSG_ERR_ARG, "tile with a NULL input or output pointer");
    if (perturb && !t.ref) return set_err(ctx, FSG_ERR_ARG, "perturbation tile without reference");
    if (perturb && t.ref->flavor != calc->flavor)
        return set_err(ctx, FSG_ERR_ARG, "reference flavor differs from the calculation flavor");
    if (perturb && t.ref->nexp != calc->nexp)
        return set_err(ctx, FSG_ERR_ARG, "reference exponent (nexp) differs from the calculation's");
    if (perturb && calc->flavor == 0) {
        if (calc->calc_dzndc && !t.ref->has_dzndc)
            return set_err(ctx, FSG_ERR_ARG, "calc_dzndc requested but the reference has no dZndc path");
        if (calc->interior && !t.ref->has_dzndz)
            return set_err(ctx, FSG_ERR_ARG, "interior detection requested but the reference has no dZndz path");
        if (calc->mode == FSG_MODE_XR64 && !t.ref->xr_paths && (calc->calc_dzndc || calc->interior))
            return set_err(ctx, FSG_ERR_ARG, "Xrange mode needs Xrange derivative paths");
        if (calc->mode == FSG_MODE_FP64 && t.ref->xr_paths && (calc->calc_dzndc || calc->interior))
            return set_err(ctx, FSG_ERR_ARG, "FP64 mode needs standard derivative paths");
        if (calc->bla && !t.ref->bla_req)
            return set_err(ctx, FSG_ERR_ARG, "BLA requested but the reference was built without it");
    }
    if (t.dzndc_scale_e != 0 && !perturb)
        return set_err(ctx, FSG_ERR_ARG, "dzndc_scale_e applies to the perturbation loops only");
    if (t.dzndc_scale_e < -100000 || t.dzndc_scale_e > 100000)
        return set_err(ctx, FSG_ERR_ARG, "dzndc_scale_e out of range");
    if (t.proj < 0 || t.proj > 1) return set_err(ctx, FSG_ERR_ARG, "bad projection kind");
    if (perturb && calc->flavor != 0) {
        if (calc->mode == FSG_MODE_XR64 && calc->calc_dzndc && !t.ref->xr_paths)
            return set_err(ctx, FSG_ERR_ARG, "Xrange mode needs Xrange Jacobian paths (fsg_ref_desc.xr_paths)");
        if (calc->calc_dzndc && !t.ref->has_dzndc)
            return set_err(ctx, FSG_ERR_ARG, "calc_hessian requested but the reference has no Jacobian paths");
        if (calc->bla && !t.ref->bla_req)
            return set_err(ctx, FSG_ERR_ARG, "BLA requested but the reference was built without it");
    }
    int nZ_min = perturb ? (calc->flavor == 0 ? 1 + (calc->interior ? 1 : 0) + (calc->calc_dzndc ? 1 : 0)
                                              : (calc->calc_dzndc ? 6 : 2))
                         : (calc->flavor == 0 ? 3 + (calc->calc_d2zndc2 ? 1 : 0) : 6);
    if (t.nZ < nZ_min) return set_err(ctx, FSG_ERR_ARG, "tile nZ too small for the requested fields");
    if (calc->backshift > 0) {
        // the orbit row(s) come after the fields above (complex zn_orbit, or
        // the real xn_orbit, yn_orbit pair of the Burning Ship family)
        const int rows = calc->flavor == 0 ? 1 : 2;
        if (t.i_znorbit < nZ_min || t.i_znorbit + rows > t.nZ)
            return set_err(ctx, FSG_ERR_ARG, "bad i_znorbit for calc_orbit");
    }
    if (perturb && calc->flavor == 0) {
        if (calc->interior && (t.i_dzndz <= 0 || t.i_dzndz >= t.nZ))
            return set_err(ctx, FSG_ERR_ARG, "bad i_dzndz");
        if (calc->calc_dzndc && (t.i_dzndc <= 0 || t.i_dzndc >= t.nZ))
            return set_err(ctx, FSG_ERR_ARG, "bad i_dzndc");
    }
    return FSG_OK;
}

int check_nexp(fsg_ctx *ctx, int flavor, int nexp) {
    if (nexp == 0) return FSG_OK;
    if (flavor != 0) return set_err(ctx, FSG_ERR_ARG, "nexp applies to flavor 0 (Mandelbrot) only");
    if (nexp < 2) return set_err(ctx, FSG_ERR_ARG, "nexp must be 0 or an exponent >= 2");
    if (nexp > FSG_MN_MAX_EXP) return set_err(ctx, FSG_ERR_LIMIT, "nexp above FSG_MN_MAX_EXP");
    return FSG_OK;
}

CalcDev make_calc(const fsg_calc *c) {
    CalcDev d;
    d.max_iter = (int)c->max_iter;
    d.M2 = c->M_divergence * c->M_divergence;
    d.eps2 = c->epsilon_stationnary * c->epsilon_stationnary;
    d.logM = log(c->M_divergence);
    d.mode = c->mode; d.calc_dzndc = c->calc_dzndc; d.interior = c->interior;
    d.bla = c->bla; d.flavor = c->flavor; d.xrsem = c->xr_semantics;
    d.nexp = c->nexp;
    d.logd = log(c->nexp ? (double)c->nexp : 2.);
    d.backshift = c->backshift;
    d.d2 = c->calc_d2zndc2;
    return d;
}

TileDev make_tile(const fsg_tile &t) {
    TileDev d;
    memset(&d, 0, sizeof(d));
    d.ref = t.ref ? t.ref->dev : nullptr;
    d.xs = t.xs; d.ys = t.ys; d.nx = t.nx; d.ny = t.ny;
    d.pix = (const double2 *)t.pix;
    for (int k = 0; k < 4; k++) d.lin[k] = t.lin_mat[k];
    d.cre = t.center_re; d.cim = t.center_im; d.dx = t.dx;
    d.dx_m = t.dx_m; d.dx_e = t.dx_e;
    d.drift_re = t.drift_re; d.drift_im = t.drift_im; d.drift_e = t.drift_e;
    d.drifty_m = t.drifty_m; d.drifty_e = t.drifty_e;
    d.Z = t.Z; d.nZ = t.nZ; d.i_dzndz = t.i_dzndz; d.i_dzndc = t.i_dzndc;
    d.U = t.U; d.stop_reason = (signed char *)t.stop_reason; d.stop_iter = t.stop_iter;
    d.pot = t.potential; d.dem = t.dem;
    d.dzs = t.dzndc_scale_e;
    d.i_orb = t.i_znorbit;
    d.proj = t.proj; d.ph = t.proj_h; d.pht_re = t.proj_ht_re; d.pht_im = t.proj_ht_im;
    return d;
}

// A launch over the pixels [base, end) of its tiles; `first` uploads the
// descriptors and resets the launch's statistics, status and budget, `last`
// closes its timing (a streamed call launches several segments in a row).
struct Segment {
    long long base, end;
    bool first, last;
    bool uploaded;             // the caller uploaded the descriptors already
    const unsigned *order;     // claim order (device), nullptr: pixel order
    bool keep_time;            // first: reset the statistics but not the timing
};

// The launch resources of one stream: the context's own, or a serving slot's
struct LaunchRes {
    cudaStream_t stream;
    TileDev *tiles_host; long long *start_host;        // pinned staging
    TileDev *tiles_dev; long long *start_dev;
    unsigned long long *counter_dev, *stats_dev, *used_dev;
    int *status_dev;
    cudaEvent_t ev_desc;       // staging reuse (nullptr: the caller orders it)
    cudaEvent_t ev0, ev1;      // kernel timing (nullptr: none)
};

long long tiles_pixels(const TileDev *tiles, int ntiles) {
    long long total = 0;
    for (int i = 0; i < ntiles; i++) total += (long long)tiles[i].nx * tiles[i].ny;
    return total;
}

// Launch the iteration kernel over the pixels [seg.base, seg.end) of ntiles
// device-resident tiles on L.stream.
// Upload the tile descriptors and their pixel offsets to L's device copies.
int upload_descriptors(fsg_ctx *ctx, const LaunchRes &L, const TileDev *tiles, int ntiles) {
    cudaStream_t s = L.stream;
    // the descriptor staging buffer is reused: wait for the previous upload
    if (L.ev_desc)
        CK(cudaEventSynchronize(L.ev_desc), "cudaEventSynchronize(descriptor upload)");
    long long total = 0;
    L.start_host[0] = 0;
    for (int i = 0; i < ntiles; i++) {
        L.tiles_host[i] = tiles[i];
        total += (long long)tiles[i].nx * tiles[i].ny;
        L.start_host[i + 1] = total;
    }
    CK(cudaMemcpyAsync(L.tiles_dev, L.tiles_host, sizeof(TileDev) * ntiles,
                       cudaMemcpyHostToDevice, s), "copy tile descriptors");
    CK(cudaMemcpyAsync(L.start_dev, L.start_host, sizeof(long long) * (ntiles + 1),
                       cudaMemcpyHostToDevice, s), "copy tile offsets");
    if (L.ev_desc) CK(cudaEventRecord(L.ev_desc, s), "cudaEventRecord");
    return FSG_OK;
}

int launch_on(fsg_ctx *ctx, const LaunchRes &L, const fsg_calc *calc, const TileDev *tiles,
              int ntiles, bool perturb, const Segment &seg) {
    cudaStream_t s = L.stream;
    if (seg.first) {
        if (!seg.uploaded) {
            int rc = upload_descriptors(ctx, L, tiles, ntiles);
            if (rc != FSG_OK) return rc;
        }
        CK(cudaMemsetAsync(L.stats_dev, 0, 4 * sizeof(unsigned long long), s), "reset stats");
        CK(cudaMemsetAsync(L.status_dev, 0, sizeof(int), s), "reset status");
        CK(cudaMemsetAsync(L.used_dev, 0, sizeof(unsigned long long), s), "reset budget");
    }
    CK(cudaMemsetAsync(L.counter_dev, 0, sizeof(unsigned long long), s), "reset counter");
    WorkDev W;
    W.tiles = L.tiles_dev; W.start = L.start_dev; W.ntiles = ntiles;
    W.base = seg.base; W.total = seg.end; W.order = seg.order;
    W.counter = L.counter_dev; W.stats = L.stats_dev;
    W.cancel = ctx->cancel_dev; W.status = L.status_dev;
    W.budget = (unsigned long long)calc->iter_budget; W.used = L.used_dev;
    CalcDev C = make_calc(calc);
    // one persistent wave at the kernel's occupancy limit, or the tuned shape
    const int block = calc->block > 0 ? calc->block : default_block(calc, perturb);
    const int grid = calc->ctas_per_sm > 0 ? -calc->ctas_per_sm : 0;
    if (L.ev0 && seg.first && !seg.keep_time) CK(cudaEventRecord(L.ev0, s), "cudaEventRecord");
    if (!perturb) fsg_launch_std(W, C, grid, block, s);
    else if (calc->flavor == 0 && calc->mode == FSG_MODE_FE32) fsg_launch_perturb_fe32(W, C, grid, block, s);
    else if (calc->mode == FSG_MODE_FE32) fsg_launch_perturb_bs_fe32(W, C, grid, block, s);
    else fsg_launch_perturb(W, C, grid, block, s);
    CK(cudaGetLastError(), "kernel launch");
    if (L.ev1 && seg.last) CK(cudaEventRecord(L.ev1, s), "cudaEventRecord");
    return FSG_OK;
}

// Launch on the context's own stream, timed (one segment: the whole launch
// by default).
int launch_tiles(fsg_ctx *ctx, const fsg_calc *calc, const TileDev *tiles, int ntiles,
                 bool perturb, const Segment *segp = nullptr, bool allow_lpt = true) {
    LaunchRes L;
    L.stream = ctx->stream;
    L.tiles_host = ctx->tiles_host; L.start_host = ctx->start_host;
    L.tiles_dev = ctx->tiles_dev; L.start_dev = ctx->start_dev;
    L.counter_dev = ctx->counter_dev; L.stats_dev = ctx->stats_dev; L.used_dev = ctx->used_dev;
    L.status_dev = ctx->status_dev;
    L.ev_desc = ctx->ev_desc; L.ev0 = ctx->ev0; L.ev1 = ctx->ev1;
    const long long total = tiles_pixels(tiles, ntiles);
    int rc;
    // (not with an iteration budget: its claims stop in claim order, and the
    // pixels left are the caller's to submit again; not for buffers written
    // in place, which keep the caller's values wherever no pixel finished)
    if (allow_lpt && !segp && perturb && calc->claim_order == FSG_ORDER_LONGEST
        && calc->iter_budget == 0 && total >= FSG_LPT_MIN_PIXELS && total < (1LL << 31)) {
        // longest pixels first: a pre-pass over one pixel per 8 x 8 block
        // with max_iter capped at max_iter / 8 (256 .. 4096 iterations), then
        // every pixel in decreasing order of its block's count; the pre-pass
        // counts in no statistic and no budget (the main pass resets them)
        std::vector<int> nx(ntiles), ny(ntiles);
        for (int i = 0; i < ntiles; i++) { nx[i] = tiles[i].nx; ny[i] = tiles[i].ny; }
        const int nblk = fsg_lpt_blocks_count(nx.data(), ny.data(), ntiles);
        const size_t need = align_up(sizeof(int) * (ntiles + 1)) + align_up(4 * 32)
                            + align_up(4 * (size_t)nblk) + align_up((size_t)nblk)
                            + align_up(4 * (size_t)total);
        if (need > ctx->lpt_size) {
            if (ctx->lpt) { cudaStreamSynchronize(ctx->stream); cudaFree(ctx->lpt); }
            ctx->lpt = nullptr; ctx->lpt_size = 0;
            if (cudaMalloc((void **)&ctx->lpt, need) != cudaSuccess) {
                (void)cudaGetLastError();
                return set_err(ctx, FSG_ERR_NOMEM, "claim-order scratch");
            }
            ctx->lpt_size = need;
        }
        char *p = ctx->lpt;
        int *blk_start = (int *)p; p += align_up(sizeof(int) * (ntiles + 1));
        unsigned *hist = (unsigned *)p; p += align_up(4 * 32);
        unsigned *rep = (unsigned *)p; p += align_up(4 * (size_t)nblk);
        unsigned char *bucket = (unsigned char *)p; p += align_up((size_t)nblk);
        unsigned *order = (unsigned *)p;
        rc = upload_descriptors(ctx, L, tiles, ntiles);
        if (rc != FSG_OK) return rc;
        fsg_lpt_prepare(L.tiles_dev, L.start_dev, ntiles, nblk, blk_start, hist, rep, L.stream);
        CK(cudaGetLastError(), "claim order (representatives)");
        fsg_calc pc = *calc;
        pc.max_iter = std::min<int64_t>(calc->max_iter,
                                        std::max<int64_t>(256, std::min<int64_t>(4096, calc->max_iter / 8)));
        pc.iter_budget = 0;
        const Segment pre = {0, nblk, true, false, true, rep, false};
        rc = launch_on(ctx, L, &pc, tiles, ntiles, perturb, pre);
        if (rc != FSG_OK) return rc;
        fsg_lpt_order(L.tiles_dev, L.start_dev, ntiles, nblk, blk_start, hist, rep, bucket,
                      order, L.stream);
        CK(cudaGetLastError(), "claim order");
        const Segment main = {0, total, true, true, true, order, true};
        rc = launch_on(ctx, L, calc, tiles, ntiles, perturb, main);
    } else {
        const Segment whole = {0, total, true, true, false, nullptr};
        rc = launch_on(ctx, L, calc, tiles, ntiles, perturb, segp ? *segp : whole);
    }
    if (rc != FSG_OK) return rc;
    ctx->timed = true;
    ctx->last_pixels = total;
    return FSG_OK;
}

// The checks of a calculation and its tiles (at most FSG_MAX_TILES_PER_LAUNCH)
int check_calc_tiles(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
                     bool perturb) {
    if (calc->max_iter <= 0 || calc->max_iter > FSG_MAX_ITER_LIMIT)
        return set_err(ctx, FSG_ERR_ARG, "max_iter out of range (1 .. 2^30 - 1)");
    if (calc->flavor < 0 || calc->flavor > 5) return set_err(ctx, FSG_ERR_ARG, "bad flavor");
    if (calc->mode < 0 || calc->mode > 2) return set_err(ctx, FSG_ERR_ARG, "bad mode");
    {
        int rc = check_nexp(ctx, calc->flavor, calc->nexp);
        if (rc != FSG_OK) return rc;
    }
    if (perturb && calc->nexp != 0 && calc->mode == FSG_MODE_FE32)
        return set_err(ctx, FSG_ERR_ARG, "the power-n model runs in FSG_MODE_FP64 or FSG_MODE_XR64");
    if (calc->backshift < 0) return set_err(ctx, FSG_ERR_ARG, "backshift must be >= 0");
    if (calc->iter_budget < 0) return set_err(ctx, FSG_ERR_ARG, "iter_budget must be >= 0");
    if (calc->claim_order != FSG_ORDER_PIXELS && calc->claim_order != FSG_ORDER_LONGEST)
        return set_err(ctx, FSG_ERR_ARG, "claim_order: FSG_ORDER_PIXELS or FSG_ORDER_LONGEST");
    if (calc->backshift > 0 && perturb && calc->mode == FSG_MODE_FE32)
        return set_err(ctx, FSG_ERR_ARG, "calc_orbit runs in FSG_MODE_FP64 or FSG_MODE_XR64");
    if (calc->calc_d2zndc2 && (perturb || calc->flavor != 0))
        return set_err(ctx, FSG_ERR_ARG, "calc_d2zndc2 applies to the standard Mandelbrot loops");
    {
        const int bound = default_block(calc, perturb);
        if (calc->block < 0 || calc->block % 32 != 0 || calc->block > bound)
            return set_err(ctx, FSG_ERR_ARG, "block: 0 or a multiple of 32 up to the kernel's 256 "
                                             "(128 for the FE32 power-2 kernel)");
        if (calc->ctas_per_sm < 0) return set_err(ctx, FSG_ERR_ARG, "ctas_per_sm must be >= 0");
    }
    for (int32_t i = 0; i < ntiles; i++) {
        int rc = check_tile(ctx, tiles[i], perturb, calc);
        if (rc != FSG_OK) return rc;
    }
    return FSG_OK;
}

// tables of derived references may still be building on another stream:
// the launch stream waits for them on the device
int wait_references(fsg_ctx *ctx, const fsg_tile *tiles, int32_t ntiles, cudaStream_t s) {
    for (int32_t i = 0; i < ntiles; i++) {
        fsg_ref *r = tiles[i].ref;
        if (r && r->ready && (i == 0 || tiles[i - 1].ref != r))
            CK(cudaStreamWaitEvent(s, r->ready, 0), "cudaStreamWaitEvent(reference)");
    }
    return FSG_OK;
}

size_t zbytes(const fsg_calc *calc) { return calc->flavor == 0 ? 16 : 8; }

// device bytes that host-buffer tiles occupy once staged
size_t staged_bytes(const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles) {
    const size_t zsz = zbytes(calc);
    size_t bytes = 0;
    for (int32_t i = 0; i < ntiles; i++) {
        const fsg_tile &t = tiles[i];
        size_t np = (size_t)t.nx * t.ny;
        bytes += (t.pix ? align_up(16 * np) : align_up(8 * t.nx) + align_up(8 * t.ny))
                 + align_up(zsz * t.nZ * np)
                 + align_up(4 * np) + align_up(np) + align_up(4 * np);
        if (t.potential) bytes += align_up(8 * np);
        if (t.dem) bytes += align_up(8 * np);
    }
    return bytes;
}

// Copy host-buffer tiles' inputs to the device area at p (staged_bytes long)
// and lay out their outputs there, on stream s; td receives the descriptors.
int stage_tiles(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
                char *p, cudaStream_t s, TileDev *td) {
    const size_t zsz = zbytes(calc);
    for (int32_t i = 0; i < ntiles; i++) {
        fsg_tile t = tiles[i];
        size_t np = (size_t)t.nx * t.ny;
        if (t.pix) {
            double *pp = (double *)p; p += align_up(16 * np);
            CK(cudaMemcpyAsync(pp, t.pix, 16 * np, cudaMemcpyHostToDevice, s), "copy pix");
            t.pix = pp; t.xs = nullptr; t.ys = nullptr;
        } else {
            double *xs = (double *)p; p += align_up(8 * t.nx);
            double *ys = (double *)p; p += align_up(8 * t.ny);
            CK(cudaMemcpyAsync(xs, t.xs, 8 * t.nx, cudaMemcpyHostToDevice, s), "copy xs");
            CK(cudaMemcpyAsync(ys, t.ys, 8 * t.ny, cudaMemcpyHostToDevice, s), "copy ys");
            t.xs = xs; t.ys = ys;
        }
        t.Z = p; p += align_up(zsz * t.nZ * np);
        // fields the kernel does not produce come back as zeros, like the
        // caller's freshly allocated arrays (core.py:2070-2073)
        CK(cudaMemsetAsync(t.Z, 0, zsz * t.nZ * np, s), "zero Z");
        t.U = tiles[i].U ? (int32_t *)p : nullptr; p += align_up(4 * np);
        t.stop_reason = (int8_t *)p; p += align_up(np);
        // -1 until a pixel stops: what a launch cut by its budget returns
        // for the pixels it did not run
        CK(cudaMemsetAsync(t.stop_reason, 0xff, np, s), "init stop_reason");
        t.stop_iter = (int32_t *)p; p += align_up(4 * np);
        if (t.potential) { t.potential = (double *)p; p += align_up(8 * np); }
        if (t.dem) { t.dem = (double *)p; p += align_up(8 * np); }
        td[i] = make_tile(t);
    }
    return FSG_OK;
}

// Copy staged outputs back into the caller's host buffers, on stream s.
int copy_back(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
              const TileDev *td, cudaStream_t s) {
    const size_t zsz = zbytes(calc);
    for (int32_t i = 0; i < ntiles; i++) {
        const fsg_tile &t = tiles[i];
        const TileDev &d = td[i];
        size_t np = (size_t)t.nx * t.ny;
        CK(cudaMemcpyAsync(t.Z, d.Z, zsz * t.nZ * np, cudaMemcpyDeviceToHost, s), "copy Z back");
        if (t.U) CK(cudaMemcpyAsync(t.U, d.U, 4 * np, cudaMemcpyDeviceToHost, s), "copy U back");
        CK(cudaMemcpyAsync(t.stop_reason, d.stop_reason, np, cudaMemcpyDeviceToHost, s), "copy stop_reason back");
        CK(cudaMemcpyAsync(t.stop_iter, d.stop_iter, 4 * np, cudaMemcpyDeviceToHost, s), "copy stop_iter back");
        if (t.potential) CK(cudaMemcpyAsync(t.potential, d.pot, 8 * np, cudaMemcpyDeviceToHost, s), "copy potential back");
        if (t.dem) CK(cudaMemcpyAsync(t.dem, d.dem, 8 * np, cudaMemcpyDeviceToHost, s), "copy dem back");
    }
    return FSG_OK;
}

// Copy the staged outputs of the pixels [p0, p1) of the concatenated tiles
// back into the caller's host buffers, on stream s.
int copy_back_range(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
                    const TileDev *td, long long p0, long long p1, cudaStream_t s) {
    const size_t zsz = zbytes(calc);
    long long ts = 0;
    for (int32_t i = 0; i < ntiles; i++) {
        const fsg_tile &t = tiles[i];
        const TileDev &d = td[i];
        const long long np = (long long)t.nx * t.ny, te = ts + np;
        const long long a = (p0 > ts ? p0 : ts) - ts, b = (p1 < te ? p1 : te) - ts;
        ts = te;
        if (a >= b) continue;
        const size_t n = (size_t)(b - a);
        for (int k = 0; k < t.nZ; k++) {
            const size_t off = zsz * ((size_t)k * np + a);
            CK(cudaMemcpyAsync((char *)t.Z + off, (const char *)d.Z + off, zsz * n,
                               cudaMemcpyDeviceToHost, s), "copy Z back");
        }
        if (t.U) CK(cudaMemcpyAsync(t.U + a, d.U + a, 4 * n, cudaMemcpyDeviceToHost, s), "copy U back");
        CK(cudaMemcpyAsync(t.stop_reason + a, d.stop_reason + a, n, cudaMemcpyDeviceToHost, s),
           "copy stop_reason back");
        CK(cudaMemcpyAsync(t.stop_iter + a, d.stop_iter + a, 4 * n, cudaMemcpyDeviceToHost, s),
           "copy stop_iter back");
        if (t.potential)
            CK(cudaMemcpyAsync(t.potential + a, d.pot + a, 8 * n, cudaMemcpyDeviceToHost, s),
               "copy potential back");
        if (t.dem)
            CK(cudaMemcpyAsync(t.dem + a, d.dem + a, 8 * n, cudaMemcpyDeviceToHost, s),
               "copy dem back");
    }
    return FSG_OK;
}

// The device address of a page-locked host array (cudaHostAlloc,
// cudaHostRegister), nullptr for pageable memory (or a null pointer).
void *pinned_device_ptr(const void *p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Host-buffer tiles whose every array is page-locked, as device-addressable
// descriptors in td: the kernels then read the inputs and write the outputs
// in place (over NVLink-C2C on GB300, as the pixels finish), with no staging
// and no copy-back.  False when any array is pageable.
bool pinned_tiles(const fsg_tile *tiles, int32_t ntiles, TileDev *td) {
    for (int32_t i = 0; i < ntiles; i++) {
        fsg_tile t = tiles[i];
        const void *in[3] = {t.pix, t.xs, t.ys};
        void *out[6] = {t.Z, t.U, t.stop_reason, t.stop_iter, t.potential, t.dem};
        void *din[3], *dout[6];
        for (int q = 0; q < 3; q++) {
            din[q] = pinned_device_ptr(in[q]);
            if (in[q] && !din[q]) return false;
        }
        for (int q = 0; q < 6; q++) {
            dout[q] = pinned_device_ptr(out[q]);
            if (out[q] && !dout[q]) return false;
        }
        t.pix = (const double *)din[0]; t.xs = (const double *)din[1];
        t.ys = (const double *)din[2];
        t.Z = dout[0]; t.U = (int32_t *)dout[1]; t.stop_reason = (int8_t *)dout[2];
        t.stop_iter = (int32_t *)dout[3]; t.potential = (double *)dout[4];
        t.dem = (double *)dout[5];
        td[i] = make_tile(t);
    }
    return true;
}

// Segments of a streamed host-buffer call: a perturbation launch of at least
// 2 FSG_COPY_SEGMENT_PIXELS pixels runs as up to FSG_COPY_SEGMENTS launches
// over consecutive pixel ranges, each segment's outputs copied back on the
// copy stream while the next one computes.
int copy_segments(bool perturb, long long total) {
    if (!perturb) return 1;
    long long k = total / FSG_COPY_SEGMENT_PIXELS;
    if (k < 2) return 1;
    return k > FSG_COPY_SEGMENTS ? FSG_COPY_SEGMENTS : (int)k;
}

int run_tiles(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
              int32_t where, bool perturb) {
    if (!ctx) return FSG_ERR_ARG;
    if (!calc || !tiles || ntiles <= 0) return set_err(ctx, FSG_ERR_ARG, "no tiles");
    if (ntiles > FSG_MAX_TILES_PER_LAUNCH) {
        // split into several launches of at most FSG_MAX_TILES_PER_LAUNCH tiles
        for (int32_t i = 0; i < ntiles; i += FSG_MAX_TILES_PER_LAUNCH) {
            int32_t n = ntiles - i < FSG_MAX_TILES_PER_LAUNCH ? ntiles - i : FSG_MAX_TILES_PER_LAUNCH;
            int rc = run_tiles(ctx, calc, tiles + i, n, where, perturb);
            if (rc != FSG_OK) return rc;
        }
        return FSG_OK;
    }
    int rc = check_calc_tiles(ctx, calc, tiles, ntiles, perturb);
    if (rc != FSG_OK) return rc;
    rc = wait_references(ctx, tiles, ntiles, ctx->stream);
    if (rc != FSG_OK) return rc;
    std::vector<TileDev> td(ntiles);
    if (where == FSG_DEVICE) {
        for (int32_t i = 0; i < ntiles; i++) td[i] = make_tile(tiles[i]);
        return launch_tiles(ctx, calc, td.data(), ntiles, perturb);
    }
    if (where != FSG_HOST) return set_err(ctx, FSG_ERR_ARG, "where must be FSG_HOST or FSG_DEVICE");
    if (pinned_tiles(tiles, ntiles, td.data())) {
        // page-locked host buffers, written in place
        if (*ctx->cancel_host) return FSG_INTERRUPTED;
        rc = launch_tiles(ctx, calc, td.data(), ntiles, perturb, nullptr, false);
        if (rc != FSG_OK) return rc;
        return fsg_sync(ctx);
    }
    // pageable host buffers: stage in the grow-only device scratch area
    rc = ensure_scratch(ctx, staged_bytes(calc, tiles, ntiles));
    if (rc != FSG_OK) return rc;
    rc = stage_tiles(ctx, calc, tiles, ntiles, ctx->scratch, ctx->stream, td.data());
    if (rc != FSG_OK) return rc;
    const long long total = tiles_pixels(td.data(), ntiles);
    const int nseg = copy_segments(perturb, total);
    if (nseg > 1) {
        // streamed: segment k computes on the context stream while the
        // outputs of segment k - 1 travel back on the copy stream.  An
        // interruption during the call may leave the outputs of the segments
        // that finished before it written (the reference's loop also writes
        // its arrays in place; it discards an interrupted tile).
        // Every segment is queued before the first copy: a copy into pageable
        // memory returns only once done, and the launches keep the GPU busy
        // meanwhile.
        if (*ctx->cancel_host) return FSG_INTERRUPTED;
        for (int k = 0; k < nseg; k++) {
            const Segment seg = {total * k / nseg, total * (k + 1) / nseg, k == 0, k == nseg - 1};
            rc = launch_tiles(ctx, calc, td.data(), ntiles, perturb, &seg);
            if (rc != FSG_OK) return rc;
            CK(cudaEventRecord(ctx->ev_seg[k], ctx->stream), "cudaEventRecord(segment)");
        }
        for (int k = 0; k < nseg; k++) {
            CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_seg[k], 0), "cudaStreamWaitEvent(segment)");
            rc = copy_back_range(ctx, calc, tiles, ntiles, td.data(), total * k / nseg,
                                 total * (k + 1) / nseg, ctx->copy_stream);
            if (rc != FSG_OK) return rc;
        }
        // the context stream's later work (the next call's staging) waits
        // for the copies out of the scratch area
        CK(cudaEventRecord(ctx->ev_seg[nseg - 1], ctx->copy_stream), "cudaEventRecord(copies)");
        CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_seg[nseg - 1], 0), "cudaStreamWaitEvent(copies)");
        CK(cudaStreamSynchronize(ctx->copy_stream), "cudaStreamSynchronize(copy stream)");
        return fsg_sync(ctx);
    }
    rc = launch_tiles(ctx, calc, td.data(), ntiles, perturb);
    if (rc != FSG_OK) return rc;
    // an interrupted launch leaves the caller's arrays untouched (the
    // reference discards an interrupted tile, core.py:2545-2547); one cut by
    // its budget returns what it ran (stop_reason -1 elsewhere)
    rc = fsg_sync(ctx);
    if (rc != FSG_OK && rc != FSG_BUDGET) return rc;
    const int launch_rc = rc;
    rc = copy_back(ctx, calc, tiles, ntiles, td.data(), ctx->stream);
    if (rc != FSG_OK) return rc;
    rc = fsg_sync(ctx);
    return rc == FSG_OK ? launch_rc : rc;
}

}  // namespace

namespace {
// Stage one host array into the scratch area (FSG_HOST) or take the device
// pointer as is; `p` advances past the staged bytes.
template <class T>
int stage_in(fsg_ctx *ctx, int32_t where, const void *src, size_t bytes, char *&p, const T *&dst) {
    if (where == FSG_DEVICE || !src) { dst = (const T *)src; return FSG_OK; }
    CK(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "copy post-processing input");
    dst = (const T *)p;
    p += align_up(bytes);
    return FSG_OK;
}
}  // namespace

extern "C" {

const char *fsg_version(void) { return FSG_VERSION; }

int fsg_ctx_create(int device, fsg_ctx **out) {
    if (!out) return FSG_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return FSG_ERR_NODEV;
    if (device < 0 || device >= n) return FSG_ERR_ARG;
    fsg_ctx *ctx = new (std::nothrow) fsg_ctx();
    if (!ctx) return FSG_ERR_NOMEM;
    ctx->device = device;
    int rc = FSG_OK;
    do {
        if (cudaSetDevice(device) != cudaSuccess) { rc = FSG_ERR_CUDA; break; }
        cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
        if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) { rc = FSG_ERR_CUDA; break; }
        if (cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess) { rc = FSG_ERR_CUDA; break; }
        {
            bool ok = true;
            for (int k = 0; k < FSG_COPY_SEGMENTS && ok; k++)
                ok = cudaEventCreateWithFlags(&ctx->ev_seg[k], cudaEventDisableTiming) == cudaSuccess;
            if (!ok) { rc = FSG_ERR_CUDA; break; }
        }
        ctx->stream = ctx->own_stream;
        int *h = nullptr;
        if (cudaHostAlloc((void **)&h, sizeof(int), cudaHostAllocMapped) != cudaSuccess) { rc = FSG_ERR_CUDA; break; }
        *h = 0;
        ctx->cancel_host = h;
        if (cudaHostGetDevicePointer((void **)&ctx->cancel_dev, h, 0) != cudaSuccess) { rc = FSG_ERR_CUDA; break; }
        if (cudaMalloc((void **)&ctx->status_dev, sizeof(int)) != cudaSuccess) { rc = FSG_ERR_NOMEM; break; }
        if (cudaMalloc((void **)&ctx->used_dev, sizeof(unsigned long long)) != cudaSuccess) { rc = FSG_ERR_NOMEM; break; }
        if (cudaMalloc((void **)&ctx->counter_dev, sizeof(unsigned long long)) != cudaSuccess) { rc = FSG_ERR_NOMEM; break; }
        if (cudaMalloc((void **)&ctx->stats_dev, 4 * sizeof(unsigned long long)) != cudaSuccess) { rc = FSG_ERR_NOMEM; break; }
        if (cudaMalloc((void **)&ctx->tiles_dev, sizeof(TileDev) * FSG_MAX_TILES_PER_LAUNCH) != cudaSuccess) { rc = FSG_ERR_NOMEM; break; }
        if (cudaMalloc((void **)&ctx->start_dev, sizeof(long long) * (FSG_MAX_TILES_PER_LAUNCH + 1)) != cudaSuccess) { rc = FSG_ERR_NOMEM; break; }
        if (cudaHostAlloc((void **)&ctx->tiles_host, sizeof(TileDev) * FSG_MAX_TILES_PER_LAUNCH, 0) != cudaSuccess) { rc = FSG_ERR_NOMEM; break; }
        if (cudaHostAlloc((void **)&ctx->start_host, sizeof(long long) * (FSG_MAX_TILES_PER_LAUNCH + 1), 0) != cudaSuccess) { rc = FSG_ERR_NOMEM; break; }
        if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess
            || cudaEventCreateWithFlags(&ctx->ev_desc, cudaEventDisableTiming) != cudaSuccess) { rc = FSG_ERR_CUDA; break; }
        cudaEventRecord(ctx->ev_desc, ctx->stream);
    } while (0);
    if (rc != FSG_OK) { fsg_ctx_destroy(ctx); return rc; }
    *out = ctx;
    return FSG_OK;
}

int fsg_ctx_destroy(fsg_ctx *ctx) {
    if (!ctx) return FSG_OK;
    cudaSetDevice(ctx->device);
    if (ctx->serve) fsg_serve_close(ctx);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->lpt) cudaFree(ctx->lpt);
    if (ctx->status_dev) cudaFree(ctx->status_dev);
    if (ctx->used_dev) cudaFree(ctx->used_dev);
    if (ctx->counter_dev) cudaFree(ctx->counter_dev);
    if (ctx->stats_dev) cudaFree(ctx->stats_dev);
    if (ctx->tiles_dev) cudaFree(ctx->tiles_dev);
    if (ctx->start_dev) cudaFree(ctx->start_dev);
    if (ctx->tiles_host) cudaFreeHost(ctx->tiles_host);
    if (ctx->start_host) cudaFreeHost(ctx->start_host);
    if (ctx->cancel_host) cudaFreeHost((void *)ctx->cancel_host);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ev_desc) cudaEventDestroy(ctx->ev_desc);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    for (int k = 0; k < FSG_COPY_SEGMENTS; k++)
        if (ctx->ev_seg[k]) cudaEventDestroy(ctx->ev_seg[k]);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return FSG_OK;
}

const char *fsg_last_error(const fsg_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int fsg_set_stream(fsg_ctx *ctx, void *stream) {
    if (!ctx) return FSG_ERR_ARG;
    cudaStreamSynchronize(ctx->stream);
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    cudaEventRecord(ctx->ev_desc, ctx->stream);
    return FSG_OK;
}

int fsg_sync(fsg_ctx *ctx) {
    if (!ctx) return FSG_ERR_ARG;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    int st = 0;
    CK(cudaMemcpy(&st, ctx->status_dev, sizeof(int), cudaMemcpyDeviceToHost), "read status");
    return st == 1 ? FSG_INTERRUPTED : (st == 2 ? FSG_BUDGET : FSG_OK);
}

int fsg_cancel(fsg_ctx *ctx) {
    if (!ctx) return FSG_ERR_ARG;
    *ctx->cancel_host = 1;
    return FSG_OK;
}

int fsg_clear_cancel(fsg_ctx *ctx) {
    if (!ctx) return FSG_ERR_ARG;
    *ctx->cancel_host = 0;
    return FSG_OK;
}

int fsg_ref_create(fsg_ctx *ctx, const fsg_ref_desc *d, fsg_ref **out) {
    if (!ctx || !d || !out) return set_err(ctx, FSG_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (!d->Zn || d->len < 2) return set_err(ctx, FSG_ERR_ARG, "orbit shorter than 2 points");
    if (d->len >= INT_MAX / 2) return set_err(ctx, FSG_ERR_ARG, "orbit too long");
    if (d->n_xr < 0 || (d->n_xr > 0 && (!d->xr_idx || !d->xr_m || !d->xr_e)))
        return set_err(ctx, FSG_ERR_ARG, "bad Xrange side table");
    if (d->flavor < 0 || d->flavor > 5) return set_err(ctx, FSG_ERR_ARG, "bad flavor");
    {
        int rc = check_nexp(ctx, d->flavor, d->nexp);
        if (rc != FSG_OK) return rc;
    }
    const int len = (int)d->len;
    // the iteration index w never passes min(order, div_iter) <= len, so every
    // orbit read stays inside [0, len] (slot len is a zero pad)
    if ((d->order <= 0 || d->order > d->len) && (d->div_iter > d->len || d->div_iter < 1))
        return set_err(ctx, FSG_ERR_ARG, "div_iter must be in [1, len] for a non-cycling reference");
    for (int k = 0; k < d->n_xr; k++) {
        if (d->xr_idx[k] < 0 || d->xr_idx[k] >= len || (k > 0 && d->xr_idx[k] <= d->xr_idx[k - 1]))
            return set_err(ctx, FSG_ERR_ARG, "Xrange side-table indices must be increasing and inside the orbit");
    }
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    fsg_ref *r = new (std::nothrow) fsg_ref();
    if (!r) return set_err(ctx, FSG_ERR_NOMEM, "out of host memory");
    r->len = len; r->flavor = d->flavor; r->xr_paths = d->xr_paths;
    r->has_dzndc = d->calc_dzndc; r->has_dzndz = (d->flavor == 0) && d->calc_dzndz;
    r->bla_req = d->bla != 0;
    RefDev &R = r->host;
    memset(&R, 0, sizeof(R));
    R.len = len;
    R.div_iter = (int)(d->div_iter < (int64_t)INT_MAX ? d->div_iter : INT_MAX);
    R.order = (d->order > 0 && d->order < (int64_t)INT_MAX) ? (int)d->order : INT_MAX;
    R.first_invalid = len;
    if (R.div_iter < R.first_invalid) R.first_invalid = R.div_iter;
    if (R.order < R.first_invalid) R.first_invalid = R.order;
    R.flavor = d->flavor;
    R.n_xr = d->n_xr;
    // binomial coefficients C(n, k) as float64, exact for n <= FSG_MN_MAX_EXP
    // (mandelbrot_Mn.py:636-640 math.comb)
    r->nexp = R.nexp = d->nexp;
    for (int k = 0; k <= d->nexp; k++) {
        unsigned long long v = 1;
        for (int j = 1; j <= k; j++) v = v * (unsigned long long)(d->nexp - k + j) / (unsigned long long)j;
        R.binom[k] = (double)v;
    }
    cudaStream_t s = ctx->stream;
    int rc = FSG_OK;
#define RA(ptr, n) do { rc = ref_alloc(ctx, r, &(ptr), (n)); if (rc != FSG_OK) { ref_release(r, s); delete r; return rc; } } while (0)
#define RCK(call, what) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { ref_release(r, s); delete r; return cuda_err(ctx, e_, what); } } while (0)
    double2 *Zn; RA(Zn, len + 1);
    RCK(cudaMemcpyAsync(Zn, d->Zn, 16 * (size_t)len, cudaMemcpyHostToDevice, s), "upload orbit");
    RCK(cudaMemsetAsync(Zn + len, 0, 16, s), "pad orbit");
    R.Zn = Zn;
    std::vector<int> slot;
    std::vector<double2> xm;
    int *xr_slot = nullptr; double2 *xr_m = nullptr; int *xr_e = nullptr;
    if (d->n_xr > 0) {
        slot.assign(len + 1, -1);
        for (int k = 0; k < d->n_xr; k++) slot[d->xr_idx[k]] = k;
        // BS: one exponent per coordinate
        const int ne = d->flavor == 0 ? d->n_xr : 2 * d->n_xr;
        RA(xr_slot, len + 1); RA(xr_m, d->n_xr); RA(xr_e, ne);
        // stream-ordered like the allocations (pageable sources: staged before return)
        RCK(cudaMemcpyAsync(xr_slot, slot.data(), 4 * (size_t)(len + 1), cudaMemcpyHostToDevice, s), "upload xr slots");
        RCK(cudaMemcpyAsync(xr_m, d->xr_m, 16 * (size_t)d->n_xr, cudaMemcpyHostToDevice, s), "upload xr mantissas");
        RCK(cudaMemcpyAsync(xr_e, d->xr_e, 4 * (size_t)ne, cudaMemcpyHostToDevice, s), "upload xr exponents");
    }
    R.xr_slot = xr_slot; R.xr_m = xr_m; R.xr_e = xr_e;
    // derivative paths
    double2 *dzndc = nullptr, *dzndc_xm = nullptr, *dzndz = nullptr, *dzndz_xm = nullptr;
    int *dzndc_xe = nullptr, *dzndz_xe = nullptr;
    double *dXa = nullptr, *dXb = nullptr, *dYa = nullptr, *dYb = nullptr;
    double *bs_xpm = nullptr; int *bs_xpe = nullptr;
    if (d->flavor == 0) {
        if (d->calc_dzndc) {
            if (d->xr_paths) { RA(dzndc_xm, len + 1); RA(dzndc_xe, len + 1); }
            else RA(dzndc, len + 1);
        }
        if (d->calc_dzndz) {
            if (d->xr_paths) { RA(dzndz_xm, len + 2); RA(dzndz_xe, len + 2); }
            else RA(dzndz, len + 2);
        }
    } else if (d->calc_dzndc) {
        RA(dXa, len + 1); RA(dXb, len + 1); RA(dYa, len + 1); RA(dYb, len + 1);
        if (d->xr_paths) { RA(bs_xpm, 4 * (size_t)(len + 1)); RA(bs_xpe, 4 * (size_t)(len + 1)); }
    }
    R.dZndc = dzndc; R.dZndc_xm = dzndc_xm; R.dZndc_xe = dzndc_xe;
    R.dZndz = dzndz; R.dZndz_xm = dzndz_xm; R.dZndz_xe = dzndz_xe;
    R.dXa = dXa; R.dXb = dXb; R.dYa = dYa; R.dYb = dYb;
    R.bs_xpm = bs_xpm; R.bs_xpe = bs_xpe;
    // BLA
    int L = len / 8;
    double2 *Mbla = nullptr; double *Mbs = nullptr, *rbla = nullptr;
    int stages = (int)ceil(log2((double)len));
    if (d->bla && L > 0) {
        if (d->flavor == 0) RA(Mbla, 4 * (size_t)L); else RA(Mbs, 16 * (size_t)L);
        RA(rbla, 2 * (size_t)L);
        RCK(cudaMemsetAsync(rbla, 0, 16 * (size_t)L, s), "zero BLA radii");
        if (Mbla) RCK(cudaMemsetAsync(Mbla, 0, 64 * (size_t)L, s), "zero BLA");
        if (Mbs) RCK(cudaMemsetAsync(Mbs, 0, 128 * (size_t)L, s), "zero BLA");
        R.bla_len = 2 * L;
    }
    R.Mbla = Mbla; R.Mbla_bs = Mbs; R.rbla = rbla; R.stages = stages;
    // fe tables (M2)
    int4 *Zf = nullptr, *Zp = nullptr, *dzndc_f = nullptr, *dzndz_f = nullptr, *bla_f = nullptr,
         *bla_first = nullptr, *bla_chain = nullptr, *fe_runs = nullptr;
    int *bla_first_step = nullptr;
    int2 *bla_chain_step = nullptr;
    const int bla_nit = (len >> 3) + 1;
    const bool fe_tables = d->flavor == 0 && d->nexp == 0;   // FE32 is the power-2 form
    if (fe_tables) {
        RA(Zf, len + 1);
        RA(Zp, len + 1);
        RA(fe_runs, 5 * (size_t)(len + 1));
        if (d->calc_dzndc) RA(dzndc_f, len + 1);
        if (d->calc_dzndz) RA(dzndz_f, len + 2);
        if (R.bla_len > 0) {
            RA(bla_f, 2 * (size_t)R.bla_len);
            RA(bla_first, 2 * (size_t)bla_nit);
            RA(bla_first_step, (size_t)bla_nit);
            RA(bla_chain, 2 * (size_t)bla_nit);
            RA(bla_chain_step, (size_t)bla_nit);
        }
    }
    R.Zf = Zf; R.Zp = Zp; R.dZndc_f = dzndc_f; R.dZndz_f = dzndz_f; R.bla_f = bla_f;
    R.bla_first = bla_first; R.bla_first_step = bla_first_step; R.bla_nit = bla_nit;
    R.bla_chain = bla_chain; R.bla_chain_step = bla_chain_step;
    R.fe_runs = fe_runs;
    // FP32+exp tables (Burning Ship)
    int4 *bs_Zf = nullptr, *bs_hf = nullptr, *bs_blaf = nullptr;
    int2 *bs_rf = nullptr;
    float4 *bs_fa = nullptr, *bs_fh = nullptr;
    int4 *bs_fz = nullptr;
    if (d->flavor != 0) {
        RA(bs_Zf, len + 1);
        RA(bs_fa, len + 1);
        RA(bs_fz, len + 1);
        if (d->calc_dzndc) {
            RA(bs_hf, 2 * (size_t)(len + 1));
            RA(bs_fh, len + 1);
        }
        if (R.bla_len > 0) {
            RA(bs_blaf, 4 * (size_t)R.bla_len);
            RA(bs_rf, (size_t)R.bla_len);
        }
    }
    R.bs_Zf = bs_Zf; R.bs_hf = bs_hf; R.bs_blaf = bs_blaf; R.bs_rf = bs_rf;
    R.bs_fa = bs_fa; R.bs_fz = bs_fz; R.bs_fh = bs_fh;
    RCK(cudaMallocAsync((void **)&r->dev, sizeof(RefDev), s), "cudaMallocAsync(reference descriptor)");
    RCK(cudaMemcpyAsync(r->dev, &R, sizeof(RefDev), cudaMemcpyHostToDevice, s), "upload descriptor");
    // builds
    if (d->flavor == 0) {
        fsg_build_paths_m2(r->dev, len, dzndc, dzndc_xm, dzndc_xe, dzndz, dzndz_xm, dzndz_xe,
                           R.div_iter, d->xr_paths, d->calc_dzndc, d->calc_dzndz, d->scale_m,
                           d->scale_e, s);
    } else if (d->calc_dzndc) {
        fsg_build_paths_bs(r->dev, len, dXa, dXb, dYa, dYb, ldexp(d->scale_m, d->scale_e), s);
        if (bs_xpm) fsg_build_paths_bs_xr(r->dev, len, bs_xpm, bs_xpe, d->scale_m, d->scale_e, s);
    }
    if (R.bla_len > 0) fsg_build_bla(r->dev, d->flavor, len, Mbla, Mbs, rbla, stages, d->kc, d->bla_eps, s);
    if (d->flavor != 0) {
        fsg_build_bs_fr(r->dev, len, bs_Zf, dXa, dXb, dYa, dYb, bs_hf, bs_fa, bs_fz, bs_fh,
                        R.div_iter, s);
        fsg_build_bs_fr_bla(Mbs, rbla, R.bla_len, bs_blaf, bs_rf, s);
    }
    if (fe_tables) {
        fsg_build_fe_tables(r->dev, len, Zf, dzndc, dzndc_xm, dzndc_xe, dzndc_f, dzndz, dzndz_xm,
                            dzndz_xe, dzndz_f, Mbla, rbla, R.bla_len, bla_f, bla_nit, bla_first,
                            bla_first_step, d->kc, bla_chain, bla_chain_step, s);
        fsg_build_plain_orbit(r->dev, len, Zf, Zp, s);
        fsg_build_fe_runs(r->dev, len, Zp, dzndc_f, fe_runs, s);
    }
    RCK(cudaGetLastError(), "reference table kernels");
    RCK(cudaStreamSynchronize(s), "reference table build");
#undef RA
#undef RCK
    *out = r;
    return FSG_OK;
}

int fsg_ref_destroy(fsg_ctx *ctx, fsg_ref *ref) {
    if (!ref) return FSG_OK;
    if (ref->derived > 0)
        return set_err(ctx, FSG_ERR_ARG, "reference still has derived references");
    cudaStream_t s = nullptr;
    if (ctx) { cudaSetDevice(ctx->device); cudaStreamSynchronize(ctx->stream); s = ctx->stream; }
    if (ref->ready) { cudaEventSynchronize(ref->ready); cudaEventDestroy(ref->ready); }
    ref_release(ref, s);
    if (ref->base) ref->base->derived--;
    delete ref;
    if (s) cudaStreamSynchronize(s);
    return FSG_OK;
}

int fsg_ref_derive_bla(fsg_ctx *ctx, fsg_ref *base, double kc, double bla_eps, fsg_ref **out) {
    if (!ctx || !base || !out) return set_err(ctx, FSG_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (base->base) return set_err(ctx, FSG_ERR_ARG, "derive from the reference that owns the orbit");
    if (!(kc >= 0.) || !(bla_eps >= 0.)) return set_err(ctx, FSG_ERR_ARG, "bad kc or BLA eps");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    fsg_ref *r = new (std::nothrow) fsg_ref();
    if (!r) return set_err(ctx, FSG_ERR_NOMEM, "out of host memory");
    r->len = base->len; r->flavor = base->flavor; r->xr_paths = base->xr_paths;
    r->has_dzndc = base->has_dzndc; r->has_dzndz = base->has_dzndz;
    r->bla_req = 1;
    r->nexp = base->nexp;
    r->base = base;
    RefDev &R = r->host;
    R = base->host;                  // shares the orbit, side table, paths, fe orbit
    const int len = (int)base->len;
    const int L = len / 8;
    cudaStream_t s = ctx->stream;
    int rc = FSG_OK;
#define RA(ptr, n) do { rc = ref_alloc(ctx, r, &(ptr), (n)); if (rc != FSG_OK) { ref_release(r, s); delete r; return rc; } } while (0)
#define RCK(call, what) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { ref_release(r, s); delete r; return cuda_err(ctx, e_, what); } } while (0)
    double2 *Mbla = nullptr; double *Mbs = nullptr, *rbla = nullptr;
    int4 *bla_f = nullptr, *bla_first = nullptr, *bla_chain = nullptr;
    int *bla_first_step = nullptr;
    int2 *bla_chain_step = nullptr;
    R.bla_len = 0;
    if (L > 0) {
        if (R.flavor == 0) RA(Mbla, 4 * (size_t)L); else RA(Mbs, 16 * (size_t)L);
        RA(rbla, 2 * (size_t)L);
        RCK(cudaMemsetAsync(rbla, 0, 16 * (size_t)L, s), "zero BLA radii");
        if (Mbla) RCK(cudaMemsetAsync(Mbla, 0, 64 * (size_t)L, s), "zero BLA");
        if (Mbs) RCK(cudaMemsetAsync(Mbs, 0, 128 * (size_t)L, s), "zero BLA");
        R.bla_len = 2 * L;
        if (R.flavor == 0 && R.nexp == 0) {
            RA(bla_f, 2 * (size_t)R.bla_len);
            RA(bla_first, 2 * (size_t)R.bla_nit);
            RA(bla_first_step, (size_t)R.bla_nit);
            RA(bla_chain, 2 * (size_t)R.bla_nit);
            RA(bla_chain_step, (size_t)R.bla_nit);
        }
    }
    int4 *bs_blaf = nullptr;
    int2 *bs_rf = nullptr;
    if (R.flavor != 0 && R.bla_len > 0) {
        RA(bs_blaf, 4 * (size_t)R.bla_len);
        RA(bs_rf, (size_t)R.bla_len);
    }
    R.Mbla = Mbla; R.Mbla_bs = Mbs; R.rbla = rbla; R.bs_blaf = bs_blaf; R.bs_rf = bs_rf;
    R.bla_f = bla_f; R.bla_first = bla_first; R.bla_first_step = bla_first_step;
    R.bla_chain = bla_chain; R.bla_chain_step = bla_chain_step;
    RCK(cudaMallocAsync((void **)&r->dev, sizeof(RefDev), s), "cudaMallocAsync(reference descriptor)");
    RCK(cudaMemcpyAsync(r->dev, &R, sizeof(RefDev), cudaMemcpyHostToDevice, s), "upload descriptor");
    if (R.bla_len > 0) {
        fsg_build_bla(r->dev, R.flavor, len, Mbla, Mbs, rbla, R.stages, kc, bla_eps, s);
        if (R.flavor == 0 && R.nexp == 0)
            fsg_build_fe_bla(r->dev, Mbla, rbla, R.bla_len, bla_f, R.bla_nit, bla_first,
                             bla_first_step, kc, bla_chain, bla_chain_step, s);
        else if (R.flavor != 0)
            fsg_build_bs_fr_bla(Mbs, rbla, R.bla_len, bs_blaf, bs_rf, s);
    }
    RCK(cudaGetLastError(), "BLA kernels");
    // no host wait: launches and downloads that use r wait for this event
    RCK(cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming), "cudaEventCreate");
    RCK(cudaEventRecord(r->ready, s), "cudaEventRecord(reference)");
#undef RA
#undef RCK
    base->derived++;
    *out = r;
    return FSG_OK;
}

int fsg_ref_info(const fsg_ref *ref, int64_t *len, int64_t *bla_len, int32_t *stages) {
    if (!ref) return FSG_ERR_ARG;
    if (len) *len = ref->len;
    if (bla_len) *bla_len = ref->host.bla_len;
    if (stages) *stages = ref->host.stages;
    return FSG_OK;
}

int fsg_ref_download(fsg_ctx *ctx, const fsg_ref *ref, int which, void *out0, void *out1) {
    if (!ctx || !ref || !out0) return set_err(ctx, FSG_ERR_ARG, "NULL argument");
    const RefDev &R = ref->host;
    size_t len = (size_t)ref->len;
    CK(cudaStreamSynchronize(ctx->stream), "sync");
    if (ref->ready) CK(cudaEventSynchronize(ref->ready), "sync reference build");
    if (ref->base && ref->base->ready) CK(cudaEventSynchronize(ref->base->ready), "sync reference build");
    if (which == 0 || which == 1) {
        size_t n = which == 0 ? len : len + 1;
        const double2 *sp = which == 0 ? R.dZndc : R.dZndz;
        const double2 *xm = which == 0 ? R.dZndc_xm : R.dZndz_xm;
        const int *xe = which == 0 ? R.dZndc_xe : R.dZndz_xe;
        if (sp) { CK(cudaMemcpy(out0, sp, 16 * n, cudaMemcpyDeviceToHost), "download path"); return FSG_OK; }
        if (xm && out1) {
            CK(cudaMemcpy(out0, xm, 16 * n, cudaMemcpyDeviceToHost), "download path");
            CK(cudaMemcpy(out1, xe, 4 * n, cudaMemcpyDeviceToHost), "download path");
            return FSG_OK;
        }
        return set_err(ctx, FSG_ERR_ARG, "path not built");
    }
    if (which == 2) {
        if (R.bla_len <= 0 || !out1) return set_err(ctx, FSG_ERR_ARG, "no BLA tree");
        if (R.Mbla) CK(cudaMemcpy(out0, R.Mbla, 32 * (size_t)R.bla_len, cudaMemcpyDeviceToHost), "download BLA");
        else CK(cudaMemcpy(out0, R.Mbla_bs, 64 * (size_t)R.bla_len, cudaMemcpyDeviceToHost), "download BLA");
        CK(cudaMemcpy(out1, R.rbla, 8 * (size_t)R.bla_len, cudaMemcpyDeviceToHost), "download BLA radii");
        return FSG_OK;
    }
    if (which == 3) {
        if (!R.dXa) return set_err(ctx, FSG_ERR_ARG, "no Jacobian paths");
        double *o = (double *)out0;
        CK(cudaMemcpy(o, R.dXa, 8 * len, cudaMemcpyDeviceToHost), "download");
        CK(cudaMemcpy(o + len, R.dXb, 8 * len, cudaMemcpyDeviceToHost), "download");
        CK(cudaMemcpy(o + 2 * len, R.dYa, 8 * len, cudaMemcpyDeviceToHost), "download");
        CK(cudaMemcpy(o + 3 * len, R.dYb, 8 * len, cudaMemcpyDeviceToHost), "download");
        return FSG_OK;
    }
    if (which == 4) {
        if (!R.bs_xpm || !out1) return set_err(ctx, FSG_ERR_ARG, "no Xrange Jacobian paths");
        double *o = (double *)out0;
        int *oe = (int *)out1;
        for (int k = 0; k < 4; k++) {
            CK(cudaMemcpy(o + k * len, R.bs_xpm + k * (len + 1), 8 * len, cudaMemcpyDeviceToHost), "download");
            CK(cudaMemcpy(oe + k * len, R.bs_xpe + k * (len + 1), 4 * len, cudaMemcpyDeviceToHost), "download");
        }
        return FSG_OK;
    }
    return set_err(ctx, FSG_ERR_ARG, "bad table selector");
}

int fsg_std_tiles(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
                  int32_t where) {
    if (ctx) cudaSetDevice(ctx->device);
    return run_tiles(ctx, calc, tiles, ntiles, where, false);
}

int fsg_perturb_tiles(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
                      int32_t where) {
    if (ctx) cudaSetDevice(ctx->device);
    return run_tiles(ctx, calc, tiles, ntiles, where, true);
}

// ---------------------------------------------------------------------------
// post-processing (fsg_postproc.cu)
// ---------------------------------------------------------------------------
int fsg_postproc_fieldlines(fsg_ctx *ctx, const fsg_fieldlines *a, int32_t where) {
    if (!ctx) return FSG_ERR_ARG;
    if (!a || a->npix < 0 || !a->c || !a->z || !a->nu_frac || !a->n || !a->k || !a->phi || !a->out)
        return set_err(ctx, FSG_ERR_ARG, "fieldlines: NULL argument");
    if (a->n_iter < 1 || a->n_iter > FSG_FIELDLINES_MAX_ITER)
        return set_err(ctx, FSG_ERR_LIMIT, "fieldlines: n_iter outside 1 .. FSG_FIELDLINES_MAX_ITER");
    if (a->model < -5 || a->model == 1 || a->model > FSG_MN_MAX_EXP)
        return set_err(ctx, FSG_ERR_ARG, "fieldlines: bad model");
    if (where != FSG_HOST && where != FSG_DEVICE)
        return set_err(ctx, FSG_ERR_ARG, "where must be FSG_HOST or FSG_DEVICE");
    if (a->npix == 0) return FSG_OK;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t n = (size_t)a->npix, nk = (size_t)a->n_iter;
    FieldlinesDev D;
    D.npix = a->npix; D.model = a->model; D.is_backward = a->is_backward;
    D.backshift = a->backshift; D.n_iter = a->n_iter;
    char *p = nullptr;
    if (where == FSG_HOST) {
        size_t bytes = 2 * align_up(16 * n) + 2 * align_up(8 * n) + align_up(4 * n) + 2 * align_up(8 * nk);
        int rc = ensure_scratch(ctx, bytes);
        if (rc != FSG_OK) return rc;
        p = ctx->scratch;
    }
    int rc = FSG_OK;
    if ((rc = stage_in(ctx, where, a->c, 16 * n, p, D.c)) != FSG_OK) return rc;
    if ((rc = stage_in(ctx, where, a->z, 16 * n, p, D.z)) != FSG_OK) return rc;
    if ((rc = stage_in(ctx, where, a->nu_frac, 8 * n, p, D.nu_frac)) != FSG_OK) return rc;
    if ((rc = stage_in(ctx, where, a->n, 4 * n, p, D.n)) != FSG_OK) return rc;
    if ((rc = stage_in(ctx, where, a->k, 8 * nk, p, D.k)) != FSG_OK) return rc;
    if ((rc = stage_in(ctx, where, a->phi, 8 * nk, p, D.phi)) != FSG_OK) return rc;
    D.out = where == FSG_HOST ? (double *)p : a->out;
    fsg_launch_fieldlines(D, ctx->stream);
    CK(cudaGetLastError(), "fieldlines kernel");
    if (where == FSG_HOST) {
        CK(cudaMemcpyAsync(a->out, D.out, 8 * n, cudaMemcpyDeviceToHost, ctx->stream), "copy fieldlines");
        CK(cudaStreamSynchronize(ctx->stream), "fieldlines");
    }
    return FSG_OK;
}

int fsg_postproc_normal(fsg_ctx *ctx, const fsg_normal *a, int32_t where) {
    if (!ctx) return FSG_ERR_ARG;
    if (!a || a->npix < 0 || !a->zn || !a->dzndc || !a->out || (a->kind == 1 && !a->d2zndc2))
        return set_err(ctx, FSG_ERR_ARG, "normal: NULL argument");
    if (a->kind < 0 || a->kind > 2) return set_err(ctx, FSG_ERR_ARG, "normal: bad kind");
    if (where != FSG_HOST && where != FSG_DEVICE)
        return set_err(ctx, FSG_ERR_ARG, "where must be FSG_HOST or FSG_DEVICE");
    if (a->npix == 0) return FSG_OK;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t n = (size_t)a->npix;
    NormalDev D;
    D.npix = a->npix; D.kind = a->kind;
    D.has_skew = a->skew != nullptr;
    for (int k = 0; k < 4; k++) D.skew[k] = a->skew ? a->skew[k] : 0.;
    D.dzndc = nullptr; D.jac = nullptr; D.d2 = nullptr;
    const size_t dbytes = a->kind == 2 ? 32 * n : 16 * n;
    char *p = nullptr;
    if (where == FSG_HOST) {
        size_t bytes = align_up(16 * n) + align_up(dbytes) + (a->kind == 1 ? align_up(16 * n) : 0)
                       + align_up(16 * n);
        int rc = ensure_scratch(ctx, bytes);
        if (rc != FSG_OK) return rc;
        p = ctx->scratch;
    }
    int rc = FSG_OK;
    if ((rc = stage_in(ctx, where, a->zn, 16 * n, p, D.zn)) != FSG_OK) return rc;
    if (a->kind == 2) {
        if ((rc = stage_in(ctx, where, a->dzndc, dbytes, p, D.jac)) != FSG_OK) return rc;
    } else if ((rc = stage_in(ctx, where, a->dzndc, dbytes, p, D.dzndc)) != FSG_OK) {
        return rc;
    }
    if (a->kind == 1 && (rc = stage_in(ctx, where, a->d2zndc2, 16 * n, p, D.d2)) != FSG_OK) return rc;
    D.out = where == FSG_HOST ? (double2 *)p : (double2 *)a->out;
    fsg_launch_normal(D, ctx->stream);
    CK(cudaGetLastError(), "normal kernel");
    if (where == FSG_HOST) {
        CK(cudaMemcpyAsync(a->out, D.out, 16 * n, cudaMemcpyDeviceToHost, ctx->stream), "copy normal");
        CK(cudaStreamSynchronize(ctx->stream), "normal");
    }
    return FSG_OK;
}

int fsg_peak_flops(fsg_ctx *ctx, int32_t fp64, double *tflops) {
    if (!ctx || !tflops) return FSG_ERR_ARG;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    void *out = nullptr;
    CK(cudaMalloc(&out, (size_t)ctx->sm_count * 8 * 256 * 8), "cudaMalloc(peak)");
    cudaEvent_t a, b;
    cudaEventCreate(&a); cudaEventCreate(&b);
    double best = 0.;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(a, ctx->stream);
        double flops = fsg_launch_fma_peak(fp64, ctx->sm_count, out, ctx->stream);
        cudaEventRecord(b, ctx->stream);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (rep > 0 && ms > 0.f) { double t = flops / (ms * 1e-3) / 1e12; if (t > best) best = t; }
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a); cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return cuda_err(ctx, e, "peak kernel");
    *tflops = best;
    return FSG_OK;
}

int fsg_last_stats(const fsg_ctx *cctx, fsg_stats *out) {
    fsg_ctx *ctx = const_cast<fsg_ctx *>(cctx);
    if (!ctx || !out) return FSG_ERR_ARG;
    memset(out, 0, sizeof(*out));
    if (!ctx->timed) return FSG_OK;
    CK(cudaEventSynchronize(ctx->ev1), "cudaEventSynchronize");
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "cudaEventElapsedTime");
    unsigned long long st[4];
    CK(cudaMemcpy(st, ctx->stats_dev, sizeof(st), cudaMemcpyDeviceToHost), "read stats");
    out->kernel_ms = ms;
    out->pixels = ctx->last_pixels;
    out->pixel_iters = (int64_t)st[0];
    out->full_steps = (int64_t)st[1];
    out->bla_steps = (int64_t)st[2];
    out->rebases = (int64_t)st[3];
    return FSG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Serving queue.  Requests of host-buffer tiles are queued, admitted when a
// launch slot is free and their staged device buffers fit in the HBM budget,
// and run on the slots' own streams, so that several overlap on the device.
// A slot owns its stream, work counter, statistics, budget and status words
// and descriptor staging; a request's device buffers are one stream-ordered
// allocation on its slot's stream, released when its results are back.
// ---------------------------------------------------------------------------
struct ServeSlot {
    cudaStream_t stream = nullptr;
    TileDev *tiles_host = nullptr; long long *start_host = nullptr;
    TileDev *tiles_dev = nullptr; long long *start_dev = nullptr;
    unsigned long long *words = nullptr;   // counter, stats[4], used
    int *status_dev = nullptr;
    cudaEvent_t done = nullptr;
    int64_t ticket = -1;                   // running request, -1 when free
};

struct ServeReq {
    fsg_calc calc;
    std::vector<fsg_tile> tiles;
    std::vector<TileDev> td;
    bool perturb = false;
    bool inplace = false;                  // page-locked buffers: no staging, no copy-back
    double work = 0.;
    double submitted = 0., started = 0.;   // steady-clock seconds
    size_t bytes = 0;
    int state = 0;                         // 0 queued, 1 running, 2 done
    int rc = FSG_OK;
    void *block = nullptr;
    int slot = -1;
};

struct ServeState {
    std::mutex m;
    int64_t budget = 0;
    int order = FSG_SERVE_FIFO;
    std::vector<ServeSlot> slots;
    std::map<int64_t, ServeReq> reqs;
    int64_t next = 1;
    int64_t reserved = 0, peak = 0;
    int64_t queued = 0, running = 0;
    double rate = 0.;                      // expected work per second of a slot
};

double steady_seconds() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

namespace {

void serve_free_slots(ServeState *S) {
    for (ServeSlot &sl : S->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.tiles_host) cudaFreeHost(sl.tiles_host);
        if (sl.start_host) cudaFreeHost(sl.start_host);
        if (sl.tiles_dev) cudaFree(sl.tiles_dev);
        if (sl.start_dev) cudaFree(sl.start_dev);
        if (sl.words) cudaFree(sl.words);
        if (sl.status_dev) cudaFree(sl.status_dev);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    S->slots.clear();
}

// Start a queued request on slot k (the caller holds the lock).  A failure
// marks the request done with its error code.
void serve_start(fsg_ctx *ctx, ServeState *S, int k, int64_t ticket, ServeReq &R) {
    ServeSlot &sl = S->slots[k];
    R.state = 1; R.slot = k; sl.ticket = ticket;
    R.started = steady_seconds();
    S->queued--; S->running++;
    S->reserved += (int64_t)R.bytes;
    if (S->reserved > S->peak) S->peak = S->reserved;
    int rc = FSG_OK;
    cudaError_t e = cudaSuccess;
    if (!R.inplace) {
        e = cudaMallocAsync(&R.block, R.bytes, sl.stream);
        if (e != cudaSuccess) rc = cuda_err(ctx, e, "cudaMallocAsync(request)");
    }
    if (rc == FSG_OK) rc = wait_references(ctx, R.tiles.data(), (int32_t)R.tiles.size(), sl.stream);
    if (rc == FSG_OK && !R.inplace) {
        R.td.resize(R.tiles.size());
        rc = stage_tiles(ctx, &R.calc, R.tiles.data(), (int32_t)R.tiles.size(), (char *)R.block,
                         sl.stream, R.td.data());
    }
    if (rc == FSG_OK) {
        LaunchRes L;
        L.stream = sl.stream;
        L.tiles_host = sl.tiles_host; L.start_host = sl.start_host;
        L.tiles_dev = sl.tiles_dev; L.start_dev = sl.start_dev;
        L.counter_dev = sl.words; L.stats_dev = sl.words + 1; L.used_dev = sl.words + 5;
        L.status_dev = sl.status_dev;
        // the slot's staging is reused only after its request has retired
        L.ev_desc = nullptr; L.ev0 = nullptr; L.ev1 = nullptr;
        const Segment whole = {0, tiles_pixels(R.td.data(), (int)R.td.size()), true, true};
        rc = launch_on(ctx, L, &R.calc, R.td.data(), (int)R.td.size(), R.perturb, whole);
    }
    if (rc == FSG_OK) {
        e = cudaEventRecord(sl.done, sl.stream);
        if (e != cudaSuccess) rc = cuda_err(ctx, e, "cudaEventRecord(request)");
    }
    if (rc != FSG_OK) {
        cudaStreamSynchronize(sl.stream);
        if (R.block) cudaFreeAsync(R.block, sl.stream);
        R.block = nullptr;
        S->reserved -= (int64_t)R.bytes;
        S->running--;
        sl.ticket = -1;
        R.state = 2; R.rc = rc;
    }
}

// Retire finished requests: results into the caller's buffers (unless the
// launch was interrupted), device buffers released.
void serve_retire(fsg_ctx *ctx, ServeState *S) {
    for (ServeSlot &sl : S->slots) {
        if (sl.ticket < 0) continue;
        if (cudaEventQuery(sl.done) != cudaSuccess) continue;
        ServeReq &R = S->reqs[sl.ticket];
        int st = 0, rc = FSG_OK;
        cudaError_t e = cudaMemcpyAsync(&st, sl.status_dev, sizeof(int), cudaMemcpyDeviceToHost,
                                        sl.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(sl.stream);
        if (e != cudaSuccess) rc = cuda_err(ctx, e, "read request status");
        const int launch_rc = st == 1 ? FSG_INTERRUPTED : (st == 2 ? FSG_BUDGET : FSG_OK);
        if (rc == FSG_OK && launch_rc != FSG_INTERRUPTED && !R.inplace) {
            rc = copy_back(ctx, &R.calc, R.tiles.data(), (int32_t)R.tiles.size(), R.td.data(),
                           sl.stream);
            if (rc == FSG_OK) {
                e = cudaStreamSynchronize(sl.stream);
                if (e != cudaSuccess) rc = cuda_err(ctx, e, "copy request back");
            }
        }
        if (R.block) cudaFreeAsync(R.block, sl.stream);
        R.block = nullptr;
        S->reserved -= (int64_t)R.bytes;
        S->running--;
        R.state = 2;
        R.rc = rc == FSG_OK ? launch_rc : rc;
        sl.ticket = -1;
        // the work rate of one slot, averaged over the finished requests
        const double dt = steady_seconds() - R.started;
        if (dt > 0.) S->rate = S->rate == 0. ? R.work / dt : 0.8 * S->rate + 0.2 * R.work / dt;
    }
}

// Admit queued requests in the configured order while a slot is free and the
// next request fits in the budget (the next one waits: no overtaking).
void serve_admit(fsg_ctx *ctx, ServeState *S) {
    for (;;) {
        int k = -1;
        for (int i = 0; i < (int)S->slots.size(); i++)
            if (S->slots[i].ticket < 0) { k = i; break; }
        if (k < 0) return;
        // FIFO: the oldest ticket; SHORTEST: the least expected work; HRRN:
        // the highest response ratio (wait + S) / S, S = work / rate (the
        // least work while no request has finished yet)
        int64_t best = -1;
        double best_key = 0.;
        const bool hrrn = S->order == FSG_SERVE_HRRN && S->rate > 0.;
        const double now = hrrn ? steady_seconds() : 0.;
        for (auto &kv : S->reqs) {
            if (kv.second.state != 0) continue;
            double key = kv.second.work;
            if (hrrn) {
                const double sv = kv.second.work / S->rate;
                key = -(now - kv.second.submitted + sv) / sv;
            }
            if (best < 0) {
                best = kv.first; best_key = key;
                if (S->order == FSG_SERVE_FIFO) break;
                continue;
            }
            if (key < best_key) { best = kv.first; best_key = key; }
        }
        if (best < 0) return;
        ServeReq &R = S->reqs[best];
        if (S->reserved + (int64_t)R.bytes > S->budget) return;
        serve_start(ctx, S, k, best, R);
    }
}

}  // namespace

extern "C" {

int fsg_serve_open(fsg_ctx *ctx, int64_t hbm_budget_bytes, int32_t slots, int32_t order) {
    if (!ctx) return FSG_ERR_ARG;
    if (ctx->serve) return set_err(ctx, FSG_ERR_ARG, "the serving queue is already open");
    if (hbm_budget_bytes <= 0 || slots <= 0 || slots > 64)
        return set_err(ctx, FSG_ERR_ARG, "serving: budget > 0 and 1 .. 64 slots");
    if (order != FSG_SERVE_FIFO && order != FSG_SERVE_SHORTEST && order != FSG_SERVE_HRRN)
        return set_err(ctx, FSG_ERR_ARG,
                       "serving: order FSG_SERVE_FIFO, FSG_SERVE_SHORTEST or FSG_SERVE_HRRN");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    ServeState *S = new (std::nothrow) ServeState();
    if (!S) return set_err(ctx, FSG_ERR_NOMEM, "out of host memory");
    S->budget = hbm_budget_bytes; S->order = order;
    S->slots.resize(slots);
    const size_t nt = FSG_MAX_TILES_PER_LAUNCH;
    for (ServeSlot &sl : S->slots) {
        cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMallocHost((void **)&sl.tiles_host, sizeof(TileDev) * nt);
        if (e == cudaSuccess) e = cudaMallocHost((void **)&sl.start_host, sizeof(long long) * (nt + 1));
        if (e == cudaSuccess) e = cudaMalloc((void **)&sl.tiles_dev, sizeof(TileDev) * nt);
        if (e == cudaSuccess) e = cudaMalloc((void **)&sl.start_dev, sizeof(long long) * (nt + 1));
        if (e == cudaSuccess) e = cudaMalloc((void **)&sl.words, 6 * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMalloc((void **)&sl.status_dev, sizeof(int));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            serve_free_slots(S);
            delete S;
            return cuda_err(ctx, e, "serving slot");
        }
    }
    ctx->serve = S;
    return FSG_OK;
}

int fsg_submit(fsg_ctx *ctx, const fsg_calc *calc, const fsg_tile *tiles, int32_t ntiles,
               double expected_work, int64_t *ticket) {
    if (!ctx || !ticket) return FSG_ERR_ARG;
    *ticket = 0;
    ServeState *S = ctx->serve;
    if (!S) return set_err(ctx, FSG_ERR_ARG, "fsg_serve_open first");
    if (!calc || !tiles || ntiles <= 0) return set_err(ctx, FSG_ERR_ARG, "no tiles");
    if (ntiles > FSG_MAX_TILES_PER_LAUNCH)
        return set_err(ctx, FSG_ERR_LIMIT, "more tiles than one launch takes");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const bool perturb = tiles[0].ref != nullptr;
    for (int32_t i = 1; i < ntiles; i++)
        if ((tiles[i].ref != nullptr) != perturb)
            return set_err(ctx, FSG_ERR_ARG, "a request mixes perturbation and standard tiles");
    int rc = check_calc_tiles(ctx, calc, tiles, ntiles, perturb);
    if (rc != FSG_OK) return rc;
    // page-locked buffers are written in place: nothing staged on the device
    std::vector<TileDev> pinned_td(ntiles);
    const bool inplace = pinned_tiles(tiles, ntiles, pinned_td.data());
    const size_t bytes = inplace ? 0 : staged_bytes(calc, tiles, ntiles);
    std::lock_guard<std::mutex> lock(S->m);
    if ((int64_t)bytes > S->budget)
        return set_err(ctx, FSG_ERR_LIMIT, "request larger than the serving budget");
    const int64_t t = S->next++;
    ServeReq &R = S->reqs[t];
    R.calc = *calc;
    R.tiles.assign(tiles, tiles + ntiles);
    R.perturb = perturb;
    long long px = 0;
    for (int32_t i = 0; i < ntiles; i++) px += (long long)tiles[i].nx * tiles[i].ny;
    R.work = expected_work > 0. ? expected_work : (double)px;
    R.submitted = steady_seconds();
    R.bytes = bytes;
    R.inplace = inplace;
    if (inplace) R.td = std::move(pinned_td);
    S->queued++;
    serve_retire(ctx, S);
    serve_admit(ctx, S);
    *ticket = t;
    return FSG_OK;
}

int fsg_poll(fsg_ctx *ctx, int64_t ticket) {
    if (!ctx) return FSG_ERR_ARG;
    ServeState *S = ctx->serve;
    if (!S) return set_err(ctx, FSG_ERR_ARG, "fsg_serve_open first");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    std::lock_guard<std::mutex> lock(S->m);
    serve_retire(ctx, S);
    serve_admit(ctx, S);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return set_err(ctx, FSG_ERR_ARG, "unknown ticket");
    if (it->second.state != 2) return FSG_PENDING;
    const int rc = it->second.rc;
    S->reqs.erase(it);
    return rc;
}

int fsg_serve_info(fsg_ctx *ctx, fsg_serve_stats *out) {
    if (!ctx || !out) return FSG_ERR_ARG;
    ServeState *S = ctx->serve;
    if (!S) return set_err(ctx, FSG_ERR_ARG, "fsg_serve_open first");
    std::lock_guard<std::mutex> lock(S->m);
    out->queued = S->queued; out->running = S->running;
    out->reserved_bytes = S->reserved; out->peak_reserved_bytes = S->peak;
    out->budget_bytes = S->budget; out->slots = (int32_t)S->slots.size();
    return FSG_OK;
}

int fsg_serve_close(fsg_ctx *ctx) {
    if (!ctx) return FSG_ERR_ARG;
    ServeState *S = ctx->serve;
    if (!S) return FSG_OK;
    cudaSetDevice(ctx->device);
    {
        std::lock_guard<std::mutex> lock(S->m);
        for (ServeSlot &sl : S->slots)
            if (sl.stream) cudaStreamSynchronize(sl.stream);
        serve_retire(ctx, S);
        serve_free_slots(S);
    }
    delete S;
    ctx->serve = nullptr;
    return FSG_OK;
}

}  // extern "C"
