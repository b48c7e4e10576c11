// fsg_lpt.cu -- the claim order of a perturbation launch, longest pixels first.
//
// A persistent launch ends when its last pixels do: on an escape-dominated
// view the pixels claimed last include some that iterate 10-100 times longer
// than the median, and the GPU idles while they finish (on a 1024^2 view of
// the seahorse valley a quarter of the launch).  The order built here claims
// them first: a pre-pass iterates one representative pixel per 8 x 8 block of
// each tile (the block's centre) with max_iter capped (so that the pre-pass's
// own tail stays short), the blocks are bucketed by the representative's
// iteration count (log2 buckets, counting sort on the device), and the main
// pass claims every pixel of the image, the blocks in decreasing order of that
// count.  The main pass rewrites the representatives' outputs; a pixel's
// outputs do not depend on when it is claimed.
#include "fsg_internal.cuh"

#define LPT_SIDE 8
#define LPT_BUCKETS 32

// block b of the launch: its tile t (binary search in the per-tile prefix of
// block counts) and its pixel rectangle [x0, x0 + bw) x [y0, y0 + bh)
__device__ __forceinline__ void lpt_block(const TileDev *tiles, const int *blk_start, int ntiles,
                                          int b, int &t, int &x0, int &y0, int &bw, int &bh) {
    int lo = 0, hi = ntiles - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (blk_start[mid] <= b) lo = mid; else hi = mid - 1;
    }
    t = lo;
    const int nx = tiles[t].nx, ny = tiles[t].ny;
    const int nbx = (nx + LPT_SIDE - 1) / LPT_SIDE;
    const int lb = b - blk_start[t];
    x0 = (lb % nbx) * LPT_SIDE; y0 = (lb / nbx) * LPT_SIDE;
    bw = min(LPT_SIDE, nx - x0); bh = min(LPT_SIDE, ny - y0);
}

// per-tile prefix of the 8 x 8 block counts (one thread: at most
// FSG_MAX_TILES_PER_LAUNCH tiles)
static __global__ void k_lpt_blocks(const TileDev *tiles, int ntiles, int *blk_start,
                                    unsigned *hist) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int acc = 0;
        blk_start[0] = 0;
        for (int t = 0; t < ntiles; t++) {
            acc += ((tiles[t].nx + LPT_SIDE - 1) / LPT_SIDE) * ((tiles[t].ny + LPT_SIDE - 1) / LPT_SIDE);
            blk_start[t + 1] = acc;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < LPT_BUCKETS) hist[threadIdx.x] = 0;
}

// the representative (centre) pixel of every block, as a claim order
static __global__ void k_lpt_reps(const TileDev *tiles, const long long *start,
                                  const int *blk_start, int ntiles, int nblk, unsigned *rep) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    int t, x0, y0, bw, bh;
    lpt_block(tiles, blk_start, ntiles, b, t, x0, y0, bw, bh);
    rep[b] = (unsigned)(start[t] + (long long)(y0 + bh / 2) * tiles[t].nx + (x0 + bw / 2));
}

// bucket of each block (decreasing log2 of the representative's iteration
// count) and the bucket sizes in pixels; the representative is marked not
// run again (stop_reason -1) until the main pass computes it in full
static __global__ void k_lpt_hist(const TileDev *tiles, const long long *start,
                                  const int *blk_start, int ntiles, int nblk,
                                  const unsigned *rep, unsigned char *bucket, unsigned *hist) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    int t, x0, y0, bw, bh;
    lpt_block(tiles, blk_start, ntiles, b, t, x0, y0, bw, bh);
    const long long ip = rep[b] - start[t];
    const int n = max(tiles[t].stop_iter[ip], 0);
    tiles[t].stop_reason[ip] = -1;
    const int k = (LPT_BUCKETS - 1) - (31 - __clz(n + 1));     // 0: the longest
    bucket[b] = (unsigned char)k;
    atomicAdd(&hist[k], (unsigned)(bw * bh));
}

// bucket offsets (exclusive prefix, longest bucket first)
static __global__ void k_lpt_scan(unsigned *hist) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        unsigned acc = 0;
        for (int k = 0; k < LPT_BUCKETS; k++) {
            const unsigned c = hist[k];
            hist[k] = acc;
            acc += c;
        }
    }
}

// the pixels of every block at its bucket's next free place
static __global__ void k_lpt_scatter(const TileDev *tiles, const long long *start,
                                     const int *blk_start, int ntiles, int nblk,
                                     const unsigned char *bucket, unsigned *cursor,
                                     unsigned *order) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    int t, x0, y0, bw, bh;
    lpt_block(tiles, blk_start, ntiles, b, t, x0, y0, bw, bh);
    unsigned pos = atomicAdd(&cursor[bucket[b]], (unsigned)(bw * bh));
    const int nx = tiles[t].nx;
    const long long base = start[t];
    for (int y = 0; y < bh; y++)
        for (int x = 0; x < bw; x++)
            order[pos++] = (unsigned)(base + (long long)(y0 + y) * nx + (x0 + x));
}

int fsg_lpt_blocks_count(const int *nx, const int *ny, int ntiles) {
    int acc = 0;
    for (int t = 0; t < ntiles; t++)
        acc += ((nx[t] + LPT_SIDE - 1) / LPT_SIDE) * ((ny[t] + LPT_SIDE - 1) / LPT_SIDE);
    return acc;
}

// Before the pre-pass: block prefix and representatives (the device copies
// of the tile descriptors and pixel offsets must be in place on stream s).
// Scratch: blk_start [ntiles + 1], hist [LPT_BUCKETS], rep [nblk].
void fsg_lpt_prepare(const TileDev *tiles, const long long *start, int ntiles, int nblk,
                     int *blk_start, unsigned *hist, unsigned *rep, cudaStream_t s) {
    k_lpt_blocks<<<1, 32, 0, s>>>(tiles, ntiles, blk_start, hist);
    k_lpt_reps<<<(nblk + 255) / 256, 256, 0, s>>>(tiles, start, blk_start, ntiles, nblk, rep);
}

// After the pre-pass: the main pass's order [total] from the
// representatives' iteration counts.  Scratch: bucket [nblk].
void fsg_lpt_order(const TileDev *tiles, const long long *start, int ntiles, int nblk,
                   const int *blk_start, unsigned *hist, const unsigned *rep,
                   unsigned char *bucket, unsigned *order, cudaStream_t s) {
    const int g = (nblk + 255) / 256;
    k_lpt_hist<<<g, 256, 0, s>>>(tiles, start, blk_start, ntiles, nblk, rep, bucket, hist);
    k_lpt_scan<<<1, 32, 0, s>>>(hist);
    k_lpt_scatter<<<g, 256, 0, s>>>(tiles, start, blk_start, ntiles, nblk, bucket, hist, order);
}
