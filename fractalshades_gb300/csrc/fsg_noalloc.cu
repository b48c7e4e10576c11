// fsg_noalloc.cu -- the standard escape-time loop for callers that cannot
// allocate GPU memory.
//
// Some callers of this library cannot call cudaMalloc: their device memory is
// entirely reserved up front by another allocator (a framework's caching
// allocator, an application that pre-allocates a fixed GPU budget at start-up
// and treats any later allocation as an error), or they run inside a frame
// loop where the implicit device synchronisation of cudaMalloc / cudaFree is
// not acceptable.  fsg_std_tiles needs a context (fsg_ctx_create) whose
// work counter, statistics and tile descriptors live in memory it allocates.
// fsg_std_tiles_noalloc runs the same kernel with that scratch held in a
// file-scope __device__ array instead, so it allocates nothing: the caller
// passes device pointers for every input and output.
//
// Limits and sharing (also stated in include/fsgpu.h):
//   * at most FSG_NOALLOC_MAX_TILES tiles per call, else FSG_ERR_LIMIT;
//   * the array is one per device, is held until the process exits, and every
//     call shares it: the work counter and statistics are cleared at the start
//     of each call, the descriptors overwritten; calls whose launches overlap
//     on the GPU (other streams, other host threads) race on it;
//   * the first call on a device resolves the array's device address with that
//     device current (cudaGetSymbolAddress); make that first call before any
//     stream capture.
// The descriptors reach the array as the parameter of a small upload kernel
// launched on the caller's stream (about 17 KB, inside the 32 KB parameter
// limit), so no host-to-device copy from the caller's stack is involved and
// the call never waits for the stream.
#include <cstddef>
#include <cstring>
#include <mutex>

#include "fsg_internal.cuh"
#include "../../include/fsgpu.h"

namespace {

struct NoallocScratch {
    unsigned long long counter;
    unsigned long long stats[4];
    int status;
    int cancel;                      // stays 0: this entry point is not cancellable
    long long start[FSG_NOALLOC_MAX_TILES + 1];
    TileDev tiles[FSG_NOALLOC_MAX_TILES];
};

// What the upload kernel receives by value: the tile offsets and descriptors
struct NoallocUpload {
    long long start[FSG_NOALLOC_MAX_TILES + 1];
    TileDev tiles[FSG_NOALLOC_MAX_TILES];
    int ntiles;
};
static_assert(sizeof(NoallocUpload) <= 32000, "upload parameter beyond the kernel parameter limit");
static_assert(sizeof(TileDev) % 8 == 0, "descriptors are copied as 8-byte words");

}  // namespace

static __device__ __align__(256) unsigned char fsg_noalloc_scratch[sizeof(NoallocScratch)];

// Clears the counter, statistics, status and cancel words and copies the
// call's descriptors into the array (device code names the array directly).
static __global__ void __launch_bounds__(256) k_noalloc_upload(const NoallocUpload u) {
    NoallocScratch *S = reinterpret_cast<NoallocScratch *>(fsg_noalloc_scratch);
    if (threadIdx.x == 0) {
        S->counter = 0ULL;
        for (int k = 0; k < 4; k++) S->stats[k] = 0ULL;
        S->status = 0;
        S->cancel = 0;
    }
    for (int i = threadIdx.x; i <= u.ntiles; i += blockDim.x) S->start[i] = u.start[i];
    const int words = u.ntiles * (int)(sizeof(TileDev) / 8);
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(u.tiles);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(S->tiles);
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
}

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
NoallocScratch *g_addr[kMaxDevices] = {nullptr};

// Device address of the array on the current device (set-up on first use).
cudaError_t scratch_address(int device, NoallocScratch **out) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, fsg_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[device] = (NoallocScratch *)p;
    }
    *out = g_addr[device];
    return cudaSuccess;
}

}  // namespace

extern "C" int fsg_std_tiles_noalloc(const fsg_calc *calc, const fsg_tile *tiles,
                                     int32_t ntiles, void *stream) {
    if (!calc || !tiles || ntiles <= 0) return FSG_ERR_ARG;
    if (ntiles > FSG_NOALLOC_MAX_TILES) return FSG_ERR_LIMIT;
    if (calc->max_iter <= 0 || calc->max_iter > FSG_MAX_ITER_LIMIT) return FSG_ERR_ARG;
    if (calc->flavor < 0 || calc->flavor > 5) return FSG_ERR_ARG;
    if (calc->nexp != 0 && (calc->flavor != 0 || calc->nexp < 2)) return FSG_ERR_ARG;
    if (calc->nexp > FSG_MN_MAX_EXP) return FSG_ERR_LIMIT;
    if (calc->backshift != 0 || calc->calc_d2zndc2 != 0) return FSG_ERR_ARG;  // fsg_std_tiles
    if (calc->iter_budget != 0) return FSG_ERR_ARG;     // no budget counter in the array
    const int nZ_min = calc->flavor == 0 ? 3 : 6;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return FSG_ERR_NODEV;
    if (device < 0 || device >= kMaxDevices) return FSG_ERR_LIMIT;
    NoallocScratch *S = nullptr;
    if (scratch_address(device, &S) != cudaSuccess) return FSG_ERR_CUDA;

    NoallocUpload host;             // the upload kernel's parameter
    host.ntiles = ntiles;
    long long total = 0;
    host.start[0] = 0;
    for (int32_t i = 0; i < ntiles; i++) {
        const fsg_tile &t = tiles[i];
        if (t.nx <= 0 || t.ny <= 0 || t.nZ < nZ_min || !t.Z || !t.stop_reason || !t.stop_iter
            || (!t.pix && (!t.xs || !t.ys)) || t.proj != 0)
            return FSG_ERR_ARG;
        TileDev &d = host.tiles[i];
        memset(&d, 0, sizeof(d));
        d.xs = t.xs; d.ys = t.ys; d.pix = (const double2 *)t.pix;
        d.nx = t.nx; d.ny = t.ny;
        for (int k = 0; k < 4; k++) d.lin[k] = t.lin_mat[k];
        d.cre = t.center_re; d.cim = t.center_im; d.dx = t.dx;
        d.Z = t.Z; d.nZ = t.nZ;
        d.stop_reason = (signed char *)t.stop_reason; d.stop_iter = t.stop_iter;
        d.pot = t.potential; d.dem = t.dem;
        total += (long long)t.nx * t.ny;
        host.start[i + 1] = total;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // An error left pending by the caller's earlier CUDA work on this thread
    // is consumed here, so that the status below reports this call's own
    // launches only.
    (void)cudaGetLastError();
    // counter, statistics, status and cancel word cleared, descriptors
    // copied: the launch carries them as its parameter
    k_noalloc_upload<<<1, 256, 0, s>>>(host);
    if (cudaGetLastError() != cudaSuccess) return FSG_ERR_CUDA;
    WorkDev W;
    W.tiles = S->tiles; W.start = S->start; W.ntiles = ntiles; W.base = 0; W.total = total;
    W.order = nullptr;
    W.counter = &S->counter; W.stats = S->stats;
    W.cancel = &S->cancel; W.status = &S->status;
    W.budget = 0ULL; W.used = nullptr;
    CalcDev C;
    C.max_iter = (int)calc->max_iter;
    C.M2 = calc->M_divergence * calc->M_divergence;
    C.eps2 = calc->epsilon_stationnary * calc->epsilon_stationnary;
    C.logM = log(calc->M_divergence);
    C.mode = FSG_MODE_FP64; C.calc_dzndc = 1; C.interior = 0; C.bla = 0;
    C.flavor = calc->flavor; C.xrsem = 0;
    C.nexp = calc->nexp; C.logd = log(calc->nexp ? (double)calc->nexp : 2.);
    C.backshift = 0; C.d2 = 0;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return FSG_ERR_CUDA;
    const int block = 256;
    long long need = (total + block - 1) / block;
    int grid = sms * 2;
    if (need < grid) grid = (int)need;
    fsg_launch_std(W, C, grid, block, s);
    return cudaGetLastError() == cudaSuccess ? FSG_OK : FSG_ERR_CUDA;
}
