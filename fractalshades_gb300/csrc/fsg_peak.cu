// fsg_peak.cu -- FMA-pipe throughput microbenchmark: the roofline
// denominator of the iteration kernels, which are bound by the FP32 (fast
// form) or FP64 (reference forms) FMA pipes, not by HBM or tensor cores.
// Each thread runs 8 independent FMA chains; the result is written so that
// the chains are not eliminated.
#include "fsg_internal.cuh"

template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(T *out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
            x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
        }
    }
    T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)-12345) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// returns flops per launch; the caller times the launch
double fsg_launch_fma_peak(int fp64, int sm_count, void *out, cudaStream_t s) {
    const int block = 256;
    const int grid = sm_count * 8;
    const int iters = fp64 ? 64 : 2048;
    if (fp64) k_fma_peak<double><<<grid, block, 0, s>>>((double *)out, iters, 0.999999, 1e-7);
    else k_fma_peak<float><<<grid, block, 0, s>>>((float *)out, iters, 0.999999f, 1e-7f);
    return 2.0 * 8 * 16 * (double)iters * grid * block;
}
