// fsg_perturb_bs32.cu -- the Burning Ship family perturbation loop with
// FP32-mantissa + int32-exponent deltas: fsg_bs.cuh instantiated on fr
// (the reference's loop, perturbation.py:1468-1811, in that arithmetic).
#include "fsg_bs.cuh"

template __global__ void k_perturb_bs<fr>(WorkDev W, CalcDev C);

void fsg_launch_perturb_bs_fe32(const WorkDev &W, const CalcDev &C, int grid, int block,
                                cudaStream_t s) {
    k_perturb_bs<fr><<<fsg_auto_grid(k_perturb_bs<fr>, grid, block, W.total), block, 0, s>>>(W, C);
}
