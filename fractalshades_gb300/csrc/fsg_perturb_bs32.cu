// fsg_perturb_bs32.cu -- the Burning Ship family perturbation loop with
// FP32-mantissa + int32-exponent deltas: fsg_bs.cuh instantiated on fr
// (the reference's loop, perturbation.py:1468-1811, in that arithmetic), one
// kernel per flavor so that the closures' flavor branches fold.
#include "fsg_bs.cuh"

template <int FL>
static void launch_bs_fr(const WorkDev &W, const CalcDev &C, int grid, int block, cudaStream_t s) {
    const size_t sm = fsg_starts_smem(W);
    k_perturb_bs<fr, FL><<<fsg_auto_grid(k_perturb_bs<fr, FL>, grid, block, W.total - W.base, sm),
                           block, sm, s>>>(W, C);
}

void fsg_launch_perturb_bs_fe32(const WorkDev &W, const CalcDev &C, int grid, int block,
                                cudaStream_t s) {
    switch (C.flavor) {
    case 1: launch_bs_fr<1>(W, C, grid, block, s); break;
    case 2: launch_bs_fr<2>(W, C, grid, block, s); break;
    case 3: launch_bs_fr<3>(W, C, grid, block, s); break;
    case 4: launch_bs_fr<4>(W, C, grid, block, s); break;
    default: launch_bs_fr<5>(W, C, grid, block, s); break;
    }
}
