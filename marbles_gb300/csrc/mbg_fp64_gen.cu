// mbg_fp64_gen.cu -- the FP64 step kernels through the general pull (mode 0
// of mbg_fp64_step.cuh), in a unit of their own so that the parallel build
// compiles them beside the other modes.  Compiled with -fmad=false, as
// every FP64 unit.
#include "mbg_fp64_step.cuh"

namespace mbg {

void launch_moments_gen(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                        const double* fAg, const double* gAg, const double* fB, const double* gB, double* md,
                        cudaStream_t s)
{
    if (lp.ngen > 0)
        k_moments<0><<<lp.ngen, TILE_CELLS, 0, s>>>(lp.view64, lp, P, ph, lp.gen_tiles, fA, gA, fAg, gAg, fB, gB,
                                                   md);
}

void launch_collide_gen(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                        const double* fAg, const double* gAg, double* fB, double* gB, const double* md,
                        const double* gqc, cudaStream_t s)
{
    if (lp.ngen > 0)
        k_collide<0><<<lp.ngen, TILE_CELLS, 0, s>>>(lp.view64, lp, P, ph, lp.gen_tiles, fA, gA, fAg, gAg, fB, gB, md,
                                                   gqc);
}

}  // namespace mbg
