// mbg_fp64_bc.cu -- the FP64 moment pass of boxes within one cell of a
// non-periodic side (modes 3 and 4 of mbg_fp64_step.cuh; the collision pass
// is in mbg_fp64_bcc.cu), in a unit of its own so that the parallel build
// compiles it beside the other modes.  Compiled with -fmad=false, as every
// FP64 unit.
#include "mbg_fp64_step.cuh"

namespace mbg {

void launch_moments_bc(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                       const double* fAg, const double* gAg, const double* fB, const double* gB, double* md,
                       cudaStream_t s)
{
    const size_t sb = slot_bytes(lp);
    const LV& L = lp.view64;
    if (lp.nfastbc > 0)
        k_moments<3><<<lp.nfastbc, TILE_CELLS, sb, s>>>(L, lp, P, ph, lp.fastbc_tiles, fA, gA, fAg, gAg, fB, gB, md);
    if (lp.nfastebbc > 0)
        k_moments<4><<<lp.nfastebbc, TILE_CELLS, sb, s>>>(L, lp, P, ph, lp.fastebbc_tiles, fA, gA, fAg, gAg, fB, gB,
                                                          md);
}

}  // namespace mbg
