// mbg_fp64_bcc.cu -- the FP64 collision pass of boxes within one cell of a
// non-periodic side (modes 3 and 4 of mbg_fp64_step.cuh), in a unit of its
// own so that the parallel build compiles it beside the other modes.
// Compiled with -fmad=false, as every FP64 unit.
#include "mbg_fp64_step.cuh"

namespace mbg {

void launch_collide_bc(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                       const double* fAg, const double* gAg, double* fB, double* gB, const double* md,
                       const double* gqc, cudaStream_t s)
{
    const size_t sb = slot_bytes(lp);
    const LV& L = lp.view64;
    if (lp.nfastbc > 0)
        k_collide<3><<<lp.nfastbc, TILE_CELLS, sb, s>>>(L, lp, P, ph, lp.fastbc_tiles, fA, gA, fAg, gAg, fB, gB, md,
                                                        gqc);
    if (lp.nfastebbc > 0)
        k_collide<4><<<lp.nfastebbc, TILE_CELLS, sb, s>>>(L, lp, P, ph, lp.fastebbc_tiles, fA, gA, fAg, gAg, fB, gB,
                                                          md, gqc);
}

}  // namespace mbg
