// mbg_fp64.cu -- FP64 form of the level step (the reference's storage and
// arithmetic): the launchers of both passes over the tile lists of a level
// and the kernels of modes 1 and 2; modes 3-4 and 0 are instantiated in
// mbg_fp64_bc.cu and mbg_fp64_gen.cu (the kernels: mbg_fp64_step.cuh).
// Compiled with -fmad=false so that every multiply and add is rounded
// separately, as in the reference's CPU build.
#include <cstdio>

#include "mbg_fp64_step.cuh"

namespace mbg {

// ---- launchers -----------------------------------------------------------
// the slot-table tiles (all fluid, holding solids), then the others through
// the general pull
void launch_moments(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                    const double* fAg, const double* gAg, const double* fB, const double* gB, double* md,
                    cudaStream_t s)
{
    const size_t sb = slot_bytes(lp);
    const LV& L = lp.view64;
    if (lp.nfast > 0)
        k_moments<1><<<lp.nfast, TILE_CELLS, sb, s>>>(L, lp, P, ph, lp.fast_tiles, fA, gA, fAg, gAg, fB, gB, md);
    if (lp.nfasteb > 0)
        k_moments<2><<<lp.nfasteb, TILE_CELLS, sb, s>>>(L, lp, P, ph, lp.fasteb_tiles, fA, gA, fAg, gAg, fB, gB, md);
    launch_moments_bc(lp, P, ph, fA, gA, fAg, gAg, fB, gB, md, s);
    launch_moments_gen(lp, P, ph, fA, gA, fAg, gAg, fB, gB, md, s);
}

void launch_collide(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                    const double* fAg, const double* gAg, double* fB, double* gB, const double* md,
                    const double* gqc, cudaStream_t s)
{
    const size_t sb = slot_bytes(lp);
    const LV& L = lp.view64;
    if (lp.nfast > 0)
        k_collide<1><<<lp.nfast, TILE_CELLS, sb, s>>>(L, lp, P, ph, lp.fast_tiles, fA, gA, fAg, gAg, fB, gB, md, gqc);
    if (lp.nfasteb > 0)
        k_collide<2><<<lp.nfasteb, TILE_CELLS, sb, s>>>(L, lp, P, ph, lp.fasteb_tiles, fA, gA, fAg, gAg, fB, gB, md,
                                                        gqc);
    launch_collide_bc(lp, P, ph, fA, gA, fAg, gAg, fB, gB, md, gqc, s);
    launch_collide_gen(lp, P, ph, fA, gA, fAg, gAg, fB, gB, md, gqc, s);
}

int fp64_step_launches(const LevelPlan& lp)
{
    return (lp.nfast > 0) + (lp.nfasteb > 0) + (lp.nfastbc > 0) + (lp.nfastebbc > 0) + (lp.ngen > 0);
}

}  // namespace mbg
