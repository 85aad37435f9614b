// mbg_fp64_shell.cu -- FP64 kernels of a fine level's coarse-fine ghost shell:
// the streamed values of the uncovered ghost cells and their q-correction
// moments, kept per box as the reference's per-FArrayBox ghosts.
#include <cstdio>

#include "mbg_fp64.cuh"

namespace mbg {

// ---- fine-level ghost shell ----------------------------------------------
// streamed values of the uncovered ghost cells (next substep reads them)
__global__ void k_ghost_stream(LV L, BCParams P, Phys64 ph, const GhostCell* gl, long long n, const double* fA,
                               const double* gA, const double* fAg, const double* gAg, double* fBg, double* gBg)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const GhostCell gc = gl[e];
    const DevBox& B = L.box[gc.box];
    const uint8_t tf = flag_at(L, B, gc.x, gc.y, gc.z);
    const long long gi = B.goff + fab_lin(B, gc.x, gc.y, gc.z);
#define MBG_GS64(q)                                                                          \
    {                                                                                        \
        fBg[q * L.NG + gi] = pull<q>(L, P, B, gc.x, gc.y, gc.z, tf, false, fA, fAg, false, ph.lat); \
        gBg[q * L.NG + gi] = pull<q>(L, P, B, gc.x, gc.y, gc.z, tf, false, gA, gAg, true, ph.lat);  \
    }
    MBG_UNROLL27(MBG_GS64)
#undef MBG_GS64
}

// Q_corr of the streamed values at first-layer uncovered ghost cells: the
// moments of what k_ghost_stream of the same advance has just written into
// the ghost fab (fBg, gBg) -- the same values the pulls would give
__global__ void k_ghost_moments(LV L, Phys64 ph, const GhostCell* gl, long long n, const double* fBg,
                                const double* gBg, double* gqc)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const GhostCell gc = gl[e];
    const DevBox& B = L.box[gc.box];
    const uint8_t tf = flag_at(L, B, gc.x, gc.y, gc.z);
    if (!(tf & FL_FLUID)) return;
    const long long gi = B.goff + fab_lin(B, gc.x, gc.y, gc.z);
    MomentAcc<double> acc;
#define MBG_GM64(q) acc.template add<q>(fBg[q * L.NG + gi], gBg[q * L.NG + gi]);
    MBG_UNROLL27(MBG_GM64)
#undef MBG_GM64
    const Macro<double> m = acc.finish(ph.mesh_speed, ph.Rg, ph.cv);
    gqc[0 * L.NG + gi] = m.qcx;
    gqc[1 * L.NG + gi] = m.qcy;
    gqc[2 * L.NG + gi] = m.qcz;
}

void launch_ghost_stream(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA,
                         const double* gA, const double* fAg, const double* gAg, double* fBg, double* gBg,
                         cudaStream_t s)
{
    if (lp.nghost_cells == 0) return;
    const int th = 128;
    const long long nb = (lp.nghost_cells + th - 1) / th;
    k_ghost_stream<<<(unsigned)nb, th, 0, s>>>(lp.view64, P, ph, lp.ghost_list, lp.nghost_cells, fA, gA, fAg, gAg,
                                               fBg, gBg);
}

void launch_ghost_moments(const LevelPlan& lp, const Phys64& ph, const double* fBg, const double* gBg, double* gqc,
                          cudaStream_t s)
{
    if (lp.nghost1 == 0) return;
    const int th = 128;
    const long long nb = (lp.nghost1 + th - 1) / th;
    k_ghost_moments<<<(unsigned)nb, th, 0, s>>>(lp.view64, ph, lp.ghost_list1, lp.nghost1, fBg, gBg, gqc);
}

}  // namespace mbg
