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

// the same for ghost cells of all-fluid boxes with a ghost-shell slot table:
// a source within the shell (-3 .. n + 2 along each axis) is read through
// the table (a valid cell of the owning box or the box's own ghost fab),
// one further out gives the stream's -1 (Source/LBM.cpp:558-604 over the
// grown box)
__global__ void k_ghost_stream_slot(LV L, const NbrSlot* __restrict__ gslots, const int* __restrict__ gslot_off,
                                    int lg0, int lg1, int lg2, const GhostCell* gl, long long n,
                                    const double* __restrict__ fA, const double* __restrict__ gA,
                                    const double* __restrict__ fAg, const double* __restrict__ gAg,
                                    double* __restrict__ fBg, double* __restrict__ gBg)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const GhostCell gc = gl[e];
    const DevBox& B = L.box[gc.box];
    const NbrSlot* __restrict__ T = gslots + gslot_off[gc.box];
    const int lg[3] = {lg0, lg1, lg2};
    int top[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) top[d] = ((B.n[d] + (1 << lg[d]) - 1) >> lg[d]) + 1;
    const int tx = top[0] + 1, ty = top[1] + 1;
    const long long gi = B.goff + fab_lin(B, gc.x, gc.y, gc.z);
#define MBG_GSS(q)                                                                                           \
    {                                                                                                        \
        const int sx = gc.x - ev_x(q), sy = gc.y - ev_y(q), sz = gc.z - ev_z(q);                              \
        double fv = -1.0, gv = -1.0;                                                                         \
        if (sx >= -3 && sy >= -3 && sz >= -3 && sx <= B.n[0] + 2 && sy <= B.n[1] + 2 && sz <= B.n[2] + 2) {  \
            const int ox = sx < 0 ? 0 : (sx < B.n[0] ? (sx >> lg0) + 1 : top[0]);                           \
            const int oy = sy < 0 ? 0 : (sy < B.n[1] ? (sy >> lg1) + 1 : top[1]);                           \
            const int oz = sz < 0 ? 0 : (sz < B.n[2] ? (sz >> lg2) + 1 : top[2]);                           \
            const NbrSlot s = T[ox + tx * (oy + ty * oz)];                                                   \
            const long long i = s.base + (long long)sz * s.sz + (long long)sy * s.sy + sx;                   \
            fv = s.ghost ? fAg[q * L.NG + i] : fA[q * L.N + i];                                              \
            gv = s.ghost ? gAg[q * L.NG + i] : gA[q * L.N + i];                                              \
        }                                                                                                    \
        fBg[q * L.NG + gi] = fv;                                                                             \
        gBg[q * L.NG + gi] = gv;                                                                             \
    }
    MBG_UNROLL27(MBG_GSS)
#undef MBG_GSS
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
    const int th = 128;
    if (lp.nghost_fast > 0)
        k_ghost_stream_slot<<<(unsigned)((lp.nghost_fast + th - 1) / th), th, 0, s>>>(
            lp.view64, lp.gslots, lp.gslot_off, lp.slot_lg[0], lp.slot_lg[1], lp.slot_lg[2], lp.ghost_fast,
            lp.nghost_fast, fA, gA, fAg, gAg, fBg, gBg);
    if (lp.nghost_gen > 0)
        k_ghost_stream<<<(unsigned)((lp.nghost_gen + th - 1) / th), th, 0, s>>>(lp.view64, P, ph, lp.ghost_gen,
                                                                               lp.nghost_gen, fA, gA, fAg, gAg, fBg,
                                                                               gBg);
}

int ghost_stream_launches(const LevelPlan& lp) { return (lp.nghost_fast > 0) + (lp.nghost_gen > 0); }

void launch_ghost_moments(const LevelPlan& lp, const Phys64& ph, const double* fBg, const double* gBg, double* gqc,
                          cudaStream_t s)
{
    if (lp.nghost1 == 0) return;
    const int th = 128;
    const long long nb = (lp.nghost1 + th - 1) / th;
    k_ghost_moments<<<(unsigned)nb, th, 0, s>>>(lp.view64, ph, lp.ghost_list1, lp.nghost1, fBg, gBg, gqc);
}

}  // namespace mbg
