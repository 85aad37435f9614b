// mbg_fp64.cu -- FP64 form of the level step (the reference's storage and
// arithmetic).  Compiled with -fmad=false so that every multiply and add is
// rounded separately, as in the reference's CPU build.
//
// A level advance is two passes over the valid cells:
//   k_moments : pull-stream f and g (Source/LBM.cpp:558-604) and compute the
//               macro fields (f_to_macrodata, LBM.cpp:810-906) into a scratch
//               array;
//   k_collide : pull the same values again, take the q-correction gradient
//               from the neighbours' scratch (LBM.cpp:959-991), build the
//               equilibria (LBM.cpp:621-762) and relax (LBM.cpp:765-807),
//               writing the new state.
// FP64 arithmetic bounds this form (about 1 kflop per cell update), so the
// second pull costs memory bandwidth that is otherwise idle.
#include <cstdio>

#include "mbg_fp64.cuh"

namespace mbg {

// ---- pass 1: stream + macro fields ----------------------------------------
__global__ void __launch_bounds__(TILE_CELLS) k_moments(LV L, BCParams P, Phys64 ph, const Tile* tiles,
                                                        const double* fA, const double* gA, const double* fAg,
                                                        const double* gAg, const double* fB, const double* gB,
                                                        double* md)
{
    int b, x, y, z;
    long long c;
    if (!cell_of_tile(L, tiles, b, x, y, z, c)) return;
    const DevBox& B = L.box[b];
    const uint8_t tf = flag_at(L, B, x, y, z);
    if (!(tf & FL_FLUID)) return;
    const bool ovr = tf & FL_OVR;
    const bool interior = !ovr && is_interior(B, x, y, z);
    const long long cell = B.voff + c;
    MomentAcc<double> acc;
#define MBG_M64(q)                                                             \
    {                                                                          \
        double fq = ovr ? fB[q * L.N + cell] : 0.0;                            \
        double gq = ovr ? gB[q * L.N + cell] : 0.0;                            \
        if (!ovr || is_noovr(fq))                                              \
            fq = pull<q>(L, P, B, x, y, z, tf, interior, fA, fAg, false, ph.lat); \
        if (!ovr || is_noovr(gq))                                              \
            gq = pull<q>(L, P, B, x, y, z, tf, interior, gA, gAg, true, ph.lat);  \
        acc.template add<q>(fq, gq);                                           \
    }
    MBG_UNROLL27(MBG_M64)
#undef MBG_M64
    const Macro<double> m = acc.finish(ph.mesh_speed, ph.Rg, ph.cv);
    const long long N = L.N;
    md[MD_RHO * N + cell] = m.rho;
    md[MD_U * N + cell] = m.u;
    md[MD_V * N + cell] = m.v;
    md[MD_W * N + cell] = m.w;
    md[MD_TRE * N + cell] = m.two_rho_e;
    md[MD_PXX * N + cell] = m.pxx;
    md[MD_PYY * N + cell] = m.pyy;
    md[MD_PZZ * N + cell] = m.pzz;
    md[MD_PXY * N + cell] = m.pxy;
    md[MD_PXZ * N + cell] = m.pxz;
    md[MD_PYZ * N + cell] = m.pyz;
    md[MD_QX * N + cell] = m.qx;
    md[MD_QY * N + cell] = m.qy;
    md[MD_QZ * N + cell] = m.qz;
    md[MD_T * N + cell] = m.temp;
    md[MD_QCX * N + cell] = m.qcx;
    md[MD_QCY * N + cell] = m.qcy;
    md[MD_QCZ * N + cell] = m.qcz;
}

// ---- pass 2: q-correction, equilibria, relaxation --------------------------
__global__ void __launch_bounds__(TILE_CELLS) k_collide(LV L, BCParams P, Phys64 ph, const Tile* tiles,
                                                        const double* fA, const double* gA, const double* fAg,
                                                        const double* gAg, double* fB, double* gB,
                                                        const double* md, const double* gqc)
{
    int b, x, y, z;
    long long c;
    if (!cell_of_tile(L, tiles, b, x, y, z, c)) return;
    const DevBox& B = L.box[b];
    const uint8_t tf = flag_at(L, B, x, y, z);
    const long long N = L.N;
    const long long cell = B.voff + c;
    const bool ovr = tf & FL_OVR;
    if (!(tf & FL_FLUID)) {
        // solid cells keep the stream's sentinel (or the coalesced value)
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            if (!ovr || is_noovr(fB[q * N + cell])) fB[q * N + cell] = -1.0;
            if (!ovr || is_noovr(gB[q * N + cell])) gB[q * N + cell] = -1.0;
        }
        return;
    }
    const bool interior = !ovr && is_interior(B, x, y, z);
    Macro<double> m;
    m.rho = md[MD_RHO * N + cell];
    m.u = md[MD_U * N + cell];
    m.v = md[MD_V * N + cell];
    m.w = md[MD_W * N + cell];
    m.two_rho_e = md[MD_TRE * N + cell];
    m.pxx = md[MD_PXX * N + cell];
    m.pyy = md[MD_PYY * N + cell];
    m.pzz = md[MD_PZZ * N + cell];
    m.pxy = md[MD_PXY * N + cell];
    m.pxz = md[MD_PXZ * N + cell];
    m.pyz = md[MD_PYZ * N + cell];
    m.qx = md[MD_QX * N + cell];
    m.qy = md[MD_QY * N + cell];
    m.qz = md[MD_QZ * N + cell];
    m.temp = md[MD_T * N + cell];
    const double dqx = qgrad(L, B, x, y, z, 0, ph.idx[0], md, gqc);
    const double dqy = qgrad(L, B, x, y, z, 1, ph.idx[1], md, gqc);
    const double dqz = qgrad(L, B, x, y, z, 2, ph.idx[2], md, gqc);
    Equilibrium<double> E;
    const double omega =
        build_equilibrium<double>(m, dqx, dqy, dqz, ph.nu, ph.alpha, ph.dt, ph.Rg, ph.cv, ph.lat, E);
#define MBG_RF64(q)                                                                                  \
    {                                                                                                \
        double fq = ovr ? fB[q * N + cell] : 0.0;                                                    \
        if (!ovr || is_noovr(fq)) fq = pull<q>(L, P, B, x, y, z, tf, interior, fA, fAg, false, ph.lat); \
        const double feq = E.template feq<q>();                                                      \
        fB[q * N + cell] = fq + omega * (feq - fq);                                                  \
    }
#define MBG_RG64(q)                                                                                  \
    {                                                                                                \
        double gq = ovr ? gB[q * N + cell] : 0.0;                                                    \
        if (!ovr || is_noovr(gq)) gq = pull<q>(L, P, B, x, y, z, tf, interior, gA, gAg, true, ph.lat); \
        const double geq = E.template geq<q>(ph.lat);                                                \
        gB[q * N + cell] = gq + omega * (geq - gq);                                                  \
    }
    MBG_UNROLL27(MBG_RF64)
    MBG_UNROLL27(MBG_RG64)
#undef MBG_RF64
#undef MBG_RG64
}

// ---- launchers -----------------------------------------------------------
void launch_moments(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                    const double* fAg, const double* gAg, const double* fB, const double* gB, double* md,
                    cudaStream_t s)
{
    if (lp.ntiles == 0) return;
    k_moments<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, P, ph, lp.tiles, fA, gA, fAg, gAg, fB, gB, md);
}

void launch_collide(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                    const double* fAg, const double* gAg, double* fB, double* gB, const double* md,
                    const double* gqc, cudaStream_t s)
{
    if (lp.ntiles == 0) return;
    k_collide<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, P, ph, lp.tiles, fA, gA, fAg, gAg, fB, gB, md, gqc);
}

}  // namespace mbg
