// mbg_fp64_out.cu -- FP64 output kernels: macro fields of the stored state and
// the EB momentum-exchange force.
#include <cstdio>

#include "mbg_fp64.cuh"

namespace mbg {

// ---- output: macro fields of the current state (no stream) ------------------
__global__ void k_macro_local(LV L, Phys64 ph, const Tile* tiles, const double* f, const double* g, double* out19)
{
    int b, x, y, z;
    long long c;
    if (!cell_of_tile(L, tiles, b, x, y, z, c)) return;
    const DevBox& B = L.box[b];
    const long long cell = B.voff + c;
    const long long N = L.N;
    // host layout [box][comp][cell]
    const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
    double* o = out19 + B.hoff * 19 + c;
    if (!(flag_at(L, B, x, y, z) & FL_FLUID)) {
        for (int k = 0; k < 19; ++k) o[k * vol] = 0.0;
        return;
    }
    MomentAcc<double> acc;
#define MBG_ML64(q) acc.template add<q>(f[q * N + cell], g[q * N + cell]);
    MBG_UNROLL27(MBG_ML64)
#undef MBG_ML64
    const Macro<double> m = acc.finish(ph.mesh_speed, ph.Rg, ph.cv);
    const double vals[19] = {m.rho, m.u, m.v, m.w, sqrt(m.u * m.u + m.v * m.v + m.w * m.w), m.two_rho_e,
                             m.qcx, m.qcy, m.qcz, m.pxx, m.pyy, m.pzz, m.pxy, m.pxz, m.pyz,
                             m.qx, m.qy, m.qz, m.temp};
    for (int k = 0; k < 19; ++k) o[k * vol] = vals[k];
}

// ---- EB momentum-exchange force (Source/LBM.cpp:994-1044) -------------------
// per-cell sums in FP64; only eb_boundary cells contribute (a thin shell), so
// each such cell adds its three components with FP64 atomics
__global__ void k_eb_forces(LV L, const Tile* tiles, const double* f, const double* fg, double* out3)
{
    int b, x, y, z;
    long long c;
    double fs[3] = {0.0, 0.0, 0.0};
    if (cell_of_tile(L, tiles, b, x, y, z, c)) {
        const DevBox& B = L.box[b];
        const uint8_t tf = flag_at(L, B, x, y, z);
        if ((tf & FL_EBB) && !(tf & FL_COV)) {
#define MBG_EB64(q)                                                                \
            {                                                                          \
                constexpr int ob = opp(q);                                             \
                const int rx = x + ev_x(ob), ry = y + ev_y(ob), rz = z + ev_z(ob);     \
                int gp[3] = {B.lo[0] + rx, B.lo[1] + ry, B.lo[2] + rz};                \
                if (!outside_nonperiodic(L, gp)) {                                     \
                    const double isf = (flag_at(L, B, rx, ry, rz) & FL_FLUID) ? 1.0 : 0.0; \
                    const double fv = fab_value(L, B, rx, ry, rz, q, f, fg);           \
                    fs[0] += 2.0 * ev_x(q) * fv * isf;                                 \
                    fs[1] += 2.0 * ev_y(q) * fv * isf;                                 \
                    fs[2] += 2.0 * ev_z(q) * fv * isf;                                 \
                }                                                                      \
            }
            MBG_UNROLL27(MBG_EB64)
#undef MBG_EB64
        }
    }
    for (int d = 0; d < 3; ++d)
        if (fs[d] != 0.0) atomicAdd(&out3[d], fs[d]);
}


// ---- conserved totals (FP64): mass, momentum, 2 rho E of the stored state ----
// over fluid cells not covered by a finer level, weighted by the cell volume;
// a shared-memory tree per block, one FP64 atomic per block and total
__global__ void __launch_bounds__(TILE_CELLS) k_conserved(LV L, Phys64 ph, const Tile* tiles, const double* f,
                                                          const double* g, double dV, double* out5)
{
    __shared__ double red[5][TILE_CELLS];
    int b, x, y, z;
    long long c;
    double v[5] = {0, 0, 0, 0, 0};
    if (cell_of_tile(L, tiles, b, x, y, z, c)) {
        const DevBox& B = L.box[b];
        const uint8_t tf = flag_at(L, B, x, y, z);
        if ((tf & FL_FLUID) && !(tf & FL_COV)) {
            const long long cell = B.voff + c;
            MomentAcc<double> acc;
#define MBG_CN64(q) acc.template add<q>(f[q * L.N + cell], g[q * L.N + cell]);
            MBG_UNROLL27(MBG_CN64)
#undef MBG_CN64
            v[0] = acc.rho * dV;
            v[1] = acc.u * ph.mesh_speed * dV;
            v[2] = acc.v * ph.mesh_speed * dV;
            v[3] = acc.w * ph.mesh_speed * dV;
            v[4] = acc.tre * dV;
        }
    }
    const int t = threadIdx.x;
    for (int k = 0; k < 5; ++k) red[k][t] = v[k];
    __syncthreads();
    for (int h = TILE_CELLS / 2; h > 0; h >>= 1) {
        if (t < h)
            for (int k = 0; k < 5; ++k) red[k][t] += red[k][t + h];
        __syncthreads();
    }
    if (t == 0)
        for (int k = 0; k < 5; ++k) atomicAdd(&out5[k], red[k][0]);
}

void launch_macro_local(const LevelPlan& lp, const Phys64& ph, const double* f, const double* g, double* out19,
                        cudaStream_t s)
{
    if (lp.ntiles == 0) return;
    k_macro_local<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, ph, lp.tiles, f, g, out19);
}

void launch_conserved(const LevelPlan& lp, const Phys64& ph, const double* f, const double* g, double dV, double* out5,
                      cudaStream_t s)
{
    if (lp.ntiles > 0) k_conserved<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, ph, lp.tiles, f, g, dV, out5);
}

void launch_eb_forces(const LevelPlan& lp, const double* f, const double* fg, double* out3, cudaStream_t s)
{
    if (lp.ntiles == 0) return;
    k_eb_forces<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, lp.tiles, f, fg, out3);
}

}  // namespace mbg
