// mbg_fp64.cuh -- device helpers shared by the FP64 kernels (mbg_fp64*.cu):
// the pull of one streamed population, tile-to-cell mapping and the
// q-correction gradient.  Every FP64 unit is compiled with -fmad=false so that
// each multiply and add is rounded separately, as in the reference's CPU build.
#pragma once

#include "mbg_kernels.h"
#include "mbg_level.cuh"

namespace mbg {

using LV = LevelView<double>;

// override value of a (coarse cell, direction) whose eight fine children were
// all masked: the step pulls the cell's own streamed value there (a NaN bit
// pattern that arithmetic does not produce)
constexpr long long NOOVR64 = (long long)0xFFF8000000000FFDULL;
__device__ __forceinline__ bool is_noovr(double v) { return __double_as_longlong(v) == NOOVR64; }

// pulled (post-stream) value of direction q at box-local target (x,y,z)
template <int q>
__device__ __forceinline__ double pull(const LV& L, const BCParams& P, const DevBox& B, int x, int y, int z,
                                       uint8_t tflag, bool interior, const double* v, const double* vg, bool is_g,
                                       const Lattice<double>& lat)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    constexpr int oq = opp(q);
    if (interior) return v[q * L.N + B.voff + val_lin(B, x - ex, y - ey, z - ez)];
    if (!(tflag & FL_FLUID)) return -1.0;
    const int sx = x - ex, sy = y - ey, sz = z - ez;
    if (sx < -3 || sy < -3 || sz < -3 || sx > B.n[0] + 2 || sy > B.n[1] + 2 || sz > B.n[2] + 2) return -1.0;
    const uint8_t sf = flag_at(L, B, sx, sy, sz);
    if (!(sf & FL_FLUID)) return fab_value(L, B, x, y, z, oq, v, vg);
    int gp[3] = {B.lo[0] + sx, B.lo[1] + sy, B.lo[2] + sz};
    if (outside_nonperiodic(L, gp))
        return bc_value<q, double, double>(L, P, B, sx, sy, sz, is_g, v, vg, lat, [](double r, int) { return r; });
    return fab_value(L, B, sx, sy, sz, q, v, vg);
}

__device__ __forceinline__ bool cell_of_tile(const LV& L, const Tile* tiles, int& b, int& x, int& y, int& z,
                                             long long& c)
{
    const Tile t = tiles[blockIdx.x];
    b = t.box;
    const DevBox& B = L.box[b];
    c = (long long)t.start + threadIdx.x;
    const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
    if (c >= vol) return false;
    x = (int)(c % B.n[0]);
    const long long r = c / B.n[0];
    y = (int)(r % B.n[1]);
    z = (int)(r / B.n[1]);
    return true;
}

__device__ __forceinline__ bool is_interior(const DevBox& B, int x, int y, int z)
{
    return B.all_fluid && x > 0 && y > 0 && z > 0 && x < B.n[0] - 1 && y < B.n[1] - 1 && z < B.n[2] - 1;
}

// Q_corr component d at box-local neighbour (x,y,z): own box, owning box
// (periodic image) or the box's own ghost scratch
__device__ __forceinline__ double qcorr_at(const LV& L, const DevBox& B, int x, int y, int z, int d,
                                           const double* md, const double* gqc)
{
    if (in_valid<double>(B, x, y, z)) return md[(MD_QCX + d) * L.N + B.voff + val_lin(B, x, y, z)];
    int p[3] = {B.lo[0] + x, B.lo[1] + y, B.lo[2] + z};
    wrap_pos(L, p);
    const int o = owner_of(L, p);
    if (o >= 0) {
        const DevBox& O = L.box[o];
        return md[(MD_QCX + d) * L.N + O.voff + val_lin(O, p[0] - O.lo[0], p[1] - O.lo[1], p[2] - O.lo[2])];
    }
    if (B.goff < 0 || gqc == nullptr) return 0.0;  // plans exclude this case
    return gqc[d * L.NG + B.goff + fab_lin(B, x, y, z)];
}

// gradient() of Source/Utilities.H:279-312 for component Q_corr_d along d
__device__ __forceinline__ double qgrad(const LV& L, const DevBox& B, int x, int y, int z, int d, double idx,
                                       const double* md, const double* gqc)
{
    int pp[3] = {x, y, z}, pm[3] = {x, y, z};
    pp[d] += 1;
    pm[d] -= 1;
    const int gpd = B.lo[d] + pp[d], gmd = B.lo[d] + pm[d];
    const bool p_out = gpd > L.dhi[d] || !(flag_at(L, B, pp[0], pp[1], pp[2]) & FL_FLUID);
    const bool m_out = gmd < L.dlo[d] || !(flag_at(L, B, pm[0], pm[1], pm[2]) & FL_FLUID);
    double vp = 0.0, vc = 0.0, vm = 0.0;
    if (p_out && m_out) {
        vp = 0.0; vc = 0.0; vm = 0.0;
    } else if (p_out) {
        vp = 0.0;
        vc = qcorr_at(L, B, x, y, z, d, md, gqc);
        vm = -qcorr_at(L, B, pm[0], pm[1], pm[2], d, md, gqc);
    } else if (m_out) {
        vp = qcorr_at(L, B, pp[0], pp[1], pp[2], d, md, gqc);
        vc = -qcorr_at(L, B, x, y, z, d, md, gqc);
        vm = 0.0;
    } else {
        vp = 0.5 * qcorr_at(L, B, pp[0], pp[1], pp[2], d, md, gqc);
        vc = 0.0;
        vm = -0.5 * qcorr_at(L, B, pm[0], pm[1], pm[2], d, md, gqc);
    }
    return (vp + vc + vm) * idx;
}

}  // namespace mbg
