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

#include "mbg_kernels.h"
#include "mbg_level.cuh"

namespace mbg {

using LV = LevelView<double>;

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
    static_for<0, NQ>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        double fq, gq;
        if (ovr) {
            fq = fB[q * L.N + cell];
            gq = gB[q * L.N + cell];
        } else {
            fq = pull<q>(L, P, B, x, y, z, tf, interior, fA, fAg, false, ph.lat);
            gq = pull<q>(L, P, B, x, y, z, tf, interior, gA, gAg, true, ph.lat);
        }
        acc.template add<q>(fq, gq);
    });
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
        if (!ovr) {
#pragma unroll
            for (int q = 0; q < NQ; ++q) { fB[q * N + cell] = -1.0; gB[q * N + cell] = -1.0; }
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
    static_for<0, NQ>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        const double fq = ovr ? fB[q * N + cell] : pull<q>(L, P, B, x, y, z, tf, interior, fA, fAg, false, ph.lat);
        const double feq = E.template feq<q>();
        fB[q * N + cell] = fq + omega * (feq - fq);
    });
    static_for<0, NQ>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        const double gq = ovr ? gB[q * N + cell] : pull<q>(L, P, B, x, y, z, tf, interior, gA, gAg, true, ph.lat);
        const double geq = E.template geq<q>(ph.lat);
        gB[q * N + cell] = gq + omega * (geq - gq);
    });
}

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
    static_for<0, NQ>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        fBg[q * L.NG + gi] = pull<q>(L, P, B, gc.x, gc.y, gc.z, tf, false, fA, fAg, false, ph.lat);
        gBg[q * L.NG + gi] = pull<q>(L, P, B, gc.x, gc.y, gc.z, tf, false, gA, gAg, true, ph.lat);
    });
}

// Q_corr of the streamed values at first-layer uncovered ghost cells
__global__ void k_ghost_moments(LV L, BCParams P, Phys64 ph, const GhostCell* gl, long long n, const double* fA,
                                const double* gA, const double* fAg, const double* gAg, double* gqc)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const GhostCell gc = gl[e];
    const DevBox& B = L.box[gc.box];
    const uint8_t tf = flag_at(L, B, gc.x, gc.y, gc.z);
    if (!(tf & FL_FLUID)) return;
    MomentAcc<double> acc;
    static_for<0, NQ>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        const double fq = pull<q>(L, P, B, gc.x, gc.y, gc.z, tf, false, fA, fAg, false, ph.lat);
        const double gq = pull<q>(L, P, B, gc.x, gc.y, gc.z, tf, false, gA, gAg, true, ph.lat);
        acc.template add<q>(fq, gq);
    });
    const Macro<double> m = acc.finish(ph.mesh_speed, ph.Rg, ph.cv);
    const long long gi = B.goff + fab_lin(B, gc.x, gc.y, gc.z);
    gqc[0 * L.NG + gi] = m.qcx;
    gqc[1 * L.NG + gi] = m.qcy;
    gqc[2 * L.NG + gi] = m.qcz;
}

// ---- explosion: conservative linear interpolation of the coarse level ------
// (AMReX cell_cons_interp as called at Source/FillPatchOps.H:124-128: MC
// slopes, one limiter factor per direction shared by all 27 components)
__device__ __forceinline__ double crse_at(const LV& C, const int p0[3], int d, int s, int q, const double* v)
{
    int p[3] = {p0[0], p0[1], p0[2]};
    p[d] += s;
    wrap_pos(C, p);
    const int o = owner_of(C, p);
    if (o < 0) return 0.0;  // plans reject fine levels whose stencil leaves the coarse level
    const DevBox& O = C.box[o];
    return v[q * C.N + O.voff + val_lin(O, p[0] - O.lo[0], p[1] - O.lo[1], p[2] - O.lo[2])];
}

__global__ void k_explode(LV F, LV C, const GhostCell* gl, long long n, const double* fc, const double* gc_,
                          double* fg, double* gg)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const GhostCell g = gl[e];
    const DevBox& B = F.box[g.box];
    int fp[3] = {B.lo[0] + g.x, B.lo[1] + g.y, B.lo[2] + g.z};
    wrap_pos(F, fp);
    const int cp[3] = {fp[0] >> 1, fp[1] >> 1, fp[2] >> 1};
    const double off[3] = {((fp[0] - 2 * cp[0]) + 0.5) / 2.0 - 0.5, ((fp[1] - 2 * cp[1]) + 0.5) / 2.0 - 0.5,
                           ((fp[2] - 2 * cp[2]) + 0.5) / 2.0 - 0.5};
    const long long gi = B.goff + fab_lin(B, g.x, g.y, g.z);
    for (int lat = 0; lat < 2; ++lat) {
        const double* v = lat ? gc_ : fc;
        double* out = lat ? gg : fg;
        double alpha[3] = {1.0, 1.0, 1.0};
        for (int d = 0; d < 3; ++d) {
            for (int q = 0; q < NQ; ++q) {
                const double u0 = crse_at(C, cp, d, 0, q, v);
                const double up = crse_at(C, cp, d, 1, q, v);
                const double um = crse_at(C, cp, d, -1, q, v);
                const double cen = 0.5 * (up - um);
                const double forw = 2.0 * (up - u0);
                const double back = 2.0 * (u0 - um);
                const double slp = (forw * back >= 0.0) ? fmin(fabs(forw), fabs(back)) : 0.0;
                if (cen != 0.0) alpha[d] = fmin(alpha[d], fmin(slp, fabs(cen)) / fabs(cen));
            }
        }
        for (int q = 0; q < NQ; ++q) {
            const double u0 = crse_at(C, cp, 0, 0, q, v);
            const double cx = 0.5 * (crse_at(C, cp, 0, 1, q, v) - crse_at(C, cp, 0, -1, q, v));
            const double cy = 0.5 * (crse_at(C, cp, 1, 1, q, v) - crse_at(C, cp, 1, -1, q, v));
            const double cz = 0.5 * (crse_at(C, cp, 2, 1, q, v) - crse_at(C, cp, 2, -1, q, v));
            out[q * F.NG + gi] = u0 + off[0] * (alpha[0] * cx) + off[1] * (alpha[1] * cy) + off[2] * (alpha[2] * cz);
        }
    }
}

// ---- coalescence: masked average of the 8 fine children --------------------
// (masked_avgdown, Source/Utilities.H:315-350).  into_state: write into the
// coarse state buffer directly (initial average_down, ng = 0); otherwise into
// the coarse post-stream override buffer, with the coarse streamed value
// where every child is masked.
__global__ void k_coalesce(LV C, LV F, BCParams P, Phys64 ph, const CoalesceCell* cl, long long n,
                           const double* ff, const double* gf, const double* ffg, const double* gfg,
                           const double* fcA, const double* gcA, const double* fcAg, const double* gcAg,
                           double* fcB, double* gcB, int into_state)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const CoalesceCell cc = cl[e];
    const DevBox& O = C.box[cc.cbox];
    const DevBox& A = F.box[cc.fbox];
    const long long cell = O.voff + val_lin(O, cc.cx, cc.cy, cc.cz);
    const uint8_t tf = flag_at(C, O, cc.cx, cc.cy, cc.cz);
    const double masked = -1.0;
    for (int lat = 0; lat < 2; ++lat) {
        const double* v = lat ? gf : ff;
        const double* vg = lat ? gfg : ffg;
        double* out = lat ? gcB : fcB;
        const double* cA = lat ? gcA : fcA;
        const double* cAg = lat ? gcAg : fcAg;
        static_for<0, NQ>([&](auto qc) {
            constexpr int q = decltype(qc)::value;
            double s = 0.0, vol = 0.0;
            for (int kr = 0; kr < 2; ++kr)
                for (int jr = 0; jr < 2; ++jr)
                    for (int ir = 0; ir < 2; ++ir) {
                        const double fv = fab_value(F, A, cc.fx + ir, cc.fy + jr, cc.fz + kr, q, v, vg);
                        if (fabs(fv - masked) > ph.small_num) { s += fv; vol += 1.0; }
                    }
            double r;
            if (vol > 0.0) r = s / vol;
            else if (into_state) r = cA[q * C.N + cell];
            else r = pull<q>(C, P, O, cc.cx, cc.cy, cc.cz, tf, false, cA, cAg, lat == 1, ph.lat);
            out[q * C.N + cell] = r;
        });
    }
}

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
    double* o = out19 + B.voff * 19 + c;
    if (!(flag_at(L, B, x, y, z) & FL_FLUID)) {
        for (int k = 0; k < 19; ++k) o[k * vol] = 0.0;
        return;
    }
    MomentAcc<double> acc;
    static_for<0, NQ>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        acc.template add<q>(f[q * N + cell], g[q * N + cell]);
    });
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
            static_for<0, NQ>([&](auto qc) {
                constexpr int q = decltype(qc)::value;
                constexpr int ob = opp(q);
                const int rx = x + ev_x(ob), ry = y + ev_y(ob), rz = z + ev_z(ob);
                int gp[3] = {B.lo[0] + rx, B.lo[1] + ry, B.lo[2] + rz};
                if (outside_nonperiodic(L, gp)) return;
                const double isf = (flag_at(L, B, rx, ry, rz) & FL_FLUID) ? 1.0 : 0.0;
                const double fv = fab_value(L, B, rx, ry, rz, q, f, fg);
                fs[0] += 2.0 * ev_x(q) * fv * isf;
                fs[1] += 2.0 * ev_y(q) * fv * isf;
                fs[2] += 2.0 * ev_z(q) * fv * isf;
            });
        }
    }
    for (int d = 0; d < 3; ++d)
        if (fs[d] != 0.0) atomicAdd(&out3[d], fs[d]);
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

void launch_ghost_moments(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA,
                          const double* gA, const double* fAg, const double* gAg, double* gqc, cudaStream_t s)
{
    if (lp.nghost1 == 0) return;
    const int th = 128;
    const long long nb = (lp.nghost1 + th - 1) / th;
    k_ghost_moments<<<(unsigned)nb, th, 0, s>>>(lp.view64, P, ph, lp.ghost_list1, lp.nghost1, fA, gA, fAg, gAg,
                                                gqc);
}

void launch_explode(const LevelPlan& fine, const LevelPlan& crse, const double* fc, const double* gc, double* fg,
                    double* gg, cudaStream_t s)
{
    if (fine.nghost_cells == 0) return;
    const int th = 64;
    const long long nb = (fine.nghost_cells + th - 1) / th;
    k_explode<<<(unsigned)nb, th, 0, s>>>(fine.view64, crse.view64, fine.ghost_list, fine.nghost_cells, fc, gc, fg,
                                          gg);
}

void launch_coalesce(const LevelPlan& crse, const LevelPlan& fine, const BCParams& P, const Phys64& ph,
                     const CoalesceCell* list, long long n, const double* ff, const double* gf, const double* ffg,
                     const double* gfg, const double* fcA, const double* gcA, const double* fcAg,
                     const double* gcAg, double* fcB, double* gcB, int into_state, cudaStream_t s)
{
    if (n == 0) return;
    const int th = 64;
    const long long nb = (n + th - 1) / th;
    k_coalesce<<<(unsigned)nb, th, 0, s>>>(crse.view64, fine.view64, P, ph, list, n, ff, gf, ffg, gfg, fcA, gcA,
                                           fcAg, gcAg, fcB, gcB, into_state);
}

void launch_macro_local(const LevelPlan& lp, const Phys64& ph, const double* f, const double* g, double* out19,
                        cudaStream_t s)
{
    if (lp.ntiles == 0) return;
    k_macro_local<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, ph, lp.tiles, f, g, out19);
}

void launch_eb_forces(const LevelPlan& lp, const double* f, const double* fg, double* out3, cudaStream_t s)
{
    if (lp.ntiles == 0) return;
    k_eb_forces<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, lp.tiles, f, fg, out3);
}

}  // namespace mbg
