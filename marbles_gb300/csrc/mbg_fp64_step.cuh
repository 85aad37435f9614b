// mbg_fp64_step.cuh -- the FP64 level step's kernels (k_moments, k_collide)
// and their neighbour-slot pulls, shared by the units that instantiate them:
// mbg_fp64.cu (modes 1 and 2), mbg_fp64_bc.cu and mbg_fp64_bcc.cu (modes 3
// and 4, moment and collision pass) and mbg_fp64_gen.cu (mode 0), so that
// the parallel build compiles them side by side.  Every including unit is compiled with -fmad=false.
//
// A level advance is two passes over the valid cells, each launched over up
// to five tile lists: boxes whose neighbourhood the chunked slot tables
// describe (every neighbour chunk held by one box, by the box's ghost fab,
// or wholly beyond a non-periodic side) pull by the table -- the same index
// arithmetic for every cell, so warps do not diverge at box faces, also on
// the uneven boxes of refined levels -- without flag checks when the box is
// all fluid and with them (bounce-back at solid sources) when it holds
// solids; the other boxes use the general pull with its boundary cases:
//   k_moments : pull-stream f and g (Source/LBM.cpp:558-604) and compute the
//               macro fields (f_to_macrodata, LBM.cpp:810-906) into a scratch
//               array;
//   k_collide : pull the same values again, take the q-correction gradient
//               from the neighbours' scratch (LBM.cpp:959-991), build the
//               equilibria (LBM.cpp:621-762) and relax (LBM.cpp:765-807),
//               writing the new state.
// FP64 arithmetic bounds this form (about 1 kflop per cell update), so the
// second pull costs memory bandwidth that is otherwise idle.
#pragma once

#include "mbg_fp64.cuh"

namespace mbg {

// ---- pulls through the neighbour-slot table of the CTA's box ---------------
// the table in shared memory and the chunking of the box
struct SlotTab {
    const NbrSlot* s;
    int lg[3];
    int tx, ty;      // table extent along x and y
    int top[3];      // chunk index of the layer above the box
};

// chunk index along one axis of box-local coordinate v (-1 .. n)
__device__ __forceinline__ int chunk_of(int v, int n, int lg, int top)
{
    return v < 0 ? 0 : (v < n ? (v >> lg) + 1 : top);
}

// (boxes of the slot tile lists: no physical boundary within one cell, every
// neighbour chunk in one box or in the box's ghost fab)
template <int q>
__device__ __forceinline__ double pull_slot(const SlotTab& T, const DevBox& B, int x, int y, int z,
                                            const double* v, const double* vg, long long N, long long NG)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    const int sx = x - ex, sy = y - ey, sz = z - ez;
    const int ox = ex == 0 ? (x >> T.lg[0]) + 1 : chunk_of(sx, B.n[0], T.lg[0], T.top[0]);
    const int oy = ey == 0 ? (y >> T.lg[1]) + 1 : chunk_of(sy, B.n[1], T.lg[1], T.top[1]);
    const int oz = ez == 0 ? (z >> T.lg[2]) + 1 : chunk_of(sz, B.n[2], T.lg[2], T.top[2]);
    const NbrSlot& s = T.s[ox + T.tx * (oy + T.ty * oz)];
    const long long i = s.base + (long long)sz * s.sz + (long long)sy * s.sy + sx;
    return s.ghost ? vg[q * NG + i] : v[q * N + i];
}

// boxes within one cell of a non-periodic side: a chunk beyond it (ghost =
// 2) gives the general pull, whose BC functor computes the value
// (Source/BC.H:345-471); every other chunk reads through the table
template <int q>
__device__ __forceinline__ double pull_slot_bc(const LV& L, const BCParams& P, const SlotTab& T, const DevBox& B,
                                               int x, int y, int z, uint8_t tf, const double* v, const double* vg,
                                               bool is_g, const Lattice<double>& lat)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    const int sx = x - ex, sy = y - ey, sz = z - ez;
    const int ox = ex == 0 ? (x >> T.lg[0]) + 1 : chunk_of(sx, B.n[0], T.lg[0], T.top[0]);
    const int oy = ey == 0 ? (y >> T.lg[1]) + 1 : chunk_of(sy, B.n[1], T.lg[1], T.top[1]);
    const int oz = ez == 0 ? (z >> T.lg[2]) + 1 : chunk_of(sz, B.n[2], T.lg[2], T.top[2]);
    const NbrSlot& s = T.s[ox + T.tx * (oy + T.ty * oz)];
    if (s.ghost == 2) return pull<q>(L, P, B, x, y, z, tf, false, v, vg, is_g, lat);
    const long long i = s.base + (long long)sz * s.sz + (long long)sy * s.sy + sx;
    return s.ghost ? vg[q * L.NG + i] : v[q * L.N + i];
}

// the same in a box holding solid cells: a solid source bounces back the
// target's own opposite population (the half-way bounce-back of the push,
// Source/LBM.cpp:574-598)
template <int q>
__device__ __forceinline__ double pull_slot_eb(const LV& L, const SlotTab& T, const DevBox& B, int x, int y, int z,
                                               const double* v, const double* vg)
{
    constexpr int oq = opp(q);
    if (!(flag_at(L, B, x - ev_x(q), y - ev_y(q), z - ev_z(q)) & FL_FLUID))
        return v[oq * L.N + B.voff + val_lin(B, x, y, z)];
    return pull_slot<q>(T, B, x, y, z, v, vg, L.N, L.NG);
}

template <int q>
__device__ __forceinline__ double pull_slot_eb_bc(const LV& L, const BCParams& P, const SlotTab& T, const DevBox& B,
                                                  int x, int y, int z, uint8_t tf, const double* v, const double* vg,
                                                  bool is_g, const Lattice<double>& lat)
{
    constexpr int oq = opp(q);
    if (!(flag_at(L, B, x - ev_x(q), y - ev_y(q), z - ev_z(q)) & FL_FLUID))
        return v[oq * L.N + B.voff + val_lin(B, x, y, z)];
    return pull_slot_bc<q>(L, P, T, B, x, y, z, tf, v, vg, is_g, lat);
}

// Q_corr component d at box-local neighbour (x, y, z) through the slot table
// (the macro scratch has the layout of the populations; the ghost fab's
// Q_corr scratch that of the ghost fab)
__device__ __forceinline__ double qcorr_slot(const SlotTab& T, const DevBox& B, int x, int y, int z, int d,
                                             const double* md, const double* gqc, long long N, long long NG)
{
    const int ox = chunk_of(x, B.n[0], T.lg[0], T.top[0]);
    const int oy = chunk_of(y, B.n[1], T.lg[1], T.top[1]);
    const int oz = chunk_of(z, B.n[2], T.lg[2], T.top[2]);
    const NbrSlot& s = T.s[ox + T.tx * (oy + T.ty * oz)];
    const long long i = s.base + (long long)z * s.sz + (long long)y * s.sy + x;
    return s.ghost ? gqc[d * NG + i] : md[(MD_QCX + d) * N + i];
}

// gradient() of Source/Utilities.H:279-312 through the slot table: one-sided
// at the domain box and, in boxes holding solids (EB), at solid neighbours
template <bool EB>
__device__ __forceinline__ double qgrad_slot(const LV& L, const SlotTab& T, const DevBox& B, int x, int y, int z,
                                             int d, double idx, const double* md, const double* gqc)
{
    int pp[3] = {x, y, z}, pm[3] = {x, y, z};
    pp[d] += 1;
    pm[d] -= 1;
    bool p_out = B.lo[d] + pp[d] > L.dhi[d];
    bool m_out = B.lo[d] + pm[d] < L.dlo[d];
    if (EB) {
        p_out = p_out || !(flag_at(L, B, pp[0], pp[1], pp[2]) & FL_FLUID);
        m_out = m_out || !(flag_at(L, B, pm[0], pm[1], pm[2]) & FL_FLUID);
    }
    double vp = 0.0, vc = 0.0, vm = 0.0;
    if (p_out && m_out) {
        vp = 0.0; vc = 0.0; vm = 0.0;
    } else if (p_out) {
        vp = 0.0;
        vc = qcorr_slot(T, B, x, y, z, d, md, gqc, L.N, L.NG);
        vm = -qcorr_slot(T, B, pm[0], pm[1], pm[2], d, md, gqc, L.N, L.NG);
    } else if (m_out) {
        vp = qcorr_slot(T, B, pp[0], pp[1], pp[2], d, md, gqc, L.N, L.NG);
        vc = -qcorr_slot(T, B, x, y, z, d, md, gqc, L.N, L.NG);
        vm = 0.0;
    } else {
        vp = 0.5 * qcorr_slot(T, B, pp[0], pp[1], pp[2], d, md, gqc, L.N, L.NG);
        vc = 0.0;
        vm = -0.5 * qcorr_slot(T, B, pm[0], pm[1], pm[2], d, md, gqc, L.N, L.NG);
    }
    return (vp + vc + vm) * idx;
}

// the CTA's tile: its box's slot table in shared memory, the thread's cell
template <int MODE>
__device__ __forceinline__ bool tile_setup(const LV& L, const LevelPlan& lp, const Tile* tiles, NbrSlot* sl,
                                           SlotTab& T, int& b, int& x, int& y, int& z, long long& c)
{
    if (MODE > 0) {
        const int box = tiles[blockIdx.x].box;
        const DevBox& B = L.box[box];
        int tc[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            T.lg[d] = lp.slot_lg[d];
            tc[d] = ((B.n[d] + (1 << T.lg[d]) - 1) >> T.lg[d]) + 2;
            T.top[d] = tc[d] - 1;
        }
        T.tx = tc[0];
        T.ty = tc[1];
        T.s = sl;
        const int n = tc[0] * tc[1] * tc[2];
        const NbrSlot* src = lp.slots + lp.slot_off[box];
        for (int i = threadIdx.x; i < n; i += blockDim.x) sl[i] = src[i];
        __syncthreads();
    }
    return cell_of_tile(L, tiles, b, x, y, z, c);
}

// ---- pass 1: stream + macro fields ----------------------------------------
// MODE 0: general pull; 1: neighbour slots, all-fluid box; 2: neighbour
// slots, box holding solid cells; 3 and 4: the same for boxes within one cell
// of a non-periodic side (chunks beyond it through the BC functor)
template <int MODE>
__global__ void __launch_bounds__(TILE_CELLS) k_moments(LV L, LevelPlan lp, BCParams P, Phys64 ph, const Tile* tiles,
                                                        const double* fA, const double* gA, const double* fAg,
                                                        const double* gAg, const double* fB, const double* gB,
                                                        double* md)
{
    extern __shared__ NbrSlot sl[];
    SlotTab T;
    int b, x, y, z;
    long long c;
    if (!tile_setup<MODE>(L, lp, tiles, sl, T, b, x, y, z, c)) return;
    const DevBox& B = L.box[b];
    const uint8_t tf = flag_at(L, B, x, y, z);
    if (!(tf & FL_FLUID)) return;
    const bool ovr = tf & FL_OVR;
    const bool interior = !ovr && is_interior(B, x, y, z);
    const long long cell = B.voff + c;
    MomentAcc<double> acc;
#define MBG_PULLF(q) (MODE == 1 ? pull_slot<q>(T, B, x, y, z, fA, fAg, L.N, L.NG)                  \
                     : MODE == 2 ? pull_slot_eb<q>(L, T, B, x, y, z, fA, fAg)                       \
                     : MODE == 3 ? pull_slot_bc<q>(L, P, T, B, x, y, z, tf, fA, fAg, false, ph.lat)  \
                     : MODE == 4 ? pull_slot_eb_bc<q>(L, P, T, B, x, y, z, tf, fA, fAg, false, ph.lat) \
                                 : pull<q>(L, P, B, x, y, z, tf, interior, fA, fAg, false, ph.lat))
#define MBG_PULLG(q) (MODE == 1 ? pull_slot<q>(T, B, x, y, z, gA, gAg, L.N, L.NG)                  \
                     : MODE == 2 ? pull_slot_eb<q>(L, T, B, x, y, z, gA, gAg)                       \
                     : MODE == 3 ? pull_slot_bc<q>(L, P, T, B, x, y, z, tf, gA, gAg, true, ph.lat)   \
                     : MODE == 4 ? pull_slot_eb_bc<q>(L, P, T, B, x, y, z, tf, gA, gAg, true, ph.lat) \
                                 : pull<q>(L, P, B, x, y, z, tf, interior, gA, gAg, true, ph.lat))
#define MBG_M64(q)                                                             \
    {                                                                          \
        double fq = ovr ? fB[q * L.N + cell] : 0.0;                            \
        double gq = ovr ? gB[q * L.N + cell] : 0.0;                            \
        if (!ovr || is_noovr(fq)) fq = MBG_PULLF(q);                           \
        if (!ovr || is_noovr(gq)) gq = MBG_PULLG(q);                           \
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
template <int MODE>
__global__ void __launch_bounds__(TILE_CELLS) k_collide(LV L, LevelPlan lp, BCParams P, Phys64 ph, const Tile* tiles,
                                                        const double* fA, const double* gA, const double* fAg,
                                                        const double* gAg, double* fB, double* gB,
                                                        const double* md, const double* gqc)
{
    extern __shared__ NbrSlot sl[];
    SlotTab T;
    int b, x, y, z;
    long long c;
    if (!tile_setup<MODE>(L, lp, tiles, sl, T, b, x, y, z, c)) return;
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
    double dqx, dqy, dqz;
    if (MODE > 0) {
        dqx = qgrad_slot<MODE == 2 || MODE == 4>(L, T, B, x, y, z, 0, ph.idx[0], md, gqc);
        dqy = qgrad_slot<MODE == 2 || MODE == 4>(L, T, B, x, y, z, 1, ph.idx[1], md, gqc);
        dqz = qgrad_slot<MODE == 2 || MODE == 4>(L, T, B, x, y, z, 2, ph.idx[2], md, gqc);
    } else {
        dqx = qgrad(L, B, x, y, z, 0, ph.idx[0], md, gqc);
        dqy = qgrad(L, B, x, y, z, 1, ph.idx[1], md, gqc);
        dqz = qgrad(L, B, x, y, z, 2, ph.idx[2], md, gqc);
    }
    Equilibrium<double> E;
    const double omega =
        build_equilibrium<double>(m, dqx, dqy, dqz, ph.nu, ph.alpha, ph.dt, ph.Rg, ph.cv, ph.lat, E);
#define MBG_RF64(q)                                                                                  \
    {                                                                                                \
        double fq = ovr ? fB[q * N + cell] : 0.0;                                                    \
        if (!ovr || is_noovr(fq)) fq = MBG_PULLF(q);                                                 \
        const double feq = E.template feq<q>();                                                      \
        fB[q * N + cell] = fq + omega * (feq - fq);                                                  \
    }
#define MBG_RG64(q)                                                                                  \
    {                                                                                                \
        double gq = ovr ? gB[q * N + cell] : 0.0;                                                    \
        if (!ovr || is_noovr(gq)) gq = MBG_PULLG(q);                                                 \
        const double geq = E.template geq<q>(ph.lat);                                                \
        gB[q * N + cell] = gq + omega * (geq - gq);                                                  \
    }
    MBG_UNROLL27(MBG_RF64)
    MBG_UNROLL27(MBG_RG64)
#undef MBG_RF64
#undef MBG_RG64
#undef MBG_PULLF
#undef MBG_PULLG
}

static inline size_t slot_bytes(const LevelPlan& lp) { return (size_t)lp.slot_max * sizeof(NbrSlot); }

}  // namespace mbg
