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

// ---- derived fields of the current state (Source/LBM.cpp:909-991) ------------
// macro fields of the stored populations of box-local cell (x, y, z): its own
// valid cell, the owning box's (periodic images included) or, in the
// coarse-fine shell, the box's ghost fab -- what f_to_macrodata computes over
// the box grown by one (Source/LBM.cpp:810-906)
__device__ __forceinline__ Macro<double> stored_macro(const LV& L, const Phys64& ph, const DevBox& B, int x, int y,
                                                      int z, const double* f, const double* g, const double* fg,
                                                      const double* gg)
{
    MomentAcc<double> acc;
#define MBG_SM64(q) acc.template add<q>(fab_value(L, B, x, y, z, q, f, fg), fab_value(L, B, x, y, z, q, g, gg));
    MBG_UNROLL27(MBG_SM64)
#undef MBG_SM64
    return acc.finish(ph.mesh_speed, ph.Rg, ph.cv);
}

__device__ __forceinline__ double macro_comp(const Macro<double>& m, int c)
{
    switch (c) {
    case MD_U: return m.u;
    case MD_V: return m.v;
    case MD_W: return m.w;
    case MD_QCX: return m.qcx;
    case MD_QCY: return m.qcy;
    case MD_QCZ: return m.qcz;
    default: return m.rho;
    }
}

// gradient() of Source/Utilities.H:279-312 along axis d of the macro
// components comps[0..n) at once: central in the interior, one-sided where a
// neighbour lies outside the domain box or is not fluid, 0 if both do
template <int NC>
__device__ __forceinline__ void grad_stored(const LV& L, const Phys64& ph, const DevBox& B, int x, int y, int z,
                                            int d, const Macro<double>& mc, const double* f, const double* g,
                                            const double* fg, const double* gg, const int (&comps)[NC],
                                            double (&out)[NC])
{
    int pp[3] = {x, y, z}, pm[3] = {x, y, z};
    pp[d] += 1;
    pm[d] -= 1;
    const bool p_out = B.lo[d] + pp[d] > L.dhi[d] || !(flag_at(L, B, pp[0], pp[1], pp[2]) & FL_FLUID);
    const bool m_out = B.lo[d] + pm[d] < L.dlo[d] || !(flag_at(L, B, pm[0], pm[1], pm[2]) & FL_FLUID);
    Macro<double> mp = mc, mm = mc;
    if (!p_out) mp = stored_macro(L, ph, B, pp[0], pp[1], pp[2], f, g, fg, gg);
    if (!m_out) mm = stored_macro(L, ph, B, pm[0], pm[1], pm[2], f, g, fg, gg);
    for (int k = 0; k < NC; ++k) {
        const double a = macro_comp(mp, comps[k]), c = macro_comp(mc, comps[k]), m = macro_comp(mm, comps[k]);
        double vp = 0.0, vc = 0.0, vm = 0.0;
        if (p_out && m_out) {
            vp = 0.0; vc = 0.0; vm = 0.0;
        } else if (p_out) {
            vp = 0.0; vc = c; vm = -m;
        } else if (m_out) {
            vp = a; vc = -c; vm = 0.0;
        } else {
            vp = 0.5 * a; vc = 0.0; vm = -0.5 * m;
        }
        out[k] = (vp + vc + vm) * ph.idx[d];
    }
}

// vort_x, vort_y, vort_z, vort_mag, dQCorrX, dQCorrY, dQCorrZ per fluid cell
// (0 elsewhere), host layout [box][7][cell]
__global__ void k_derived(LV L, Phys64 ph, const Tile* tiles, const double* f, const double* g, const double* fg,
                          const double* gg, double* out7)
{
    int b, x, y, z;
    long long c;
    if (!cell_of_tile(L, tiles, b, x, y, z, c)) return;
    const DevBox& B = L.box[b];
    const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
    double* o = out7 + B.hoff * 7 + c;
    if (!(flag_at(L, B, x, y, z) & FL_FLUID)) {
        for (int k = 0; k < 7; ++k) o[k * vol] = 0.0;
        return;
    }
    const Macro<double> mc = stored_macro(L, ph, B, x, y, z, f, g, fg, gg);
    double gx[3], gy[3], gz[3];
    grad_stored(L, ph, B, x, y, z, 0, mc, f, g, fg, gg, {MD_V, MD_W, MD_QCX}, gx);   // vx, wx, dQx
    grad_stored(L, ph, B, x, y, z, 1, mc, f, g, fg, gg, {MD_U, MD_W, MD_QCY}, gy);   // uy, wy, dQy
    grad_stored(L, ph, B, x, y, z, 2, mc, f, g, fg, gg, {MD_U, MD_V, MD_QCZ}, gz);   // uz, vz, dQz
    const double vx = gx[0], wx = gx[1], uy = gy[0], wy = gy[1], uz = gz[0], vz = gz[1];
    o[0] = wy - vz;
    o[vol] = uz - wx;
    o[2 * vol] = vx - uy;
    o[3 * vol] = sqrt((wy - vz) * (wy - vz) + (uz - wx) * (uz - wx) + (vx - uy) * (vx - uy));
    o[4 * vol] = gx[2];
    o[5 * vol] = gy[2];
    o[6 * vol] = gz[2];
}

// ---- EB momentum-exchange force (Source/LBM.cpp:994-1044) -------------------
// Each eb_boundary cell not covered by a finer level sums 2 e_q f(x - e_q, q)
// over its fluid neighbours in FP64; the block reduces its cells' sums by warp
// shuffles and a fixed tree over the warps and writes one partial per block,
// and k_sum_partials adds the partials of all levels in a fixed order: the
// result does not depend on the schedule (no atomics), run after run.
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(TILE_CELLS) k_eb_forces(LV L, const Tile* tiles, const double* f, const double* fg,
                                                          double* partial3)
{
    __shared__ double red[3][TILE_CELLS / 32];
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
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = 0; d < 3; ++d) {
        const double v = warp_sum(fs[d]);
        if (lane == 0) red[d][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int w = 0; w < TILE_CELLS / 32; ++w) s += red[threadIdx.x][w];
        partial3[(long long)blockIdx.x * 3 + threadIdx.x] = s;
    }
}

// out3 = sum of n partials (3 components each), in a fixed order: each of
// the 256 threads sums a fixed strided subset, then a fixed tree
__global__ void __launch_bounds__(256) k_sum_partials(const double* partial3, long long n, double* out3)
{
    __shared__ double red[3][256];
    double s[3] = {0.0, 0.0, 0.0};
    for (long long i = threadIdx.x; i < n; i += 256)
        for (int d = 0; d < 3; ++d) s[d] += partial3[i * 3 + d];
    for (int d = 0; d < 3; ++d) red[d][threadIdx.x] = s[d];
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int d = 0; d < 3; ++d) red[d][threadIdx.x] += red[d][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x < 3) out3[threadIdx.x] = red[threadIdx.x][0];
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

// NaN and sentinel scan of one level's FP64 (or decoded) state: counts of
// bad values at fluid and at solid cells into out[0..1], the first bad value
// (level, box, cell, 2 q + lattice as one ordered key) by an integer
// minimum into out[2] -- both order-free, so the result is the same bits on
// every call
__global__ void __launch_bounds__(TILE_CELLS) k_check(LV L, const Tile* __restrict__ tiles,
                                                      const double* __restrict__ f, const double* __restrict__ g,
                                                      int lev, unsigned long long* __restrict__ out)
{
    int b, x, y, z;
    long long c;
    if (!cell_of_tile(L, tiles, b, x, y, z, c)) return;
    const DevBox& B = L.box[b];
    const uint8_t tf = flag_at(L, B, x, y, z);
    const long long cell = B.voff + c;
    const bool fluid = tf & FL_FLUID;
    const bool ovr = tf & FL_OVR;
    unsigned bad = 0u;
    int first = -1;
    for (int q = 0; q < NQ; ++q)
        for (int lat = 0; lat < 2; ++lat) {
            const double v = (lat ? g : f)[q * L.N + cell];
            const bool wrong = fluid ? (!isfinite(v) || v == -1.0) : (!ovr && v != -1.0);
            if (wrong) {
                ++bad;
                if (first < 0) first = 2 * q + lat;
            }
        }
    if (bad) {
        atomicAdd(&out[fluid ? 0 : 1], (unsigned long long)bad);
        const unsigned long long key = ((unsigned long long)lev << 58) | ((unsigned long long)b << 38) |
                                       ((unsigned long long)c << 7) | (unsigned long long)first;
        atomicMin(&out[2], key);
    }
}

void launch_check(const LevelPlan& lp, const double* f, const double* g, int lev, unsigned long long* out,
                  cudaStream_t s)
{
    if (lp.ntiles > 0) k_check<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, lp.tiles, f, g, lev, out);
}

// host layout [box][q][cell] <-> the FP64 state [q][N]: the staging pass of
// mbg_set_state / mbg_get_state (one contiguous copy over the link instead
// of one strided copy per box and lattice)
__global__ void __launch_bounds__(TILE_CELLS) k_stage(LV L, const Tile* __restrict__ tiles,
                                                      double* __restrict__ stage, double* __restrict__ v, int to_state)
{
    int b, x, y, z;
    long long c;
    if (!cell_of_tile(L, tiles, b, x, y, z, c)) return;
    const DevBox& B = L.box[b];
    const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
    double* h = stage + B.hoff * NQ + c;
    double* d = v + B.voff + c;
    if (to_state) {
#pragma unroll 9
        for (int q = 0; q < NQ; ++q) d[q * L.N] = h[q * vol];
    } else {
#pragma unroll 9
        for (int q = 0; q < NQ; ++q) h[q * vol] = d[q * L.N];
    }
}

void launch_stage(const LevelPlan& lp, double* stage, double* v, int to_state, cudaStream_t s)
{
    if (lp.ntiles > 0) k_stage<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, lp.tiles, stage, v, to_state);
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

void launch_eb_forces(const LevelPlan& lp, const double* f, const double* fg, double* partial3, cudaStream_t s)
{
    if (lp.ntiles == 0) return;
    k_eb_forces<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, lp.tiles, f, fg, partial3);
}

void launch_sum_partials(const double* partial3, long long n, double* out3, cudaStream_t s)
{
    k_sum_partials<<<1, 256, 0, s>>>(partial3, n, out3);
}

void launch_derived(const LevelPlan& lp, const Phys64& ph, const double* f, const double* g, const double* fg,
                    const double* gg, double* out7, cudaStream_t s)
{
    if (lp.ntiles == 0) return;
    k_derived<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, ph, lp.tiles, f, g, fg, gg, out7);
}

// ---- ErrorEst tags (Source/LBM.cpp:1597-1611, AMReX AMRErrorTag) ------------
struct Geo3 {
    double plo[3], dx[3];
};

__global__ void k_tags(LV L, Phys64 ph, const Tile* tiles, const double* md, const double* f, const double* g,
                       TagSet ts, double time, int lev, Geo3 geo, uint8_t* out)
{
    int b, x, y, z;
    long long c;
    if (!cell_of_tile(L, tiles, b, x, y, z, c)) return;
    const DevBox& B = L.box[b];
    const uint8_t tf = flag_at(L, B, x, y, z);
    const long long cell = B.voff + c;
    double m[19];
    bool have = false;
    uint8_t t = 0;
    for (int k = 0; k < ts.n; ++k) {
        const mbg_tag& tg = ts.t[k];
        if (!(time >= tg.start_time && time <= tg.end_time) || lev >= tg.max_level) continue;
        if (tg.has_box) {
            const int p[3] = {B.lo[0] + x, B.lo[1] + y, B.lo[2] + z};
            bool in = true;
            for (int d = 0; d < 3; ++d) {
                const double xc = geo.plo[d] + (p[d] + 0.5) * geo.dx[d];
                in &= xc >= tg.box_lo[d] && xc <= tg.box_hi[d];
            }
            if (!in) continue;
        }
        if (tg.kind == 0) { t = 1; continue; }
        double v;
        if (tg.field == 19) {
            v = (tf & FL_FLUID) ? 1.0 : 0.0;
        } else {
            if (!have) {
                have = true;
                if (!(tf & FL_FLUID)) {
                    for (int q = 0; q < 19; ++q) m[q] = 0.0;   // the macro data of solid cells stays 0
                } else if (md) {
                    const long long N = L.N;
                    const double u = md[MD_U * N + cell], vv = md[MD_V * N + cell], w = md[MD_W * N + cell];
                    const double vals[19] = {md[MD_RHO * N + cell], u, vv, w, sqrt(u * u + vv * vv + w * w),
                                             md[MD_TRE * N + cell], md[MD_QCX * N + cell], md[MD_QCY * N + cell],
                                             md[MD_QCZ * N + cell], md[MD_PXX * N + cell], md[MD_PYY * N + cell],
                                             md[MD_PZZ * N + cell], md[MD_PXY * N + cell], md[MD_PXZ * N + cell],
                                             md[MD_PYZ * N + cell], md[MD_QX * N + cell], md[MD_QY * N + cell],
                                             md[MD_QZ * N + cell], md[MD_T * N + cell]};
                    for (int q = 0; q < 19; ++q) m[q] = vals[q];
                } else {
                    MomentAcc<double> acc;
#define MBG_TG64(q) acc.template add<q>(f[q * L.N + cell], g[q * L.N + cell]);
                    MBG_UNROLL27(MBG_TG64)
#undef MBG_TG64
                    const Macro<double> a = acc.finish(ph.mesh_speed, ph.Rg, ph.cv);
                    const double vals[19] = {a.rho, a.u, a.v, a.w, sqrt(a.u * a.u + a.v * a.v + a.w * a.w),
                                             a.two_rho_e, a.qcx, a.qcy, a.qcz, a.pxx, a.pyy, a.pzz, a.pxy, a.pxz,
                                             a.pyz, a.qx, a.qy, a.qz, a.temp};
                    for (int q = 0; q < 19; ++q) m[q] = vals[q];
                }
            }
            v = m[tg.field];
        }
        if ((tg.kind == 1 && v > tg.value) || (tg.kind == 2 && v < tg.value)) t = 1;
    }
    out[B.hoff + c] = t;
}

void launch_tags(const LevelPlan& lp, const Phys64& ph, const double* md, const double* f, const double* g,
                 const TagSet& ts, double time, int lev, const double plo[3], const double dx[3], uint8_t* out,
                 cudaStream_t s)
{
    if (lp.ntiles == 0) return;
    Geo3 geo;
    for (int d = 0; d < 3; ++d) { geo.plo[d] = plo[d]; geo.dx[d] = dx[d]; }
    k_tags<<<lp.ntiles, TILE_CELLS, 0, s>>>(lp.view64, ph, lp.tiles, md, f, g, ts, time, lev, geo, out);
}

}  // namespace mbg
