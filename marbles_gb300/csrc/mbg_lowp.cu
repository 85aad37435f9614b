// mbg_lowp.cu -- FP32-arithmetic / 16-bit-storage form of the level step.
//
// Storage.  Each population is kept as a 16-bit float (FP16 or BF16) holding
// its scaled deviation from the equilibrium at the reference state
// (rho_ref, u_ref, T_ref):  f = f_rest[q] + scale[q] * h.  scale[q] is the rest
// value itself for f (h is then the relative deviation) and the rest value of
// g floored at 1e-3 w_q (2 rho E)_ref (g_rest vanishes for some directions).
// The stream's -1 sentinel (solid cells, unreached ghosts) is the code 0xFFFF,
// a NaN in both formats, decoded to exactly -1.
//
// Arithmetic.  FP32 throughout the collision; FP64 only where sums of many
// terms meet: the coalescence averages and the output moments.
//
// One level advance is one fused pass (k_fused): a CTA owns a 32 x 8 column
// tile of a box and marches through 8 planes.  For each plane it pulls the 54
// streamed values of its cells, forms the moments and Q_corr, and keeps Q_corr
// of the tile plus a one-cell halo in shared memory (halo cells are computed
// from the perspective of the box that owns them, so the coarse-fine ghost
// semantics match the reference); the previous plane is then collided:
// q-correction gradient from shared memory, equilibria, relaxation, with its
// 54 values pulled again from L1/L2.  DRAM sees each population read once and
// written once.
//
// Code size.  Everything a kernel needs lives in one device-resident LowpK per
// level and buffer parity, read through a restrict pointer.  Interior cells
// take an inline pull (the codec table passed by value, so its entries are
// constant-bank operands); every other pull -- box faces, other boxes,
// coarse-fine ghosts, physical BCs, solid neighbours -- is one non-inlined
// function per direction.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

#include "mbg_lowp.h"

namespace mbg {

using u16 = uint16_t;
using LV16 = LevelView<u16>;

constexpr u16 SENT16 = 0xFFFFu;
constexpr int FT_X = 32;   // fused tile width (one warp)
constexpr int FT_Y = 8;    // fused tile height (warps per CTA)
constexpr int FT_Z = 8;    // planes a CTA marches through

struct CodecTab {
    float frest[NQ], grest[NQ], fsc[NQ], gsc[NQ], fisc[NQ], gisc[NQ];
};

template <bool BF>
__device__ __forceinline__ float h2f(u16 r)
{
    if constexpr (BF) return __uint_as_float(((unsigned)r) << 16);
    else return __half2float(__ushort_as_half(r));
}
template <bool BF>
__device__ __forceinline__ u16 f2h(float v)
{
    if constexpr (BF) return __bfloat16_as_ushort(__float2bfloat16_rn(v));
    else return __half_as_ushort(__float2half_rn(v));
}
template <bool BF>
__device__ __forceinline__ float dec(const CodecTab& ct, u16 r, int q, bool g)
{
    if (r == SENT16) return -1.0f;
    return g ? fmaf(h2f<BF>(r), ct.gsc[q], ct.grest[q]) : fmaf(h2f<BF>(r), ct.fsc[q], ct.frest[q]);
}
template <bool BF>
__device__ __forceinline__ u16 enc(const CodecTab& ct, float v, int q, bool g)
{
    if (v == -1.0f) return SENT16;
    const float h = g ? (v - ct.grest[q]) * ct.gisc[q] : (v - ct.frest[q]) * ct.fisc[q];
    const u16 r = f2h<BF>(h);
    return r == SENT16 ? (u16)0xFFFEu : r;
}

struct Bufs16 {
    const u16 *f, *g, *fg, *gg;   // source state (valid, ghost)
    const u16 *fo, *go;           // coalescence override (coarse levels), or null
};

// everything the kernels of one level read, for one buffer parity
struct LowpK {
    LV16 L;
    BCParams P;
    Phys32 ph;
    CodecTab ct;
    Lattice<double> lat64;
    Bufs16 s;                      // source: the current state
    u16 *fB, *gB, *fBg, *gBg;      // destination: the other buffer
};

// general pull (everything but an interior cell of an all-fluid box), the
// 16-bit counterpart of mbg_fp64.cu's pull; which: bit 0 = g lattice
template <int q, bool BF>
__device__ __noinline__ float pull16_slow(const LowpK* __restrict__ K, int b, int x, int y, int z, uint8_t tflag,
                                          int which)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    constexpr int oq = opp(q);
    const bool is_g = which & 1;
    const u16* v = is_g ? K->s.g : K->s.f;
    const u16* vg = is_g ? K->s.gg : K->s.fg;
    const LV16& L = K->L;
    const DevBox& B = L.box[b];
    if (!(tflag & FL_FLUID)) return -1.0f;
    const int sx = x - ex, sy = y - ey, sz = z - ez;
    if (sx < -3 || sy < -3 || sz < -3 || sx > B.n[0] + 2 || sy > B.n[1] + 2 || sz > B.n[2] + 2) return -1.0f;
    const uint8_t sf = flag_at(L, B, sx, sy, sz);
    if (!(sf & FL_FLUID)) return dec<BF>(K->ct, fab_value(L, B, x, y, z, oq, v, vg), oq, is_g);
    int gp[3] = {B.lo[0] + sx, B.lo[1] + sy, B.lo[2] + sz};
    if (outside_nonperiodic(L, gp))
        return bc_value<q, u16, float>(L, K->P, B, sx, sy, sz, is_g, v, vg, K->lat64,
                                       [&](u16 r, int slot) { return dec<BF>(K->ct, r, slot, is_g); });
    return dec<BF>(K->ct, fab_value(L, B, sx, sy, sz, q, v, vg), q, is_g);
}

// cached view of the box a thread works in
struct BoxReg {
    int n0, n1, n2;
    long long voff, N;
    bool all_fluid;
};

// interior pull: the source is inside the same box and fluid
template <int q, bool BF>
__device__ __forceinline__ float pull16_in(const CodecTab& ct, const BoxReg& R, int x, int y, int z,
                                           const u16* __restrict__ v, bool is_g)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    const long long i = q * R.N + R.voff + ((long long)(z - ez) * R.n1 + (y - ey)) * R.n0 + (x - ex);
    return dec<BF>(ct, __ldg(v + i), q, is_g);
}

// moments of the streamed values at box-local (x, y, z) of box b; a cell
// overwritten by coalescence reads the override buffer instead
template <bool BF>
__device__ __noinline__ MomentAcc<float> moments16_slow(const LowpK* __restrict__ K, int b, int x, int y, int z,
                                                        uint8_t tf)
{
    MomentAcc<float> acc;
    const LV16& L = K->L;
    const DevBox& B = L.box[b];
    const bool ovr = (tf & FL_OVR) && in_valid<u16>(B, x, y, z) && K->s.fo;
    const long long cell = B.voff + (in_valid<u16>(B, x, y, z) ? val_lin(B, x, y, z) : 0);
#define MBG_MS16(q)                                                                  \
    {                                                                                \
        float fq, gq;                                                                \
        if (ovr) {                                                                   \
            fq = dec<BF>(K->ct, K->s.fo[q * L.N + cell], q, false);                  \
            gq = dec<BF>(K->ct, K->s.go[q * L.N + cell], q, true);                   \
        } else {                                                                     \
            fq = pull16_slow<q, BF>(K, b, x, y, z, tf, 0);                           \
            gq = pull16_slow<q, BF>(K, b, x, y, z, tf, 1);                           \
        }                                                                            \
        acc.template add<q>(fq, gq);                                                 \
    }
    MBG_UNROLL27(MBG_MS16)
#undef MBG_MS16
    return acc;
}

// Q_corr component d at box-local position (x, y, z) of box b, as the
// reference's macro FillBoundary leaves it: computed by the box that owns the
// cell, or by box b itself where no box covers it
template <bool BF>
__device__ __noinline__ float qcorr_pos(const LowpK* __restrict__ K, int b, int x, int y, int z, int d)
{
    const LV16& L = K->L;
    const DevBox& B = L.box[b];
    int vb = b, lx = x, ly = y, lz = z;
    if (!in_valid<u16>(B, x, y, z)) {
        int p[3] = {B.lo[0] + x, B.lo[1] + y, B.lo[2] + z};
        if (!wrap_pos(L, p)) return 0.0f;
        const int o = owner_of(L, p);
        if (o >= 0) {
            vb = o;
            const DevBox& O = L.box[o];
            lx = p[0] - O.lo[0];
            ly = p[1] - O.lo[1];
            lz = p[2] - O.lo[2];
        }
    }
    const uint8_t tf = flag_at(L, L.box[vb], lx, ly, lz);
    if (!(tf & FL_FLUID)) return 0.0f;
    const Macro<float> m = moments16_slow<BF>(K, vb, lx, ly, lz, tf).finish(K->ph.mesh_speed, K->ph.Rg, K->ph.cv);
    return d == 0 ? m.qcx : d == 1 ? m.qcy : m.qcz;
}

struct FusedTile {
    int box;
    short x0, y0, z0, z1;
};

// neighbour along d is part of the gradient stencil (Utilities.H:279-312)
__device__ __forceinline__ bool present(const LV16& L, const DevBox& B, int x, int y, int z, int d, int s)
{
    int p[3] = {x, y, z};
    p[d] += s;
    const int gd = B.lo[d] + p[d];
    if (gd < L.dlo[d] || gd > L.dhi[d]) return false;
    return flag_at(L, B, p[0], p[1], p[2]) & FL_FLUID;
}

__device__ __forceinline__ float grad1(bool pin, bool min, float vpv, float vcv, float vmv, float idx)
{
    float vp = 0.f, vc = 0.f, vm = 0.f;
    if (!pin && !min) {
    } else if (!pin) {
        vc = vcv; vm = -vmv;
    } else if (!min) {
        vp = vpv; vc = -vcv;
    } else {
        vp = 0.5f * vpv; vm = -0.5f * vmv;
    }
    return (vp + vc + vm) * idx;
}

template <bool BF>
__global__ void __launch_bounds__(FT_X * FT_Y, 2) k_fused(const LowpK* __restrict__ K, const CodecTab ct,
                                                          const FusedTile* __restrict__ tiles)
{
    __shared__ float sqx[2][FT_Y][FT_X + 2];
    __shared__ float sqy[2][FT_Y + 2][FT_X];
    __shared__ float sqz[3][FT_Y][FT_X];
    const FusedTile t = tiles[blockIdx.x];
    const LV16& L = K->L;
    const DevBox& B = L.box[t.box];
    BoxReg R;
    R.n0 = B.n[0]; R.n1 = B.n[1]; R.n2 = B.n[2];
    R.voff = B.voff;
    R.N = L.N;
    R.all_fluid = B.all_fluid;
    const u16* __restrict__ sf = K->s.f;
    const u16* __restrict__ sg = K->s.g;
    const u16* __restrict__ sfo = K->s.fo;
    const u16* __restrict__ sgo = K->s.go;
    u16* __restrict__ fB = K->fB;
    u16* __restrict__ gB = K->gB;
    const float ms = K->ph.mesh_speed, Rg = K->ph.Rg, cv = K->ph.cv;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = t.x0 + tx, y = t.y0 + ty;
    const bool mine = x < R.n0 && y < R.n1;
    const int tid = ty * FT_X + tx;
    const int z0 = t.z0, z1 = t.z1;
    Macro<float> prev, cur;
    uint8_t prevf = 0, curf = 0;
    for (int z = z0 - 1; z <= z1; ++z) {
        // ---- phase A: moments and Q_corr of plane z ----
        const int ia = z & 1, iz = (z + 3) % 3;
        if (mine) {
            if (z >= z0 && z < z1) {
                const uint8_t tf = flag_at(L, B, x, y, z);
                float qx = 0.f, qy = 0.f, qz = 0.f;
                if (tf & FL_FLUID) {
                    const bool ovr = (tf & FL_OVR) && sfo;
                    const bool interior = !ovr && R.all_fluid && x > 0 && y > 0 && z > 0 && x < R.n0 - 1 &&
                                          y < R.n1 - 1 && z < R.n2 - 1;
                    MomentAcc<float> acc;
                    if (interior) {
#define MBG_MF16(q) \
    acc.template add<q>(pull16_in<q, BF>(ct, R, x, y, z, sf, false), pull16_in<q, BF>(ct, R, x, y, z, sg, true));
                        MBG_UNROLL27(MBG_MF16)
#undef MBG_MF16
                    } else {
                        acc = moments16_slow<BF>(K, t.box, x, y, z, tf);
                    }
                    cur = acc.finish(ms, Rg, cv);
                    qx = cur.qcx; qy = cur.qcy; qz = cur.qcz;
                }
                curf = tf;
                sqx[ia][ty][tx + 1] = qx;
                sqy[ia][ty + 1][tx] = qy;
                sqz[iz][ty][tx] = qz;
            } else {
                // z-halo plane: Q_corr_z only, where the gradient will read it
                const int zz = z < z0 ? z0 : z1 - 1;
                const int s_ = z < z0 ? -1 : 1;
                float v = 0.f;
                if (present(L, B, x, y, zz, 2, s_)) v = qcorr_pos<BF>(K, t.box, x, y, z, 2);
                sqz[iz][ty][tx] = v;
            }
        }
        if (z >= z0 && z < z1) {
            // x- and y-halo of the tile in this plane
            const int tw = R.n0 - t.x0 < FT_X ? R.n0 - t.x0 : FT_X;
            const int th = R.n1 - t.y0 < FT_Y ? R.n1 - t.y0 : FT_Y;
            const int nh = 2 * th + 2 * tw;
            for (int h = tid; h < nh; h += FT_X * FT_Y) {
                if (h < 2 * th) {
                    const int j = h >> 1, side = h & 1;
                    const int hx = side ? t.x0 + tw : t.x0 - 1, hy = t.y0 + j;
                    float v = 0.f;
                    if (present(L, B, side ? hx - 1 : hx + 1, hy, z, 0, side ? 1 : -1))
                        v = qcorr_pos<BF>(K, t.box, hx, hy, z, 0);
                    sqx[ia][j][side ? tw + 1 : 0] = v;
                } else {
                    const int k = h - 2 * th;
                    const int i = k >> 1, side = k & 1;
                    const int hx = t.x0 + i, hy = side ? t.y0 + th : t.y0 - 1;
                    float v = 0.f;
                    if (present(L, B, hx, side ? hy - 1 : hy + 1, z, 1, side ? 1 : -1))
                        v = qcorr_pos<BF>(K, t.box, hx, hy, z, 1);
                    sqy[ia][side ? th + 1 : 0][i] = v;
                }
            }
        }
        __syncthreads();
        // ---- phase B: collide plane z - 1 ----
        const int zc = z - 1;
        if (mine && zc >= z0 && zc < z1) {
            const int ib = zc & 1;
            const long long cell = R.voff + ((long long)zc * R.n1 + y) * R.n0 + x;
            const bool ovr = (prevf & FL_OVR) && sfo;
            if (!(prevf & FL_FLUID)) {
#define MBG_SOL16(q)                                                    \
    {                                                                   \
        fB[q * R.N + cell] = ovr ? sfo[q * R.N + cell] : SENT16;        \
        gB[q * R.N + cell] = ovr ? sgo[q * R.N + cell] : SENT16;        \
    }
                MBG_UNROLL27(MBG_SOL16)
#undef MBG_SOL16
            } else {
                const float dqx = grad1(present(L, B, x, y, zc, 0, 1), present(L, B, x, y, zc, 0, -1),
                                        sqx[ib][ty][tx + 2], sqx[ib][ty][tx + 1], sqx[ib][ty][tx], K->ph.idx[0]);
                const float dqy = grad1(present(L, B, x, y, zc, 1, 1), present(L, B, x, y, zc, 1, -1),
                                        sqy[ib][ty + 2][tx], sqy[ib][ty + 1][tx], sqy[ib][ty][tx], K->ph.idx[1]);
                const float dqz = grad1(present(L, B, x, y, zc, 2, 1), present(L, B, x, y, zc, 2, -1),
                                        sqz[(z + 3) % 3][ty][tx], sqz[(zc + 3) % 3][ty][tx],
                                        sqz[(zc - 1 + 3) % 3][ty][tx], K->ph.idx[2]);
                Equilibrium<float> E;
                const float omega = build_equilibrium<float>(prev, dqx, dqy, dqz, K->ph.nu, K->ph.alpha, K->ph.dt,
                                                             Rg, cv, K->ph.lat, E);
                const bool interior = !ovr && R.all_fluid && x > 0 && y > 0 && zc > 0 && x < R.n0 - 1 &&
                                      y < R.n1 - 1 && zc < R.n2 - 1;
                if (interior) {
#define MBG_RI16(q)                                                                                        \
    {                                                                                                      \
        const float fq = pull16_in<q, BF>(ct, R, x, y, zc, sf, false);                                     \
        fB[q * R.N + cell] = enc<BF>(ct, fmaf(omega, E.template feq<q>() - fq, fq), q, false);             \
        const float gq = pull16_in<q, BF>(ct, R, x, y, zc, sg, true);                                      \
        gB[q * R.N + cell] = enc<BF>(ct, fmaf(omega, E.template geq<q>(K->ph.lat) - gq, gq), q, true);     \
    }
                    MBG_UNROLL27(MBG_RI16)
#undef MBG_RI16
                } else {
#define MBG_RS16(q)                                                                                        \
    {                                                                                                      \
        const float fq = ovr ? dec<BF>(ct, sfo[q * R.N + cell], q, false)                                  \
                             : pull16_slow<q, BF>(K, t.box, x, y, zc, prevf, 0);                           \
        fB[q * R.N + cell] = enc<BF>(ct, fmaf(omega, E.template feq<q>() - fq, fq), q, false);             \
        const float gq = ovr ? dec<BF>(ct, sgo[q * R.N + cell], q, true)                                   \
                             : pull16_slow<q, BF>(K, t.box, x, y, zc, prevf, 1);                           \
        gB[q * R.N + cell] = enc<BF>(ct, fmaf(omega, E.template geq<q>(K->ph.lat) - gq, gq), q, true);     \
    }
                    MBG_UNROLL27(MBG_RS16)
#undef MBG_RS16
                }
            }
        }
        prev = cur;
        prevf = curf;
        __syncthreads();
    }
}

// streamed values of the uncovered ghost cells of a fine level
template <bool BF>
__global__ void k_ghost_stream16(const LowpK* __restrict__ K, const GhostCell* gl, long long n)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const GhostCell gc = gl[e];
    const LV16& L = K->L;
    const DevBox& B = L.box[gc.box];
    const uint8_t tf = flag_at(L, B, gc.x, gc.y, gc.z);
    const long long gi = B.goff + fab_lin(B, gc.x, gc.y, gc.z);
#define MBG_GS16(q)                                                                                               \
    {                                                                                                             \
        K->fBg[q * L.NG + gi] = enc<BF>(K->ct, pull16_slow<q, BF>(K, gc.box, gc.x, gc.y, gc.z, tf, 0), q, false); \
        K->gBg[q * L.NG + gi] = enc<BF>(K->ct, pull16_slow<q, BF>(K, gc.box, gc.x, gc.y, gc.z, tf, 1), q, true);  \
    }
    MBG_UNROLL27(MBG_GS16)
#undef MBG_GS16
}

// explosion (conservative linear interpolation, as in mbg_fp64.cu) in FP32
template <bool BF>
__device__ __forceinline__ float crse16(const LowpK* __restrict__ KC, const int p0[3], int d, int s_, int q,
                                        bool g)
{
    int p[3] = {p0[0], p0[1], p0[2]};
    p[d] += s_;
    const LV16& C = KC->L;
    wrap_pos(C, p);
    const int o = owner_of(C, p);
    if (o < 0) return 0.0f;
    const DevBox& O = C.box[o];
    const u16* v = g ? KC->s.g : KC->s.f;
    return dec<BF>(KC->ct, v[q * C.N + O.voff + val_lin(O, p[0] - O.lo[0], p[1] - O.lo[1], p[2] - O.lo[2])], q, g);
}

template <bool BF>
__global__ void k_explode16(const LowpK* __restrict__ KF, const LowpK* __restrict__ KC, const GhostCell* gl,
                            long long n, u16* fg, u16* gg)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const LV16& F = KF->L;
    const GhostCell g = gl[e];
    const DevBox& B = F.box[g.box];
    int fp[3] = {B.lo[0] + g.x, B.lo[1] + g.y, B.lo[2] + g.z};
    wrap_pos(F, fp);
    const int cp[3] = {fp[0] >> 1, fp[1] >> 1, fp[2] >> 1};
    const float off[3] = {((fp[0] - 2 * cp[0]) + 0.5f) / 2.0f - 0.5f, ((fp[1] - 2 * cp[1]) + 0.5f) / 2.0f - 0.5f,
                          ((fp[2] - 2 * cp[2]) + 0.5f) / 2.0f - 0.5f};
    const long long gi = B.goff + fab_lin(B, g.x, g.y, g.z);
    for (int lat = 0; lat < 2; ++lat) {
        const bool isg = lat == 1;
        u16* out = isg ? gg : fg;
        float alpha[3] = {1.f, 1.f, 1.f};
        for (int d = 0; d < 3; ++d)
            for (int q = 0; q < NQ; ++q) {
                const float u0 = crse16<BF>(KC, cp, d, 0, q, isg);
                const float up = crse16<BF>(KC, cp, d, 1, q, isg);
                const float um = crse16<BF>(KC, cp, d, -1, q, isg);
                const float cen = 0.5f * (up - um);
                const float forw = 2.0f * (up - u0);
                const float back = 2.0f * (u0 - um);
                const float slp = (forw * back >= 0.f) ? fminf(fabsf(forw), fabsf(back)) : 0.f;
                if (cen != 0.f) alpha[d] = fminf(alpha[d], fminf(slp, fabsf(cen)) / fabsf(cen));
            }
        for (int q = 0; q < NQ; ++q) {
            const float u0 = crse16<BF>(KC, cp, 0, 0, q, isg);
            const float cx = 0.5f * (crse16<BF>(KC, cp, 0, 1, q, isg) - crse16<BF>(KC, cp, 0, -1, q, isg));
            const float cy = 0.5f * (crse16<BF>(KC, cp, 1, 1, q, isg) - crse16<BF>(KC, cp, 1, -1, q, isg));
            const float cz = 0.5f * (crse16<BF>(KC, cp, 2, 1, q, isg) - crse16<BF>(KC, cp, 2, -1, q, isg));
            out[q * F.NG + gi] = enc<BF>(
                KF->ct, u0 + off[0] * (alpha[0] * cx) + off[1] * (alpha[1] * cy) + off[2] * (alpha[2] * cz), q, isg);
        }
    }
}

// coalescence: FP64 masked average of the 8 fine children into the override
// buffer (advance) or the coarse state (initial average_down)
template <bool BF>
__global__ void k_coalesce16(const LowpK* __restrict__ KC, const LowpK* __restrict__ KF, const CoalesceCell* cl,
                             long long n, u16* fo, u16* go, int into_state)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const LV16& C = KC->L;
    const LV16& F = KF->L;
    const CoalesceCell cc = cl[e];
    const DevBox& O = C.box[cc.cbox];
    const DevBox& A = F.box[cc.fbox];
    const long long cell = O.voff + val_lin(O, cc.cx, cc.cy, cc.cz);
    const uint8_t tf = flag_at(C, O, cc.cx, cc.cy, cc.cz);
    const double small_num = 2.220446049250313e-16 * 1e10;
    for (int lat = 0; lat < 2; ++lat) {
        const bool isg = lat == 1;
        const u16* v = isg ? KF->s.g : KF->s.f;
        const u16* vg = isg ? KF->s.gg : KF->s.fg;
        u16* out = isg ? go : fo;
        const u16* cA = isg ? KC->s.g : KC->s.f;
#define MBG_CO16(q)                                                                                          \
        {                                                                                                    \
            double sum = 0.0, vol = 0.0;                                                                     \
            for (int kr = 0; kr < 2; ++kr)                                                                   \
                for (int jr = 0; jr < 2; ++jr)                                                               \
                    for (int ir = 0; ir < 2; ++ir) {                                                         \
                        const double fv =                                                                    \
                            dec<BF>(KF->ct, fab_value(F, A, cc.fx + ir, cc.fy + jr, cc.fz + kr, q, v, vg), q, isg); \
                        if (fabs(fv - (-1.0)) > small_num) { sum += fv; vol += 1.0; }                        \
                    }                                                                                        \
            u16 r;                                                                                           \
            if (vol > 0.0) r = enc<BF>(KC->ct, (float)(sum / vol), q, isg);                                  \
            else if (into_state) r = cA[q * C.N + cell];                                                     \
            else r = enc<BF>(KC->ct, pull16_slow<q, BF>(KC, cc.cbox, cc.cx, cc.cy, cc.cz, tf, isg ? 1 : 0), q, isg); \
            out[q * C.N + cell] = r;                                                                         \
        }
        MBG_UNROLL27(MBG_CO16)
#undef MBG_CO16
    }
}

// FP64 staging <-> 16-bit state, one thread per (cell, q)
template <bool BF>
__global__ void k_encode(const CodecTab ct, long long N, const double* src, u16* dst, int isg)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N * NQ) return;
    dst[i] = enc<BF>(ct, (float)src[i], (int)(i / N), isg != 0);
}
template <bool BF>
__global__ void k_decode(const CodecTab ct, long long N, const u16* src, double* dst, int isg)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N * NQ) return;
    dst[i] = (double)dec<BF>(ct, src[i], (int)(i / N), isg != 0);
}

// macro fields (host layout [box][19][cell]) in FP64 from the decoded state
template <bool BF>
__global__ void k_macro16(const LowpK* __restrict__ K, const CodecTab ct, const Tile* tiles, double* out19)
{
    const LV16& L = K->L;
    const Tile t = tiles[blockIdx.x];
    const DevBox& B = L.box[t.box];
    const long long c = (long long)t.start + threadIdx.x;
    const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
    if (c >= vol) return;
    const long long x = c % B.n[0], r = c / B.n[0];
    const uint8_t tf = flag_at(L, B, (int)x, (int)(r % B.n[1]), (int)(r / B.n[1]));
    double* o = out19 + B.voff * 19 + c;
    if (!(tf & FL_FLUID)) {
        for (int k = 0; k < 19; ++k) o[k * vol] = 0.0;
        return;
    }
    const long long cell = B.voff + c;
    const u16* f = K->s.f;
    const u16* g = K->s.g;
    MomentAcc<double> acc;
#define MBG_MA16(q) \
    acc.template add<q>((double)dec<BF>(ct, f[q * L.N + cell], q, false), (double)dec<BF>(ct, g[q * L.N + cell], q, true));
    MBG_UNROLL27(MBG_MA16)
#undef MBG_MA16
    const Macro<double> m = acc.finish((double)K->ph.mesh_speed, (double)K->ph.Rg, (double)K->ph.cv);
    const double vals[19] = {m.rho, m.u, m.v, m.w, sqrt(m.u * m.u + m.v * m.v + m.w * m.w), m.two_rho_e,
                             m.qcx, m.qcy, m.qcz, m.pxx, m.pyy, m.pzz, m.pxy, m.pxz, m.pyz,
                             m.qx, m.qy, m.qz, m.temp};
    for (int k = 0; k < 19; ++k) o[k * vol] = vals[k];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct LowpDev {
    CodecTab ct;
    LowpK hk[2];                 // host copies, indexed by the source parity
    bool uploaded = false;
    bool with_override = false;
    LowpK* dk = nullptr;         // device copies [2]
    FusedTile* tiles = nullptr;
    int ntiles = 0;
    u16* fo = nullptr;           // coalescence override buffers
    u16* go = nullptr;
};

static LowpDev* dev_of(LowpLevel& L) { return (LowpDev*)L.impl; }

static LevelView<u16> view16(const LevelPlan& plan)
{
    const LevelView<double>& v = plan.view64;
    LevelView<u16> w;
    w.box = v.box;
    w.nbox = v.nbox;
    for (int d = 0; d < 3; ++d) {
        w.dlo[d] = v.dlo[d];
        w.dhi[d] = v.dhi[d];
        w.per[d] = v.per[d];
        w.G[d] = v.G[d];
        w.nb[d] = v.nb[d];
    }
    w.omap = v.omap;
    w.N = v.N;
    w.NG = v.NG;
    w.flags = v.flags;
    return w;
}

static mbg_status lalloc(LowpLevel& L, void** p, size_t bytes, std::string& err)
{
    *p = nullptr;
    if (bytes == 0) return MBG_OK;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        err = std::string("cudaMalloc (16-bit form): ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? MBG_ENOMEM : MBG_ECUDA;
    }
    L.allocs.push_back(*p);
    return MBG_OK;
}

static Phys32 phys32(const mbg_params& p, double dt, const double idx[3])
{
    Phys32 ph;
    ph.mesh_speed = (float)(p.dx_outer / p.dt_outer);
    ph.Rg = (float)(28.96 / p.m_bar);
    ph.cv = (float)((28.96 / p.m_bar) / (p.adiabatic_exponent - 1.0));
    ph.nu = (float)p.nu;
    ph.alpha = (float)p.alpha;
    ph.dt = (float)dt;
    for (int d = 0; d < 3; ++d) ph.idx[d] = (float)idx[d];
    ph.small_num = 0.f;
    ph.lat = make_lattice<float>();
    return ph;
}

static Bufs16 bufs(const LowpLevel& L, int b)
{
    Bufs16 s;
    s.f = (const u16*)L.f[b];
    s.g = (const u16*)L.g[b];
    s.fg = (const u16*)L.fg[b];
    s.gg = (const u16*)L.gg[b];
    s.fo = nullptr;
    s.go = nullptr;
    return s;
}

mbg_status lowp_define(const mbg_params& p, const LevelPlan& plan, const std::vector<DevBox>& hbox, long long N,
                       long long NG, double dt, const double idx[3], LowpLevel& L, std::string& err)
{
    L.precision = p.precision;
    L.N = N;
    L.NG = NG;
    L.ph = phys32(p, dt, idx);
    auto* D = new LowpDev();
    L.impl = D;
    const Lattice<double> lat64 = make_lattice<double>();
    // equilibria at the reference state and the scales
    const double Rg = 28.96 / p.m_bar;
    const double vel0[3] = {p.u_ref[0], p.u_ref[1], p.u_ref[2]};
    const double rho = p.rho_ref > 0 ? p.rho_ref : 1.0;
    const double T = p.t_ref > 0 ? p.t_ref : 1.0 / 3.0;
    const double cv = Rg / (p.adiabatic_exponent - 1.0);
    const double tre = rho * (2.0 * cv * T + (vel0[0] * vel0[0] + vel0[1] * vel0[1] + vel0[2] * vel0[2]));
    for (int q = 0; q < NQ; ++q) {
        const double fr = eq_f_plain<double>(q, rho, vel0, Rg * T);
        const double gr = eq_g_plain<double>(q, rho, vel0, Rg, T, p.adiabatic_exponent, lat64);
        const double fs = std::fabs(fr) > 0 ? std::fabs(fr) : lat64.w[q];
        const double gs = std::max(std::fabs(gr), 1e-3 * lat64.w[q] * std::fabs(tre));
        D->ct.frest[q] = (float)fr;
        D->ct.grest[q] = (float)gr;
        D->ct.fsc[q] = (float)fs;
        D->ct.gsc[q] = (float)gs;
        D->ct.fisc[q] = (float)(1.0 / fs);
        D->ct.gisc[q] = (float)(1.0 / gs);
    }
    // fused tiles: 32 x 8 x 8 cells of every box
    std::vector<FusedTile> tiles;
    for (size_t n = 0; n < hbox.size(); ++n)
        for (int z0 = 0; z0 < hbox[n].n[2]; z0 += FT_Z)
            for (int y0 = 0; y0 < hbox[n].n[1]; y0 += FT_Y)
                for (int x0 = 0; x0 < hbox[n].n[0]; x0 += FT_X)
                    tiles.push_back(FusedTile{(int)n, (short)x0, (short)y0, (short)z0,
                                              (short)std::min(hbox[n].n[2], z0 + FT_Z)});
    D->ntiles = (int)tiles.size();
    mbg_status st;
    if ((st = lalloc(L, (void**)&D->tiles, tiles.size() * sizeof(FusedTile), err)) != MBG_OK) return st;
    cudaMemcpy(D->tiles, tiles.data(), tiles.size() * sizeof(FusedTile), cudaMemcpyHostToDevice);
    for (int b = 0; b < 2; ++b) {
        if ((st = lalloc(L, &L.f[b], (size_t)N * NQ * 2, err)) != MBG_OK) return st;
        if ((st = lalloc(L, &L.g[b], (size_t)N * NQ * 2, err)) != MBG_OK) return st;
        cudaMemset(L.f[b], 0xFF, (size_t)N * NQ * 2);
        cudaMemset(L.g[b], 0xFF, (size_t)N * NQ * 2);
        if (NG > 0) {
            if ((st = lalloc(L, &L.fg[b], (size_t)NG * NQ * 2, err)) != MBG_OK) return st;
            if ((st = lalloc(L, &L.gg[b], (size_t)NG * NQ * 2, err)) != MBG_OK) return st;
            cudaMemset(L.fg[b], 0xFF, (size_t)NG * NQ * 2);
            cudaMemset(L.gg[b], 0xFF, (size_t)NG * NQ * 2);
        }
    }
    if ((st = lalloc(L, (void**)&D->fo, (size_t)N * NQ * 2, err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->go, (size_t)N * NQ * 2, err)) != MBG_OK) return st;
    cudaMemset(D->fo, 0xFF, (size_t)N * NQ * 2);
    cudaMemset(D->go, 0xFF, (size_t)N * NQ * 2);
    if ((st = lalloc(L, (void**)&L.tmp, (size_t)N * NQ * sizeof(double), err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->dk, 2 * sizeof(LowpK), err)) != MBG_OK) return st;
    cudaDeviceSynchronize();
    (void)plan;
    return MBG_OK;
}

// the per-parity constant blocks (re-uploaded when the plan, the BCs or the
// use of the override buffers change; the plan's device arrays are final
// once the next finer level is defined)
static void upload_k(LowpLevel& L, const LevelPlan& plan, const BCParams& bc, bool with_override, cudaStream_t s)
{
    LowpDev* D = dev_of(L);
    for (int a = 0; a < 2; ++a) {
        LowpK& k = D->hk[a];
        k.L = view16(plan);
        k.P = bc;
        k.ph = L.ph;
        k.ct = D->ct;
        k.lat64 = make_lattice<double>();
        k.s = bufs(L, a);
        if (with_override) {
            k.s.fo = D->fo;
            k.s.go = D->go;
        }
        k.fB = (u16*)L.f[1 - a];
        k.gB = (u16*)L.g[1 - a];
        k.fBg = (u16*)L.fg[1 - a];
        k.gBg = (u16*)L.gg[1 - a];
    }
    cudaMemcpyAsync(D->dk, D->hk, 2 * sizeof(LowpK), cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    D->uploaded = true;
    D->with_override = with_override;
}

static void ensure_k(LowpLevel& L, const LevelPlan& plan, const BCParams& bc, bool with_override, cudaStream_t s)
{
    LowpDev* D = dev_of(L);
    if (!D->uploaded || D->with_override != with_override || std::memcmp(&D->hk[0].P, &bc, sizeof(bc)) != 0)
        upload_k(L, plan, bc, with_override, s);
}

static BCParams known_bc(LowpLevel& L)
{
    BCParams bc{};
    LowpDev* D = dev_of(L);
    return D->uploaded ? D->hk[0].P : bc;
}

mbg_status lowp_set_state(LowpLevel& L, const LevelPlan& plan, const std::vector<DevBox>& hbox, const double* f,
                          const double* g, cudaStream_t s, std::string& err)
{
    const LowpDev* D = dev_of(L);
    for (int lat = 0; lat < 2; ++lat) {
        const double* src = lat ? g : f;
        if (!src) continue;
        long long off = 0;
        for (size_t n = 0; n < hbox.size(); ++n) {
            const long long vol = (long long)hbox[n].n[0] * hbox[n].n[1] * hbox[n].n[2];
            cudaError_t e = cudaMemcpy2DAsync(L.tmp + hbox[n].voff, L.N * sizeof(double), src + off * NQ,
                                              vol * sizeof(double), vol * sizeof(double), NQ, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) { err = std::string("set_state copy: ") + cudaGetErrorString(e); return MBG_ECUDA; }
            off += vol;
        }
        const long long tot = L.N * NQ;
        u16* dst = (u16*)(lat ? L.g[L.cur] : L.f[L.cur]);
        if (L.precision == MBG_FP32C_BF16S)
            k_encode<true><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(D->ct, L.N, L.tmp, dst, lat);
        else
            k_encode<false><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(D->ct, L.N, L.tmp, dst, lat);
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { err = std::string("set_state: ") + cudaGetErrorString(e); return MBG_ECUDA; }
    (void)plan;
    return MBG_OK;
}

mbg_status lowp_get_state(LowpLevel& L, const LevelPlan& plan, const std::vector<DevBox>& hbox, double* f,
                          double* g, cudaStream_t s, std::string& err)
{
    const LowpDev* D = dev_of(L);
    for (int lat = 0; lat < 2; ++lat) {
        double* dst = lat ? g : f;
        if (!dst) continue;
        const long long tot = L.N * NQ;
        const u16* src = (const u16*)(lat ? L.g[L.cur] : L.f[L.cur]);
        if (L.precision == MBG_FP32C_BF16S)
            k_decode<true><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(D->ct, L.N, src, L.tmp, lat);
        else
            k_decode<false><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(D->ct, L.N, src, L.tmp, lat);
        long long off = 0;
        for (size_t n = 0; n < hbox.size(); ++n) {
            const long long vol = (long long)hbox[n].n[0] * hbox[n].n[1] * hbox[n].n[2];
            cudaError_t e = cudaMemcpy2DAsync(dst + off * NQ, vol * sizeof(double), L.tmp + hbox[n].voff,
                                              L.N * sizeof(double), vol * sizeof(double), NQ, cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) { err = std::string("get_state copy: ") + cudaGetErrorString(e); return MBG_ECUDA; }
            off += vol;
        }
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { err = std::string("get_state: ") + cudaGetErrorString(e); return MBG_ECUDA; }
    }
    (void)plan;
    return MBG_OK;
}

mbg_status lowp_macro(LowpLevel& L, const LevelPlan& plan, double* out19, cudaStream_t s, std::string& err)
{
    if (plan.ntiles == 0) return MBG_OK;
    LowpDev* D = dev_of(L);
    ensure_k(L, plan, known_bc(L), D->with_override, s);
    const LowpK* k = D->dk + L.cur;
    if (L.precision == MBG_FP32C_BF16S)
        k_macro16<true><<<plan.ntiles, TILE_CELLS, 0, s>>>(k, D->ct, plan.tiles, out19);
    else
        k_macro16<false><<<plan.ntiles, TILE_CELLS, 0, s>>>(k, D->ct, plan.tiles, out19);
    (void)err;
    return MBG_OK;
}

int lowp_advance(const mbg_params& p, const BCParams& bc, LowpLevel& L, const LevelPlan& plan, double dt,
                 const double idx[3], const CoalesceCell* coal, long long ncoal, const LowpLevel* fine,
                 const LevelPlan* fplan, cudaStream_t s, const LowpRunner& run)
{
    LowpDev* D = dev_of(L);
    const bool ovr = fine && ncoal > 0;
    ensure_k(L, plan, bc, ovr, s);
    int launches = 0;
    const int A = L.cur;
    const LowpK* k = D->dk + A;
    const bool bf = L.precision == MBG_FP32C_BF16S;
    if (ovr) {
        LowpLevel& F = const_cast<LowpLevel&>(*fine);
        ensure_k(F, *fplan, bc, dev_of(F)->with_override, s);
        const LowpK* kf = dev_of(F)->dk + F.cur;
        const unsigned nb = (unsigned)((ncoal + 63) / 64);
        run(LOWP_STAGE_COALESCE, [&] {
            if (bf) k_coalesce16<true><<<nb, 64, 0, s>>>(k, kf, coal, ncoal, D->fo, D->go, 0);
            else k_coalesce16<false><<<nb, 64, 0, s>>>(k, kf, coal, ncoal, D->fo, D->go, 0);
        });
        ++launches;
    }
    if (L.NG > 0 && plan.nghost_cells > 0) {
        const unsigned nb = (unsigned)((plan.nghost_cells + 127) / 128);
        run(LOWP_STAGE_GHOST_STREAM, [&] {
            if (bf) k_ghost_stream16<true><<<nb, 128, 0, s>>>(k, plan.ghost_list, plan.nghost_cells);
            else k_ghost_stream16<false><<<nb, 128, 0, s>>>(k, plan.ghost_list, plan.nghost_cells);
        });
        ++launches;
    }
    run(LOWP_STAGE_FUSED, [&] {
        if (bf) k_fused<true><<<D->ntiles, dim3(FT_X, FT_Y), 0, s>>>(k, D->ct, D->tiles);
        else k_fused<false><<<D->ntiles, dim3(FT_X, FT_Y), 0, s>>>(k, D->ct, D->tiles);
    });
    ++launches;
    L.cur = 1 - A;
    (void)p;
    (void)dt;
    (void)idx;
    return launches;
}

void lowp_explode(LowpLevel& F, const LevelPlan& fplan, const LowpLevel& C, const LevelPlan& cplan, cudaStream_t s)
{
    if (fplan.nghost_cells == 0) return;
    LowpLevel& Cm = const_cast<LowpLevel&>(C);
    LowpDev* FD = dev_of(F);
    LowpDev* CD = dev_of(Cm);
    ensure_k(F, fplan, known_bc(F), FD->with_override, s);
    ensure_k(Cm, cplan, known_bc(Cm), CD->with_override, s);
    const LowpK* kf = FD->dk + F.cur;
    const LowpK* kc = CD->dk + C.cur;
    const unsigned nb = (unsigned)((fplan.nghost_cells + 63) / 64);
    u16* fg = (u16*)F.fg[F.cur];
    u16* gg = (u16*)F.gg[F.cur];
    if (F.precision == MBG_FP32C_BF16S)
        k_explode16<true><<<nb, 64, 0, s>>>(kf, kc, fplan.ghost_list, fplan.nghost_cells, fg, gg);
    else
        k_explode16<false><<<nb, 64, 0, s>>>(kf, kc, fplan.ghost_list, fplan.nghost_cells, fg, gg);
}

void lowp_average_down(LowpLevel& C, const LevelPlan& cplan, const LowpLevel& F, const LevelPlan& fplan,
                       const CoalesceCell* list, long long n, cudaStream_t s)
{
    if (n == 0) return;
    LowpLevel& Fm = const_cast<LowpLevel&>(F);
    LowpDev* D = dev_of(C);
    LowpDev* FD = dev_of(Fm);
    ensure_k(C, cplan, known_bc(C), D->with_override, s);
    ensure_k(Fm, fplan, known_bc(Fm), FD->with_override, s);
    const LowpK* kc = D->dk + C.cur;
    const LowpK* kf = FD->dk + F.cur;
    const unsigned nb = (unsigned)((n + 63) / 64);
    if (C.precision == MBG_FP32C_BF16S)
        k_coalesce16<true><<<nb, 64, 0, s>>>(kc, kf, list, n, (u16*)C.f[C.cur], (u16*)C.g[C.cur], 1);
    else
        k_coalesce16<false><<<nb, 64, 0, s>>>(kc, kf, list, n, (u16*)C.f[C.cur], (u16*)C.g[C.cur], 1);
}

void lowp_release(LowpLevel& L)
{
    for (void* p : L.allocs) cudaFree(p);
    L.allocs.clear();
    delete (LowpDev*)L.impl;
    L.impl = nullptr;
}

}  // namespace mbg
