// mbg_lowp_kern.cuh -- kernels of the FP32-arithmetic / 16-bit-storage form of
// the level step, compiled once per storage format (mbg_lowp_f16.cu,
// mbg_lowp_bf16.cu); the host side is mbg_lowp.cu.
//
// Storage.  Each population is kept as a 16-bit float (FP16 or BF16) holding
// its scaled deviation from the equilibrium at the reference state
// (rho_ref, u_ref, T_ref):  f = f_rest[q] + scale[q] * h.  scale[q] is the rest
// value itself for f (h is then the relative deviation) and the rest value of
// g floored at 1e-3 w_q (2 rho E)_ref (g_rest vanishes for some directions).
// The stream's -1 sentinel (solid cells, unreached ghosts) is the code 0xFFFF,
// a NaN in both formats, decoded to exactly -1.
//
// Layout.  Every box is stored padded by one cell on each side,
// component-major over the level: v[q * N + voff + z sz + y sy + x] with
// sy = nx + 2, sz = (nx + 2)(ny + 2).  Before each advance k_halo16 writes
// into the pad of the source buffer, for every direction q that crosses a box
// face, the exact value the pull of the cell behind that face must see: the
// neighbour box's value (periodic images included), the physical-BC value,
// the coarse-fine ghost value, the bounce-back value or the -1 sentinel.
// The step kernel then pulls every direction by index arithmetic alone.
//
// Arithmetic.  FP32 throughout the collision; FP64 only where sums of many
// terms meet: the coalescence averages and the output moments.
//
// One level advance is one fused pass (k_fused): a CTA owns a tw x (256/tw)
// column tile of a box (tw = 8, 16 or 32) and marches through a run of planes.
// For each plane it pulls the 54 streamed values of its cells, forms the
// moments and Q_corr, and keeps Q_corr of the tile plus a one-cell halo in
// shared memory (halo cells are computed from the perspective of the box
// that owns them, so the coarse-fine ghost semantics match the reference);
// the previous plane is then collided: q-correction gradient from shared
// memory, equilibria, relaxation, with its 54 values pulled again from L1/L2.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "mbg_lowp_types.cuh"
#include "mbg_pair.cuh"

namespace mbg {

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
    return (r == SENT16 || r == NOOVR16) ? (u16)0xFFFEu : r;
}



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
        const u16 of = ovr ? K->s.fo[q * L.N + cell] : NOOVR16;                       \
        const u16 og = ovr ? K->s.go[q * L.N + cell] : NOOVR16;                       \
        const float fq = of != NOOVR16 ? dec<BF>(K->ct, of, q, false)                 \
                                       : pull16_slow<q, BF>(K, b, x, y, z, tf, 0);    \
        const float gq = og != NOOVR16 ? dec<BF>(K->ct, og, q, true)                  \
                                       : pull16_slow<q, BF>(K, b, x, y, z, tf, 1);    \
        acc.template add<q>(fq, gq);                                                 \
    }
    MBG_UNROLL27(MBG_MS16)
#undef MBG_MS16
    return acc;
}

// raw code of the value the pull of direction q at target (x,y,z) of box b
// sees; computed values (physical BCs) are encoded, stored ones copied
template <int q, bool BF>
__device__ __noinline__ u16 pull16_code(const LowpK* __restrict__ K, int b, int x, int y, int z, uint8_t tflag,
                                        int which)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    const bool is_g = which & 1;
    const u16* v = is_g ? K->s.g : K->s.f;
    const u16* vg = is_g ? K->s.gg : K->s.fg;
    const LV16& L = K->L;
    const DevBox& B = L.box[b];
    if (!(tflag & FL_FLUID)) return SENT16;
    const int sx = x - ex, sy = y - ey, sz = z - ez;
    if (sx < -3 || sy < -3 || sz < -3 || sx > B.n[0] + 2 || sy > B.n[1] + 2 || sz > B.n[2] + 2) return SENT16;
    // a solid source bounces back; the step kernel does that itself from the
    // target's own opposite population, so the pad value is never read
    const uint8_t sf = flag_at(L, B, sx, sy, sz);
    if (!(sf & FL_FLUID)) return SENT16;
    int gp[3] = {B.lo[0] + sx, B.lo[1] + sy, B.lo[2] + sz};
    if (outside_nonperiodic(L, gp))
        return enc<BF>(K->ct,
                       bc_value<q, u16, float>(L, K->P, B, sx, sy, sz, is_g, v, vg, K->lat64,
                                               [&](u16 r, int slot) { return dec<BF>(K->ct, r, slot, is_g); }),
                       q, is_g);
    return fab_value(L, B, sx, sy, sz, q, v, vg);
}


// fill the pad of the source buffer: for every direction q whose pull from
// the pad cell lands in the box, the value that pull must see
template <bool BF>
__global__ void k_halo16(const LowpK* __restrict__ K, const HaloCell* __restrict__ hl, long long n)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const HaloCell h = hl[e];
    const LV16& L = K->L;
    const DevBox& B = L.box[h.box];
    const long long hc = B.voff + val_lin(B, h.x, h.y, h.z);
#define MBG_HF16(q)                                                                                      \
    {                                                                                                    \
        const int tx = h.x + ev_x(q), ty = h.y + ev_y(q), tz = h.z + ev_z(q);                            \
        if (in_valid<u16>(B, tx, ty, tz)) {                                                              \
            const uint8_t tf = flag_at(L, B, tx, ty, tz);                                                \
            K->fA[q * L.N + hc] = pull16_code<q, BF>(K, h.box, tx, ty, tz, tf, 0);                       \
            K->gA[q * L.N + hc] = pull16_code<q, BF>(K, h.box, tx, ty, tz, tf, 1);                       \
        }                                                                                                \
    }
    MBG_UNROLL27(MBG_HF16)
#undef MBG_HF16
}

// pad fill along the plan of mbg_lowp.cu::halo_plan: one thread per pad
// cell, a copy of f and g for each direction of its mask from one valid cell
// (src >= 0) or the box's ghost fab (src < 0); the cells of one face share
// their mask, so warps run the same directions
template <bool BF>
__global__ void k_halo_copy16(const LowpK* __restrict__ K, const HaloCopy* __restrict__ hc, long long n)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const HaloCopy h = hc[e];
    const long long N = K->L.N, NG = K->L.NG;
    const bool own = h.src >= 0;
    const u16* __restrict__ f = own ? K->s.f + h.src : K->s.fg + (-h.src - 1);
    const u16* __restrict__ g = own ? K->s.g + h.src : K->s.gg + (-h.src - 1);
    const long long stride = own ? N : NG;
    // every load before the first store: the pad is written in place in
    // the source buffer, so the compiler would otherwise keep each load
    // behind the previous direction's store (pad cells are never sources)
    u16 vf[NQ], vg[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        if ((h.qmask >> q) & 1u) {
            vf[q] = f[q * stride];
            vg[q] = g[q * stride];
        }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        if ((h.qmask >> q) & 1u) {
            K->fA[q * N + h.dst] = vf[q];
            K->gA[q * N + h.dst] = vg[q];
        }
    }
}

// pad of self-periodic boxes (batched independent domains): a copy of the
// opposite face, edge or corner of the same box
template <bool BF>
__global__ void k_halo_periodic16(const LowpK* __restrict__ K, const HaloCell* __restrict__ hl, long long n)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const HaloCell h = hl[e];
    const LV16& L = K->L;
    const DevBox& B = L.box[h.box];
    const long long hc = B.voff + val_lin(B, h.x, h.y, h.z);
    const int wx = h.x < 0 ? B.n[0] - 1 : h.x >= B.n[0] ? 0 : h.x;
    const int wy = h.y < 0 ? B.n[1] - 1 : h.y >= B.n[1] ? 0 : h.y;
    const int wz = h.z < 0 ? B.n[2] - 1 : h.z >= B.n[2] ? 0 : h.z;
    const long long sc = B.voff + val_lin(B, wx, wy, wz);
#define MBG_HP16(q)                                                                  \
    if (in_valid<u16>(B, h.x + ev_x(q), h.y + ev_y(q), h.z + ev_z(q))) {             \
        K->fA[q * L.N + hc] = K->s.f[q * L.N + sc];                                  \
        K->gA[q * L.N + hc] = K->s.g[q * L.N + sc];                                  \
    }
    MBG_UNROLL27(MBG_HP16)
#undef MBG_HP16
}

// pull of direction q at valid cell c = (x,y,z) of box B from the padded
// storage: a solid source (in the box or in its pad) bounces back, any other
// source holds the streamed value; vf: the box grown by one is all fluid
template <int q, bool BF>
__device__ __forceinline__ float pullp(const CodecTab& ct, const LV16& L, const DevBox& B, const u16* __restrict__ v,
                                       long long c, int x, int y, int z, bool vf, bool is_g)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    if (!vf && !(flag_at(L, B, x - ex, y - ey, z - ez) & FL_FLUID))
        return dec<BF>(ct, v[opp(q) * L.N + c], opp(q), is_g);
    return dec<BF>(ct, __ldg(v + q * L.N + c - ((long long)ez * B.sz + (long long)ey * B.sy + ex)), q, is_g);
}

// uniform pull (every cell of the box grown by one is fluid)
template <int q, bool BF>
__device__ __forceinline__ float pullu(const CodecTab& ct, const u16* __restrict__ v, long long N, long long c,
                                       int sy, int sz, bool is_g)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    return dec<BF>(ct, __ldg(v + q * N + c - ((long long)ez * sz + (long long)ey * sy + ex)), q, is_g);
}

// moments of the streamed values at valid fluid cell (x,y,z) of box b
template <bool BF>
__device__ __noinline__ MomentAcc<float> moments_cell(const LowpK* __restrict__ K, int b, int x, int y, int z,
                                                      uint8_t tf)
{
    const LV16& L = K->L;
    const DevBox& B = L.box[b];
    const long long c = B.voff + val_lin(B, x, y, z);
    const CodecTab& ct = K->ct;
    MomentAcc<float> acc;
    const bool vf = B.vfluid;
    if ((tf & FL_OVR) && K->s.fo) {
#define MBG_MO16(q)                                                                                 \
    {                                                                                               \
        const u16 of = K->s.fo[q * L.N + c], og = K->s.go[q * L.N + c];                             \
        acc.template add<q>(of != NOOVR16 ? dec<BF>(ct, of, q, false)                               \
                                          : pullp<q, BF>(ct, L, B, K->s.f, c, x, y, z, vf, false),  \
                            og != NOOVR16 ? dec<BF>(ct, og, q, true)                                \
                                          : pullp<q, BF>(ct, L, B, K->s.g, c, x, y, z, vf, true));  \
    }
        MBG_UNROLL27(MBG_MO16)
#undef MBG_MO16
        return acc;
    }
#define MBG_MC16(q)                                                                     \
    acc.template add<q>(pullp<q, BF>(ct, L, B, K->s.f, c, x, y, z, vf, false),          \
                        pullp<q, BF>(ct, L, B, K->s.g, c, x, y, z, vf, true));
    MBG_UNROLL27(MBG_MC16)
#undef MBG_MC16
    return acc;
}

// Q_corr component d at box-local position (x, y, z) of box b, as the
// reference's macro FillBoundary leaves it: computed by the box that owns the
// cell, or by box b itself where no box covers it
template <bool BF>
__device__ __noinline__ float qcorr16(const LowpK* __restrict__ K, int b, int x, int y, int z, int d)
{
    const LV16& L = K->L;
    const DevBox& B = L.box[b];
    const float ms = K->ph.mesh_speed, Rg = K->ph.Rg, cv = K->ph.cv;
    int vb = b, lx = x, ly = y, lz = z;
    if (!in_valid<u16>(B, x, y, z)) {
        int p[3] = {B.lo[0] + x, B.lo[1] + y, B.lo[2] + z};
        if (!wrap_pos(L, p)) return 0.0f;
        const int o = owner_of(L, p);
        if (o < 0) {
            // coarse-fine ghost: streamed values of the box's own ghost fab
            const uint8_t tf = flag_at(L, B, x, y, z);
            if (!(tf & FL_FLUID)) return 0.0f;
            const Macro<float> m = moments16_slow<BF>(K, b, x, y, z, tf).finish(ms, Rg, cv);
            return d == 0 ? m.qcx : d == 1 ? m.qcy : m.qcz;
        }
        vb = o;
        const DevBox& O = L.box[o];
        lx = p[0] - O.lo[0];
        ly = p[1] - O.lo[1];
        lz = p[2] - O.lo[2];
    }
    const uint8_t tf = flag_at(L, L.box[vb], lx, ly, lz);
    if (!(tf & FL_FLUID)) return 0.0f;
    const Macro<float> m = moments_cell<BF>(K, vb, lx, ly, lz, tf).finish(ms, Rg, cv);
    return d == 0 ? m.qcx : d == 1 ? m.qcy : m.qcz;
}

// pull for the collision of a cell that is not on the uniform path
template <int q, bool BF>
__device__ __noinline__ float pull_gen(const LowpK* __restrict__ K, int b, int x, int y, int z, int which)
{
    const LV16& L = K->L;
    const DevBox& B = L.box[b];
    const long long c = B.voff + val_lin(B, x, y, z);
    const bool is_g = which & 1;
    const uint8_t tf = flag_at(L, B, x, y, z);
    if ((tf & FL_OVR) && K->s.fo) {
        const u16 o = (is_g ? K->s.go : K->s.fo)[q * L.N + c];
        if (o != NOOVR16) return dec<BF>(K->ct, o, q, is_g);
    }
    return pullp<q, BF>(K->ct, L, B, is_g ? K->s.g : K->s.f, c, x, y, z, B.vfluid, is_g);
}


// neighbour along d is part of the gradient stencil (Utilities.H:279-312)
__device__ __forceinline__ bool present(const LV16& L, const DevBox& B, int x, int y, int z, int d, int s)
{
    int p[3] = {x, y, z};
    p[d] += s;
    const int gd = B.lo[d] + p[d];
    if (gd < L.dlo[d] || gd > L.dhi[d]) return false;
    if (B.own_domain && (p[d] < 0 || p[d] >= B.n[d])) return false;
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

// One fused step over a list of tiles; a persistent grid strides through it.
template <bool BF>
__global__ void __launch_bounds__(FT_THREADS, 2)
    k_fused(const LowpK* __restrict__ K, const CodecTab ct, const Lattice<float> lat,
            const FusedTile* __restrict__ tiles, int ntiles)
{
    __shared__ float sqx[2][FT_QX];
    __shared__ float sqy[2][FT_QY];
    __shared__ float sqz[3][FT_THREADS];
    const LV16& L = K->L;
    const long long N = L.N;
    const u16* __restrict__ sf = K->s.f;
    const u16* __restrict__ sg = K->s.g;
    const u16* __restrict__ sfo = K->s.fo;
    const u16* __restrict__ sgo = K->s.go;
    u16* __restrict__ fB = K->fB;
    u16* __restrict__ gB = K->gB;
    const float ms = K->ph.mesh_speed, Rg = K->ph.Rg, cv = K->ph.cv;
    const int tid = threadIdx.x;
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
        const FusedTile t = tiles[ti];
        const DevBox& B = L.box[t.box];
        const int n0 = B.n[0], n1 = B.n[1], n2 = B.n[2], sy = B.sy, sz = B.sz;
        const long long voff = B.voff;
        const bool vf = B.vfluid;
        const Phys32* __restrict__ PH = K->phys ? K->phys + B.phys : &K->ph;
        const float nu = PH->nu, alpha = PH->alpha, dt = PH->dt;
        const float idx0 = PH->idx[0], idx1 = PH->idx[1], idx2 = PH->idx[2];
        const int lgw = t.lgw, tw = 1 << lgw, th = FT_THREADS >> lgw;
        const int lx = tid & (tw - 1), ly = tid >> lgw;
        const int x = t.x0 + lx, y = t.y0 + ly;
        const bool mine = x < n0 && y < n1;
        const int twe = n0 - t.x0 < tw ? n0 - t.x0 : tw, the = n1 - t.y0 < th ? n1 - t.y0 : th;
        const int px = tw + 2;   // row pitch of sqx
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
                        MomentAcc<float> acc;
                        if (vf && !((tf & FL_OVR) && sfo)) {
                            const long long c = voff + (long long)z * sz + (long long)y * sy + x;
#define MBG_MF16(q) \
    acc.template add<q>(pullu<q, BF>(ct, sf, N, c, sy, sz, false), pullu<q, BF>(ct, sg, N, c, sy, sz, true));
                            MBG_UNROLL27(MBG_MF16)
#undef MBG_MF16
                        } else {
                            acc = moments_cell<BF>(K, t.box, x, y, z, tf);
                        }
                        cur = acc.finish(ms, Rg, cv);
                        qx = cur.qcx; qy = cur.qcy; qz = cur.qcz;
                    }
                    curf = tf;
                    sqx[ia][ly * px + lx + 1] = qx;
                    sqy[ia][(ly + 1) * tw + lx] = qy;
                    sqz[iz][tid] = qz;
                } else {
                    // z-halo plane: Q_corr_z only, where the gradient will read it
                    const int zz = z < z0 ? z0 : z1 - 1;
                    const int s_ = z < z0 ? -1 : 1;
                    float v = 0.f;
                    if (present(L, B, x, y, zz, 2, s_)) v = qcorr16<BF>(K, t.box, x, y, z, 2);
                    sqz[iz][tid] = v;
                }
            }
            if (z >= z0 && z < z1) {
                // x- and y-halo of the tile in this plane
                const int nh = 2 * the + 2 * twe;
                for (int h = tid; h < nh; h += FT_THREADS) {
                    if (h < 2 * the) {
                        const int j = h >> 1, side = h & 1;
                        const int hx = side ? t.x0 + twe : t.x0 - 1, hy = t.y0 + j;
                        float v = 0.f;
                        if (present(L, B, side ? hx - 1 : hx + 1, hy, z, 0, side ? 1 : -1))
                            v = qcorr16<BF>(K, t.box, hx, hy, z, 0);
                        sqx[ia][j * px + (side ? twe + 1 : 0)] = v;
                    } else {
                        const int k = h - 2 * the;
                        const int i = k >> 1, side = k & 1;
                        const int hx = t.x0 + i, hy = side ? t.y0 + the : t.y0 - 1;
                        float v = 0.f;
                        if (present(L, B, hx, side ? hy - 1 : hy + 1, z, 1, side ? 1 : -1))
                            v = qcorr16<BF>(K, t.box, hx, hy, z, 1);
                        sqy[ia][(side ? the + 1 : 0) * tw + i] = v;
                    }
                }
            }
            __syncthreads();
            // ---- phase B: collide plane z - 1 ----
            const int zc = z - 1;
            if (mine && zc >= z0 && zc < z1) {
                const int ib = zc & 1;
                const long long c = voff + (long long)zc * sz + (long long)y * sy + x;
                const bool ovr = (prevf & FL_OVR) && sfo;
                if (!(prevf & FL_FLUID)) {
#define MBG_SOL16(q)                                                \
    {                                                               \
        const u16 of = ovr ? sfo[q * N + c] : SENT16;               \
        const u16 og = ovr ? sgo[q * N + c] : SENT16;               \
        fB[q * N + c] = of == NOOVR16 ? SENT16 : of;                \
        gB[q * N + c] = og == NOOVR16 ? SENT16 : og;                \
    }
                    MBG_UNROLL27(MBG_SOL16)
#undef MBG_SOL16
                } else {
                    const float dqx = grad1(present(L, B, x, y, zc, 0, 1), present(L, B, x, y, zc, 0, -1),
                                            sqx[ib][ly * px + lx + 2], sqx[ib][ly * px + lx + 1],
                                            sqx[ib][ly * px + lx], idx0);
                    const float dqy = grad1(present(L, B, x, y, zc, 1, 1), present(L, B, x, y, zc, 1, -1),
                                            sqy[ib][(ly + 2) * tw + lx], sqy[ib][(ly + 1) * tw + lx],
                                            sqy[ib][ly * tw + lx], idx1);
                    const float dqz = grad1(present(L, B, x, y, zc, 2, 1), present(L, B, x, y, zc, 2, -1),
                                            sqz[(z + 3) % 3][tid], sqz[(zc + 3) % 3][tid],
                                            sqz[(zc - 1 + 3) % 3][tid], idx2);
                    Equilibrium<float> E;
                    const float omega = build_equilibrium<float>(prev, dqx, dqy, dqz, nu, alpha, dt, Rg, cv, lat, E);
                    if (vf && !ovr) {
#define MBG_RI16(q)                                                                                  \
    {                                                                                                \
        const float fq = pullu<q, BF>(ct, sf, N, c, sy, sz, false);                                  \
        fB[q * N + c] = enc<BF>(ct, fmaf(omega, E.template feq<q>() - fq, fq), q, false);            \
        const float gq = pullu<q, BF>(ct, sg, N, c, sy, sz, true);                                   \
        gB[q * N + c] = enc<BF>(ct, fmaf(omega, E.template geq<q>(lat) - gq, gq), q, true);          \
    }
                        MBG_UNROLL27(MBG_RI16)
#undef MBG_RI16
                    } else {
#define MBG_RS16(q)                                                                                  \
    {                                                                                                \
        const float fq = pull_gen<q, BF>(K, t.box, x, y, zc, 0);                                     \
        fB[q * N + c] = enc<BF>(ct, fmaf(omega, E.template feq<q>() - fq, fq), q, false);            \
        const float gq = pull_gen<q, BF>(K, t.box, x, y, zc, 1);                                     \
        gB[q * N + c] = enc<BF>(ct, fmaf(omega, E.template geq<q>(lat) - gq, gq), q, true);          \
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
}

// ---- two-pass step ------------------------------------------------------------
// pass 1 (k_qcorr16, or k_qcorr16p on cell pairs): Q_corr of every valid cell
// into qs[d * N + c], padded layout; the face cells of each box's pad then
// get Q_corr as the owning box computes it (k_qpad_copy) or, on the
// coarse-fine shell, as the box itself computes it from its ghost fab (the
// ghost stream k_ghost_stream16s, or k_qhalo16 for boxes without a
// ghost-shell table); pass 2 (k_collide16 / k_collide16p) pulls again, takes
// the gradient from qs and collides.  No barriers and no halo recomputation;
// the populations are read twice.

// box-local cell of thread threadIdx.x of a Tile (128 cells in x-fastest order)
__device__ __forceinline__ bool tile_cell(const DevBox& B, const Tile& t, int& x, int& y, int& z)
{
    // boxes hold fewer than 2^31 cells: 32-bit division
    const unsigned ci = (unsigned)t.start + threadIdx.x;
    const unsigned nxy = (unsigned)B.n[0] * (unsigned)B.n[1];
    if (ci >= nxy * (unsigned)B.n[2]) return false;
    z = (int)(ci / nxy);
    const unsigned r = ci - (unsigned)z * nxy;
    y = (int)(r / (unsigned)B.n[0]);
    x = (int)(r - (unsigned)y * (unsigned)B.n[0]);
    return true;
}

// present() for a box whose cells one layer out are all fluid: only the
// domain bounds (and the box itself for a domain of its own) matter
__device__ __forceinline__ bool present_vf(const LV16& L, const DevBox& B, int c, int d, int s)
{
    const int p = c + s;
    const int gd = B.lo[d] + p;
    if (gd < L.dlo[d] || gd > L.dhi[d]) return false;
    return !(B.own_domain && (p < 0 || p >= B.n[d]));
}

// uniform pull through the per-direction base pointer (c: 32-bit storage
// index of the target within one component)
template <int q, bool BF>
__device__ __forceinline__ float pullq(const CodecTab& ct, const u16* __restrict__ base, int c, int sy, int sz,
                                       bool is_g)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    return dec<BF>(ct, __ldg(base + (c - (ez * sz + ey * sy + ex))), q, is_g);
}

template <bool BF>
__device__ __forceinline__ MomentAcc<float> moments_at(const LowpK* __restrict__ K, const CodecTab& ct,
                                                       const QPtrs& qp, const DevBox& B, int b, int x, int y, int z,
                                                       long long c, uint8_t tf)
{
    MomentAcc<float> acc;
    if (B.vfluid && !((tf & FL_OVR) && K->s.fo)) {
        const int c32 = (int)c, sy = B.sy, sz = B.sz;
#define MBG_MT16(q) \
    acc.template add<q>(pullq<q, BF>(ct, qp.f[q], c32, sy, sz, false), pullq<q, BF>(ct, qp.g[q], c32, sy, sz, true));
        MBG_UNROLL27(MBG_MT16)
#undef MBG_MT16
    } else {
        acc = moments_cell<BF>(K, b, x, y, z, tf);
    }
    return acc;
}

template <bool BF>
__global__ void __launch_bounds__(TILE_CELLS) k_qcorr16(const LowpK* __restrict__ K, const CodecTab ct,
                                                        const Tile* __restrict__ tiles, float* __restrict__ qs,
                                                        const QPtrs qp)
{
    const LV16& L = K->L;
    const Tile t = tiles[blockIdx.x];
    const DevBox& B = L.box[t.box];
    int x, y, z;
    if (!tile_cell(B, t, x, y, z)) return;
    const long long c = B.voff + val_lin(B, x, y, z);
    const uint8_t tf = flag_at(L, B, x, y, z);
    float qx = 0.f, qy = 0.f, qz = 0.f;
    if (tf & FL_FLUID) {
        const Macro<float> m =
            moments_at<BF>(K, ct, qp, B, t.box, x, y, z, c, tf).finish(K->ph.mesh_speed, K->ph.Rg, K->ph.cv);
        qx = m.qcx;
        qy = m.qcy;
        qz = m.qcz;
    }
    qs[c] = qx;
    qs[L.N + c] = qy;
    qs[2 * L.N + c] = qz;
}

// face cells of the pad: the normal component of Q_corr there
template <bool BF>
__global__ void k_qhalo16(const LowpK* __restrict__ K, const HaloCell* __restrict__ hl, long long n,
                          float* __restrict__ qs)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const HaloCell h = hl[e];
    const LV16& L = K->L;
    const DevBox& B = L.box[h.box];
    const int out0 = h.x < 0 || h.x >= B.n[0], out1 = h.y < 0 || h.y >= B.n[1], out2 = h.z < 0 || h.z >= B.n[2];
    if (out0 + out1 + out2 != 1) return;   // edges and corners are not on any gradient stencil
    const int d = out0 ? 0 : out1 ? 1 : 2;
    const long long hc = B.voff + val_lin(B, h.x, h.y, h.z);
    int p[3] = {B.lo[0] + h.x, B.lo[1] + h.y, B.lo[2] + h.z};
    float v = 0.f;
    // outside the domain box the gradient is one-sided, so nothing reads it
    if (p[0] >= L.dlo[0] && p[1] >= L.dlo[1] && p[2] >= L.dlo[2] && p[0] <= L.dhi[0] && p[1] <= L.dhi[1] &&
        p[2] <= L.dhi[2] && (flag_at(L, B, h.x, h.y, h.z) & FL_FLUID)) {
        const int o = owner_of(L, p);
        if (o >= 0) {
            const DevBox& O = L.box[o];
            v = qs[d * L.N + O.voff + val_lin(O, p[0] - O.lo[0], p[1] - O.lo[1], p[2] - O.lo[2])];
        } else if (B.goff >= 0) {
            // coarse-fine ghost: moments of the values the ghost stream of
            // this advance has just written into the destination's ghost fab
            const long long gi = B.goff + fab_lin(B, h.x, h.y, h.z);
            MomentAcc<float> acc;
#define MBG_QG16(q) \
    acc.template add<q>(dec<BF>(K->ct, K->fBg[q * L.NG + gi], q, false), dec<BF>(K->ct, K->gBg[q * L.NG + gi], q, true));
            MBG_UNROLL27(MBG_QG16)
#undef MBG_QG16
            const Macro<float> m = acc.finish(K->ph.mesh_speed, K->ph.Rg, K->ph.cv);
            v = d == 0 ? m.qcx : d == 1 ? m.qcy : m.qcz;
        }
    }
    qs[d * L.N + hc] = v;
}

template <bool BF, int MINB>
__global__ void __launch_bounds__(TILE_CELLS, MINB)
    k_collide16(const LowpK* __restrict__ K, const CodecTab ct, const Lattice<float> lat,
                const Tile* __restrict__ tiles, const float* __restrict__ qs, const QPtrs qp)
{
    const LV16& L = K->L;
    const Tile t = tiles[blockIdx.x];
    const DevBox& B = L.box[t.box];
    int x, y, z;
    if (!tile_cell(B, t, x, y, z)) return;
    const long long N = L.N;
    const long long c = B.voff + val_lin(B, x, y, z);
    const uint8_t tf = flag_at(L, B, x, y, z);
    const u16* __restrict__ sfo = K->s.fo;
    const u16* __restrict__ sgo = K->s.go;
    u16* __restrict__ fB = K->fB;
    u16* __restrict__ gB = K->gB;
    const bool ovr = (tf & FL_OVR) && sfo;
    if (!(tf & FL_FLUID)) {
#define MBG_SOLC16(q)                                               \
    {                                                               \
        const u16 of = ovr ? sfo[q * N + c] : SENT16;               \
        const u16 og = ovr ? sgo[q * N + c] : SENT16;               \
        fB[q * N + c] = of == NOOVR16 ? SENT16 : of;                \
        gB[q * N + c] = og == NOOVR16 ? SENT16 : og;                \
    }
        MBG_UNROLL27(MBG_SOLC16)
#undef MBG_SOLC16
        return;
    }
    const Phys32* __restrict__ PH = K->phys ? K->phys + B.phys : &K->ph;
    const float Rg = K->ph.Rg, cv = K->ph.cv;
    const Macro<float> m = moments_at<BF>(K, ct, qp, B, t.box, x, y, z, c, tf).finish(K->ph.mesh_speed, Rg, cv);
    const int sy = B.sy, sz = B.sz;
    bool pr[6];
    if (B.vfluid) {
        pr[0] = present_vf(L, B, x, 0, 1); pr[1] = present_vf(L, B, x, 0, -1);
        pr[2] = present_vf(L, B, y, 1, 1); pr[3] = present_vf(L, B, y, 1, -1);
        pr[4] = present_vf(L, B, z, 2, 1); pr[5] = present_vf(L, B, z, 2, -1);
    } else {
        pr[0] = present(L, B, x, y, z, 0, 1); pr[1] = present(L, B, x, y, z, 0, -1);
        pr[2] = present(L, B, x, y, z, 1, 1); pr[3] = present(L, B, x, y, z, 1, -1);
        pr[4] = present(L, B, x, y, z, 2, 1); pr[5] = present(L, B, x, y, z, 2, -1);
    }
    const float dqx = grad1(pr[0], pr[1], qs[c + 1], m.qcx, qs[c - 1], PH->idx[0]);
    const float dqy = grad1(pr[2], pr[3], qs[N + c + sy], m.qcy, qs[N + c - sy], PH->idx[1]);
    const float dqz = grad1(pr[4], pr[5], qs[2 * N + c + sz], m.qcz, qs[2 * N + c - sz], PH->idx[2]);
    Equilibrium<float> E;
    const float omega = build_equilibrium<float>(m, dqx, dqy, dqz, PH->nu, PH->alpha, PH->dt, Rg, cv, lat, E);
    if (B.vfluid && !ovr) {
        const int c32 = (int)c;
#define MBG_RC16(q)                                                                                  \
    {                                                                                                \
        const float fq = pullq<q, BF>(ct, qp.f[q], c32, sy, sz, false);                              \
        qp.fo[q][c32] = enc<BF>(ct, fmaf(omega, E.template feq<q>() - fq, fq), q, false);            \
        const float gq = pullq<q, BF>(ct, qp.g[q], c32, sy, sz, true);                               \
        qp.go[q][c32] = enc<BF>(ct, fmaf(omega, E.template geq<q>(lat) - gq, gq), q, true);          \
    }
        MBG_UNROLL27(MBG_RC16)
#undef MBG_RC16
    } else {
#define MBG_RG16(q)                                                                                  \
    {                                                                                                \
        const float fq = pull_gen<q, BF>(K, t.box, x, y, z, 0);                                      \
        fB[q * N + c] = enc<BF>(ct, fmaf(omega, E.template feq<q>() - fq, fq), q, false);            \
        const float gq = pull_gen<q, BF>(K, t.box, x, y, z, 1);                                      \
        gB[q * N + c] = enc<BF>(ct, fmaf(omega, E.template geq<q>(lat) - gq, gq), q, true);          \
    }
        MBG_UNROLL27(MBG_RG16)
#undef MBG_RG16
    }
}

// ---- the two-pass step on cell pairs ----------------------------------------
// Boxes with an even x extent whose cells one layer out are all fluid run
// the same two passes on two x-adjacent cells per thread (x even): the
// codes of a direction are one 32-bit word per lattice where the source
// pair is aligned (directions with ex = 0) and two 16-bit loads otherwise,
// the collision pulls again for the relaxation (L1 hits, so that the 54 code
// pairs need no registers across the equilibria), and the moments, equilibria,
// relaxation and encoding of both cells run as paired FP32 instructions
// (mbg_pair.cuh).  The new codes of a direction go out as one aligned
// 32-bit store per lattice.  Pulls of fluid targets in such boxes never
// meet the stream sentinel, and the outputs of fluid cells are encoded
// without the -1 test; a NaN encodes to the canonical NaN code (0x7FFF in
// both formats), never to a sentinel.

// codec constants per direction, each broadcast to both lanes
struct CodecPair {
    float2 frest[NQ], grest[NQ], fsc[NQ], gsc[NQ], fisc[NQ], gisc[NQ];
};

inline CodecPair make_codec_pair(const CodecTab& ct)
{
    CodecPair c;
    for (int q = 0; q < NQ; ++q) {
        c.frest[q] = make_float2(ct.frest[q], ct.frest[q]);
        c.grest[q] = make_float2(ct.grest[q], ct.grest[q]);
        c.fsc[q] = make_float2(ct.fsc[q], ct.fsc[q]);
        c.gsc[q] = make_float2(ct.gsc[q], ct.gsc[q]);
        c.fisc[q] = make_float2(ct.fisc[q], ct.fisc[q]);
        c.gisc[q] = make_float2(ct.gisc[q], ct.gisc[q]);
    }
    return c;
}

// the two 16-bit codes of a word (low half: cell x) as FP32
template <bool BF>
__device__ __forceinline__ float2 h2f_pair(unsigned w)
{
    if constexpr (BF) {
        return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xFFFF0000u));
    } else {
        __half2_raw r;
        r.x = (unsigned short)(w & 0xFFFFu);
        r.y = (unsigned short)(w >> 16);
        return __half22float2(__half2(r));
    }
}

template <bool BF>
__device__ __forceinline__ unsigned f2h_pair(float2 v)
{
    if constexpr (BF) {
        const __nv_bfloat162_raw r = __float22bfloat162_rn(v);
        return (unsigned)r.x | ((unsigned)r.y << 16);
    } else {
        const __half2_raw r = __float22half2_rn(v);
        return (unsigned)r.x | ((unsigned)r.y << 16);
    }
}

// read-only loads the compiler neither merges with the first pull's loads
// of the same values (which would hold all 54 code pairs in registers across
// the equilibria) nor drops
__device__ __forceinline__ unsigned ld_pin32(const void* p)
{
    unsigned r;
    asm volatile("ld.global.nc.b32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
}
__device__ __forceinline__ unsigned ld_pin16(const void* p)
{
    unsigned short r;
    asm volatile("ld.global.nc.b16 %0, [%1];" : "=h"(r) : "l"(p));
    return r;
}

// codes of direction q pulled to the target pair at storage index c (even)
template <int q, bool PIN = false>
__device__ __forceinline__ unsigned ld_pair(const u16* __restrict__ base, int c, int sy, int sz)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    const u16* p = base + (c - (ez * sz + ey * sy + ex));
    if constexpr (ex == 0) {
        return PIN ? ld_pin32(p) : __ldg(reinterpret_cast<const unsigned*>(p));
    } else {
        const unsigned lo = PIN ? ld_pin16(p) : __ldg(p), hi = PIN ? ld_pin16(p + 1) : __ldg(p + 1);
        return lo | (hi << 16);
    }
}

// box-local cell pair of thread threadIdx.x of a pair tile (256 cells)
__device__ __forceinline__ bool pair_cell(const DevBox& B, const Tile& t, int& x, int& y, int& z)
{
    const unsigned ci = (unsigned)t.start + 2u * threadIdx.x;
    const unsigned nxy = (unsigned)B.n[0] * (unsigned)B.n[1];
    if (ci >= nxy * (unsigned)B.n[2]) return false;
    z = (int)(ci / nxy);
    const unsigned r = ci - (unsigned)z * nxy;
    y = (int)(r / (unsigned)B.n[0]);
    x = (int)(r - (unsigned)y * (unsigned)B.n[0]);
    return true;
}

// coalescence overrides of a cell pair: o0 / o1 when cell x / x + 1 is
// overwritten (FL_OVR on a level with override buffers)
struct PairOvr {
    bool any, o0, o1;
};

template <bool BF>
__device__ __forceinline__ PairOvr pair_ovr(const LowpK* __restrict__ K, const DevBox& B, int x, int y, int z)
{
    PairOvr o{false, false, false};
    if (K->s.fo) {
        o.o0 = flag_at(K->L, B, x, y, z) & FL_OVR;
        o.o1 = flag_at(K->L, B, x + 1, y, z) & FL_OVR;
        o.any = o.o0 || o.o1;
    }
    return o;
}

// pass 1: the pulled code pair of direction q of one lattice (v: its
// source, ov: its override buffer); an overwritten cell takes the override
// code where it is not NOOVR16.  Pairs with an overwritten cell store the
// merged pair back into the override buffer (idempotent: a merged code is
// never NOOVR16), so that pass 2 reads one word there instead of merging;
// where both codes come from the override buffer (cells under the finer
// level) nothing is pulled and nothing stored.
template <int q>
__device__ __forceinline__ unsigned code_merge(const u16* __restrict__ v, u16* __restrict__ ov, long long N,
                                               const PairOvr& o, int c, int sy, int sz)
{
    if (!o.any) return ld_pair<q>(v, c, sy, sz);
    unsigned* w = reinterpret_cast<unsigned*>(ov + q * N + c);
    const unsigned ow = *w;
    unsigned m = 0u;
    if (o.o0 && (ow & 0xFFFFu) != NOOVR16) m |= 0x0000FFFFu;
    if (o.o1 && (ow >> 16) != NOOVR16) m |= 0xFFFF0000u;
    if (m == 0xFFFFFFFFu) return ow;
    const unsigned r = (ow & m) | (ld_pair<q>(v, c, sy, sz) & ~m);
    *w = r;
    return r;
}

// pass 2: the code pair of direction q, from the override buffer for pairs
// with an overwritten cell (merged there by pass 1), else pulled
template <int q, bool PIN>
__device__ __forceinline__ unsigned code_sel(const u16* __restrict__ v, const u16* __restrict__ ov, long long N,
                                             bool any, int c, int sy, int sz)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    const u16* p = any ? ov + q * N + c : v + (c - (ez * sz + ey * sy + ex));
    if constexpr (ex == 0) {
        return PIN ? ld_pin32(p) : __ldg(reinterpret_cast<const unsigned*>(p));
    } else {
        const unsigned lo = PIN ? ld_pin16(p) : __ldg(p), hi = PIN ? ld_pin16(p + 1) : __ldg(p + 1);
        return lo | (hi << 16);
    }
}

template <bool BF, int q>
__device__ __forceinline__ F2 dec_pair(unsigned w, float2 sc, float2 rest)
{
    return fma2(F2(h2f_pair<BF>(w)), F2(sc), F2(rest));
}

// boxes holding solid cells: a fluid cell whose source x - e_q is solid
// (bit q of its neighbour mask m0 / m1) takes its own opposite population,
// decoded with the opposite direction's codec (the half-way bounce-back of
// the push, Source/LBM.cpp:574-598); v: the pulled pair already decoded
template <bool BF, int q, bool PIN>
__device__ __forceinline__ F2 bounce(F2 v, const u16* __restrict__ vopp, int c, unsigned m0, unsigned m1,
                                     float2 sc_opp, float2 rest_opp)
{
    const unsigned b0 = (m0 >> q) & 1u, b1 = (m1 >> q) & 1u;
    if (b0 | b1) {
        const unsigned own = PIN ? ld_pin32(vopp + c) : __ldg(reinterpret_cast<const unsigned*>(vopp + c));
        const F2 vb = fma2(F2(h2f_pair<BF>(own)), F2(sc_opp), F2(rest_opp));
        if (b0) v.v.x = vb.v.x;
        if (b1) v.v.y = vb.v.y;
    }
    return v;
}

// moments of a pair: MERGE for pass 1, else the pass-2 selection
template <bool BF, bool MERGE, bool OVR = false, bool EB = false>
__device__ __forceinline__ MomentAcc<F2> moments_pair(const LowpK* __restrict__ K, const CodecPair& cp,
                                                      const QPtrs& qp, const PairOvr& o, int c, int sy, int sz,
                                                      unsigned m0 = 0u, unsigned m1 = 0u)
{
    u16* __restrict__ fo = const_cast<u16*>(K->s.fo);
    u16* __restrict__ go = const_cast<u16*>(K->s.go);
    const long long N = K->L.N;
    // all 54 code pairs first (54 loads in flight per thread), then the sums
    unsigned wf[NQ], wg[NQ];
    static_for<0, NQ>([&](auto Q) {
        constexpr int q = Q.value;
        if constexpr (MERGE) {
            wf[q] = code_merge<q>(qp.f[q], fo, N, o, c, sy, sz);
            wg[q] = code_merge<q>(qp.g[q], go, N, o, c, sy, sz);
        } else {
            wf[q] = code_sel<q, false>(qp.f[q], fo, N, OVR, c, sy, sz);
            wg[q] = code_sel<q, false>(qp.g[q], go, N, OVR, c, sy, sz);
        }
    });
    MomentAcc<F2> acc;
    static_for<0, NQ>([&](auto Q) {
        constexpr int q = Q.value;
        F2 vf = dec_pair<BF, q>(wf[q], cp.fsc[q], cp.frest[q]);
        F2 vg = dec_pair<BF, q>(wg[q], cp.gsc[q], cp.grest[q]);
        if constexpr (EB) {
            constexpr int oq = opp(q);
            vf = bounce<BF, q, false>(vf, qp.f[oq], c, m0, m1, cp.fsc[oq], cp.frest[oq]);
            vg = bounce<BF, q, false>(vg, qp.g[oq], c, m0, m1, cp.gsc[oq], cp.grest[oq]);
        }
        acc.template add<q>(vf, vg);
    });
    return acc;
}

// pass 1 on pairs: Q_corr of both cells into qs (one aligned 8-byte store
// per component)
// OVR: a tile holding cells overwritten by coalescence (the others never
// look at flags or override buffers)
// EB: a tile of a box holding solid cells (never with OVR): bounce-back by
// the neighbour masks, Q_corr 0 at solid cells
template <bool BF, bool OVR, bool EB>
__global__ void __launch_bounds__(TILE_CELLS) k_qcorr16p(const LowpK* __restrict__ K, const CodecPair cp,
                                                         const Tile* __restrict__ tiles, float* __restrict__ qs,
                                                         const QPtrs qp)
{
    static_assert(!(OVR && EB), "tiles with overwritten cells next to solids run per cell");
    const LV16& L = K->L;
    const Tile t = tiles[blockIdx.x];
    const DevBox& B = L.box[t.box];
    int x, y, z;
    if (!pair_cell(B, t, x, y, z)) return;
    const int c = (int)(B.voff + val_lin(B, x, y, z));
    const long long N = L.N;
    unsigned m0 = 0u, m1 = 0u;
    if constexpr (EB) {
        const uint2 mm = *reinterpret_cast<const uint2*>(K->nmask + c);
        m0 = mm.x;
        m1 = mm.y;
        if (!(((m0 | m1) >> NMASK_FLUID) & 1u)) {
            const float2 zero = make_float2(0.f, 0.f);
            *reinterpret_cast<float2*>(qs + c) = zero;
            *reinterpret_cast<float2*>(qs + N + c) = zero;
            *reinterpret_cast<float2*>(qs + 2 * N + c) = zero;
            return;
        }
    }
    const PairOvr o = OVR ? pair_ovr<BF>(K, B, x, y, z) : PairOvr{false, false, false};
    const Macro<F2> m = moments_pair<BF, true, false, EB>(K, cp, qp, o, c, B.sy, B.sz, m0, m1)
                            .finish(F2(K->ph.mesh_speed), F2(K->ph.Rg), F2(K->ph.cv));
    float2 qx = m.qcx.v, qy = m.qcy.v, qz = m.qcz.v;
    if constexpr (EB) {
        if (!((m0 >> NMASK_FLUID) & 1u)) qx.x = qy.x = qz.x = 0.f;
        if (!((m1 >> NMASK_FLUID) & 1u)) qx.y = qy.y = qz.y = 0.f;
    }
    *reinterpret_cast<float2*>(qs + c) = qx;
    *reinterpret_cast<float2*>(qs + N + c) = qy;
    *reinterpret_cast<float2*>(qs + 2 * N + c) = qz;
}

// relaxation and encoding of the three directions (ex, ey, -1 .. 1) of a
// cell pair: f_eq = rf[ex][ey] phz[ez] (Equilibrium::feq); g_eq of
// Equilibrium::geq regrouped as w_q (b + A4[ez^2] / 2 + ez cz) with b and cz
// shared by the three, so that few partial sums are live at a time
template <bool BF, int ex, int ey, bool OVR, bool EB>
__device__ __forceinline__ void relax_group(const LowpK* __restrict__ K, const CodecPair& cp,
                                            const Lattice<float>& lat, const QPtrs& qp, const PairOvr& o,
                                            const Equilibrium<F2>& E, F2 omega, F2 h0, F2 h1, int c, int sy, int sz,
                                            unsigned m0, unsigned m1, unsigned solid)
{
    const F2 half(0.5f);
    F2 s2 = E.A1[ex * ex] + E.A2[ey * ey];
    if constexpr (ex * ey == 1) s2 = s2 + E.t3; else if constexpr (ex * ey == -1) s2 = s2 - E.t3;
    F2 b = E.grho;
    if constexpr (ex == 1) b = b + E.a1[0]; else if constexpr (ex == -1) b = b - E.a1[0];
    if constexpr (ey == 1) b = b + E.a1[1]; else if constexpr (ey == -1) b = b - E.a1[1];
    b = fma2(half, s2, b);
    F2 cz = E.a1[2];
    if constexpr (ex == 1) cz = fma2(half, E.t5, cz); else if constexpr (ex == -1) cz = cz - half * E.t5;
    if constexpr (ey == 1) cz = fma2(half, E.t6, cz); else if constexpr (ey == -1) cz = cz - half * E.t6;
    const F2 b1 = b + h1;
    const u16* __restrict__ fo = K->s.fo;
    const u16* __restrict__ go = K->s.go;
    const long long N = K->L.N;
    static_for<0, 3>([&](auto Z) {
        constexpr int ez = Z.value - 1;
        constexpr int q = find_dir(ex, ey, ez);
        const unsigned wf = code_sel<q, true>(qp.f[q], fo, N, OVR, c, sy, sz);
        const unsigned wg = code_sel<q, true>(qp.g[q], go, N, OVR, c, sy, sz);
        constexpr int oq = opp(q);
        F2 fq = dec_pair<BF, q>(wf, cp.fsc[q], cp.frest[q]);
        if constexpr (EB) fq = bounce<BF, q, true>(fq, qp.f[oq], c, m0, m1, cp.fsc[oq], cp.frest[oq]);
        const F2 fn = fma2(omega, E.rf[ex + 1][ey + 1] * E.phz[ez + 1] - fq, fq);
        // solid cells keep the stream sentinel (all bits set)
        *reinterpret_cast<unsigned*>(qp.fo[q] + c) =
            f2h_pair<BF>(((fn - F2(cp.frest[q])) * F2(cp.fisc[q])).v) | solid;
        const F2 gsum = ez == 0 ? b + h0 : (ez == 1 ? b1 + cz : b1 - cz);
        const F2 geq = gsum * F2(lat.w[q]);
        F2 gq = dec_pair<BF, q>(wg, cp.gsc[q], cp.grest[q]);
        if constexpr (EB) gq = bounce<BF, q, true>(gq, qp.g[oq], c, m0, m1, cp.gsc[oq], cp.grest[oq]);
        const F2 gn = fma2(omega, geq - gq, gq);
        *reinterpret_cast<unsigned*>(qp.go[q] + c) =
            f2h_pair<BF>(((gn - F2(cp.grest[q])) * F2(cp.gisc[q])).v) | solid;
    });
}

// pass 2 on pairs: moments again from the same codes, q-correction
// gradient, equilibria, relaxation, encoding (OVR: a pair with a cell
// overwritten by coalescence, its codes read from the override buffers; EB:
// a box holding solid cells, bounce-back and presence by the neighbour
// masks m0 / m1, solid cells keep the sentinel)
template <bool BF, bool OVR, bool EB>
__device__ __forceinline__ void collide_pair(const LowpK* __restrict__ K, const CodecPair& cp,
                                             const Lattice<float>& lat, const float* __restrict__ qs, const QPtrs& qp,
                                             const DevBox& B, const PairOvr& o, int x, int y, int z, int c,
                                             unsigned m0, unsigned m1)
{
    const LV16& L = K->L;
    const int sy = B.sy, sz = B.sz;
    const Phys32* __restrict__ PH = K->phys ? K->phys + B.phys : &K->ph;
    const float Rg = K->ph.Rg, cv = K->ph.cv;
    const Macro<F2> m = moments_pair<BF, false, OVR, EB>(K, cp, qp, o, c, sy, sz, m0, m1)
                            .finish(F2(K->ph.mesh_speed), F2(Rg), F2(cv));
    // gradient() of Source/Utilities.H:279-312: the x neighbours inside the
    // pair are the other cell's own value; in EB boxes a solid neighbour is
    // not on the stencil (the source of direction -e along the axis)
    const long long N = L.N;
    const float xm = qs[c - 1], xp = qs[c + 2];
    const float2 ym = *reinterpret_cast<const float2*>(qs + N + c - sy);
    const float2 yp = *reinterpret_cast<const float2*>(qs + N + c + sy);
    const float2 zm = *reinterpret_cast<const float2*>(qs + 2 * N + c - sz);
    const float2 zp = *reinterpret_cast<const float2*>(qs + 2 * N + c + sz);
    constexpr int QXP = find_dir(-1, 0, 0), QXM = find_dir(1, 0, 0);   // sources x + 1, x - 1
    constexpr int QYP = find_dir(0, -1, 0), QYM = find_dir(0, 1, 0);
    constexpr int QZP = find_dir(0, 0, -1), QZM = find_dir(0, 0, 1);
    auto fl = [&](unsigned mk, int q) { return !EB || !((mk >> q) & 1u); };
    const bool px0 = present_vf(L, B, x, 0, 1) && fl(m0, QXP), mx0 = present_vf(L, B, x, 0, -1) && fl(m0, QXM);
    const bool px1 = present_vf(L, B, x + 1, 0, 1) && fl(m1, QXP), mx1 = present_vf(L, B, x + 1, 0, -1) && fl(m1, QXM);
    const bool py = present_vf(L, B, y, 1, 1), my = present_vf(L, B, y, 1, -1);
    const bool pz = present_vf(L, B, z, 2, 1), mz = present_vf(L, B, z, 2, -1);
    const float ix = PH->idx[0], iy = PH->idx[1], iz = PH->idx[2];
    const F2 dqx(grad1(px0, mx0, m.qcx.v.y, m.qcx.v.x, xm, ix), grad1(px1, mx1, xp, m.qcx.v.y, m.qcx.v.x, ix));
    const F2 dqy(grad1(py && fl(m0, QYP), my && fl(m0, QYM), yp.x, m.qcy.v.x, ym.x, iy),
                 grad1(py && fl(m1, QYP), my && fl(m1, QYM), yp.y, m.qcy.v.y, ym.y, iy));
    const F2 dqz(grad1(pz && fl(m0, QZP), mz && fl(m0, QZM), zp.x, m.qcz.v.x, zm.x, iz),
                 grad1(pz && fl(m1, QZP), mz && fl(m1, QZM), zp.y, m.qcz.v.y, zm.y, iz));
    Equilibrium<F2> E;
    const F2 omega = build_equilibrium<F2>(m, dqx, dqy, dqz, F2(PH->nu), F2(PH->alpha), F2(PH->dt), F2(Rg), F2(cv),
                                           lat, E);
    const F2 h0 = F2(0.5f) * E.A4[0], h1 = F2(0.5f) * E.A4[1];
    unsigned solid = 0u;
    if constexpr (EB) {
        if (!((m0 >> NMASK_FLUID) & 1u)) solid |= 0x0000FFFFu;
        if (!((m1 >> NMASK_FLUID) & 1u)) solid |= 0xFFFF0000u;
    }
    static_for<0, 9>([&](auto G) {
        relax_group<BF, G.value % 3 - 1, G.value / 3 - 1, OVR, EB>(K, cp, lat, qp, o, E, omega, h0, h1, c, sy, sz,
                                                                   m0, m1, solid);
    });
}

template <bool BF, bool OVR, bool EB>
__global__ void __launch_bounds__(TILE_CELLS, EB ? 3 : 4) k_collide16p(const LowpK* __restrict__ K, const CodecPair cp,
                                                           const Lattice<float> lat, const Tile* __restrict__ tiles,
                                                           const float* __restrict__ qs, const QPtrs qp)
{
    static_assert(!(OVR && EB), "tiles with overwritten cells next to solids run per cell");
    const LV16& L = K->L;
    const Tile t = tiles[blockIdx.x];
    const DevBox& B = L.box[t.box];
    int x, y, z;
    if (!pair_cell(B, t, x, y, z)) return;
    const int c = (int)(B.voff + val_lin(B, x, y, z));
    if constexpr (OVR) {
        const PairOvr o = pair_ovr<BF>(K, B, x, y, z);
        if (o.any) collide_pair<BF, true, false>(K, cp, lat, qs, qp, B, o, x, y, z, c, 0u, 0u);
        else collide_pair<BF, false, false>(K, cp, lat, qs, qp, B, o, x, y, z, c, 0u, 0u);
    } else if constexpr (EB) {
        const uint2 mm = *reinterpret_cast<const uint2*>(K->nmask + c);
        if (!(((mm.x | mm.y) >> NMASK_FLUID) & 1u)) {
            // two solid cells: the stream sentinel in every direction
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                *reinterpret_cast<unsigned*>(qp.fo[q] + c) = 0xFFFFFFFFu;
                *reinterpret_cast<unsigned*>(qp.go[q] + c) = 0xFFFFFFFFu;
            }
            return;
        }
        collide_pair<BF, false, true>(K, cp, lat, qs, qp, B, PairOvr{false, false, false}, x, y, z, c, mm.x, mm.y);
    } else {
        collide_pair<BF, false, false>(K, cp, lat, qs, qp, B, PairOvr{false, false, false}, x, y, z, c, 0u, 0u);
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

// ghost stream by gather (mbg_lowp.cu::ghost_plan) into the destination's
// ghost fab
template <bool BF>
__global__ void k_ghost_gather16(const LowpK* __restrict__ K, const long long* __restrict__ dst,
                                 const long long* __restrict__ src, long long n)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const long long d = dst[e], s_ = src[e];
    u16 vf = SENT16, vg = SENT16;
    if (s_ >= 0) {
        vf = K->s.f[s_];
        vg = K->s.g[s_];
    } else if (s_ <= -2) {
        vf = K->s.fg[-s_ - 2];
        vg = K->s.gg[-s_ - 2];
    }
    K->fBg[d] = vf;
    K->gBg[d] = vg;
}

template <bool BF>
__device__ __noinline__ float pull16_rt(int q, const LowpK* __restrict__ K, int b, int x, int y, int z,
                                        uint8_t tflag, int which);

// ghost stream through the ghost-shell slot tables (mbg_lowp.cu::
// ghost_slots16): the code of each pulled value, or the sentinel for a
// source beyond the shell (Source/LBM.cpp:558-604 over the grown box)
template <bool BF>
__global__ void k_ghost_stream16s(const LowpK* __restrict__ K, const NbrSlot* __restrict__ T0,
                                  const int* __restrict__ toff, int lg0, int lg1, int lg2,
                                  const GhostCell* __restrict__ gl, long long n, float* __restrict__ qs)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const GhostCell gc = gl[e];
    const LV16& L = K->L;
    const DevBox& B = L.box[gc.box];
    const NbrSlot* __restrict__ T = T0 + toff[gc.box];
    const int top0 = ((B.n[0] + (1 << lg0) - 1) >> lg0) + 1, top1 = ((B.n[1] + (1 << lg1) - 1) >> lg1) + 1,
              top2 = ((B.n[2] + (1 << lg2) - 1) >> lg2) + 1;
    const int tx = top0 + 1, ty = top1 + 1;
    const long long gi = B.goff + fab_lin(B, gc.x, gc.y, gc.z);
    const u16* __restrict__ f = K->s.f;
    const u16* __restrict__ g = K->s.g;
    const u16* __restrict__ fg = K->s.fg;
    const u16* __restrict__ gg = K->s.gg;
    // a pad face cell (one coordinate one cell out) inside the domain box:
    // its Q_corr normal to the face is the step's gradient input (the
    // moments of the values streamed here, as k_qhalo16 takes them)
    const int o0 = gc.x < 0 || gc.x >= B.n[0], o1 = gc.y < 0 || gc.y >= B.n[1], o2 = gc.z < 0 || gc.z >= B.n[2];
    const bool face1 = o0 + o1 + o2 == 1 && gc.x >= -1 && gc.y >= -1 && gc.z >= -1 && gc.x <= B.n[0] &&
                       gc.y <= B.n[1] && gc.z <= B.n[2] && B.lo[0] + gc.x >= L.dlo[0] &&
                       B.lo[1] + gc.y >= L.dlo[1] && B.lo[2] + gc.z >= L.dlo[2] && B.lo[0] + gc.x <= L.dhi[0] &&
                       B.lo[1] + gc.y <= L.dhi[1] && B.lo[2] + gc.z <= L.dhi[2];
    // every code first, then the stores (the compiler cannot tell the
    // destination ghost fab from the sources, so it would keep each load
    // behind the previous direction's store)
    u16 cf[NQ], cg[NQ];
    static_for<0, NQ>([&](auto Q) {
        constexpr int q = Q.value;
        const int sx = gc.x - ev_x(q), sy = gc.y - ev_y(q), sz = gc.z - ev_z(q);
        cf[q] = SENT16;
        cg[q] = SENT16;
        if (sx >= -3 && sy >= -3 && sz >= -3 && sx <= B.n[0] + 2 && sy <= B.n[1] + 2 && sz <= B.n[2] + 2) {
            const int ox = sx < 0 ? 0 : (sx < B.n[0] ? (sx >> lg0) + 1 : top0);
            const int oy = sy < 0 ? 0 : (sy < B.n[1] ? (sy >> lg1) + 1 : top1);
            const int oz = sz < 0 ? 0 : (sz < B.n[2] ? (sz >> lg2) + 1 : top2);
            const NbrSlot S = T[ox + tx * (oy + ty * oz)];
            const long long i = S.base + (long long)sz * S.sz + (long long)sy * S.sy + sx;
            cf[q] = S.ghost ? fg[q * L.NG + i] : f[q * L.N + i];
            cg[q] = S.ghost ? gg[q * L.NG + i] : g[q * L.N + i];
        }
    });
    MomentAcc<float> acc;
    static_for<0, NQ>([&](auto Q) {
        constexpr int q = Q.value;
        K->fBg[q * L.NG + gi] = cf[q];
        K->gBg[q * L.NG + gi] = cg[q];
        if (face1) acc.template add<q>(dec<BF>(K->ct, cf[q], q, false), dec<BF>(K->ct, cg[q], q, true));
    });
    if (face1) {
        const Macro<float> m = acc.finish(K->ph.mesh_speed, K->ph.Rg, K->ph.cv);
        const int d = o0 ? 0 : o1 ? 1 : 2;
        qs[d * L.N + B.voff + (long long)gc.z * B.sz + (long long)gc.y * B.sy + gc.x] =
            d == 0 ? m.qcx : d == 1 ? m.qcy : m.qcz;
    }
}

// the ghost stream's remaining entries (bounce-back, physical BCs)
template <bool BF>
__global__ void k_ghost_general16(const LowpK* __restrict__ K, const GhostCell* __restrict__ gl,
                                  const int* __restrict__ gcell, const int* __restrict__ gq, long long n)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const GhostCell gc = gl[gcell[e]];
    const int q = gq[e];
    const LV16& L = K->L;
    const DevBox& B = L.box[gc.box];
    const uint8_t tf = flag_at(L, B, gc.x, gc.y, gc.z);
    const long long gi = B.goff + fab_lin(B, gc.x, gc.y, gc.z);
    K->fBg[q * L.NG + gi] = enc<BF>(K->ct, pull16_rt<BF>(q, K, gc.box, gc.x, gc.y, gc.z, tf, 0), q, false);
    K->gBg[q * L.NG + gi] = enc<BF>(K->ct, pull16_rt<BF>(q, K, gc.box, gc.x, gc.y, gc.z, tf, 1), q, true);
}

// explosion (conservative linear interpolation, as in mbg_fp64_amr.cu) in
// FP32, the limiter factor of each axis the minimum over the 27 components
template <bool BF>
__device__ __forceinline__ long long crse16_index(const LV16& C, const int p0[3], int d, int s_)
{
    int p[3] = {p0[0], p0[1], p0[2]};
    p[d] += s_;
    wrap_pos(C, p);
    const int o = owner_of(C, p);
    if (o < 0) return -1;
    const DevBox& O = C.box[o];
    return O.voff + val_lin(O, p[0] - O.lo[0], p[1] - O.lo[1], p[2] - O.lo[2]);
}

// Explosion (cell_cons_interp restated: one MC-limited slope per axis, the
// limiter shared by the 27 components of a lattice) in three launches.  The
// slopes and the limiter depend only on the coarse cell, so they are computed
// once per coarse cell under the ghost shell rather than once per fine child;
// each child then evaluates the same expression.
//
// 1. the 7 coarse storage indices (centre, -x, +x, -y, +y, -z, +z) of each
//    slot, -1 where the coarse level has no cell; limiter reset to 1
template <bool BF>
__global__ void k_xindex16(const LowpK* __restrict__ KC, const XSlot* __restrict__ xc, long long nx,
                           int* __restrict__ ix, float* __restrict__ al)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nx) return;
    const LV16& C = KC->L;
    const XSlot c = xc[e];
    const int cp[3] = {c.x, c.y, c.z};
    ix[e] = (int)crse16_index<BF>(C, cp, 0, 0);
    for (int d = 0; d < 3; ++d) {
        ix[(1 + 2 * d) * nx + e] = (int)crse16_index<BF>(C, cp, d, -1);
        ix[(2 + 2 * d) * nx + e] = (int)crse16_index<BF>(C, cp, d, 1);
    }
    for (int k = 0; k < 6; ++k) al[k * nx + e] = 1.0f;
}

// 2. per (slot, direction): value, centred slopes, and each axis' limiter
//    ratio folded into the slot's minimum (non-negative floats order like
//    their bit patterns, so an integer atomicMin is exact and order-free)
template <bool BF>
__global__ void k_xslope16(const LowpK* __restrict__ KC, const int* __restrict__ ix, long long nx,
                           float* __restrict__ xs, float* __restrict__ al)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (e >= nx) return;
    const LV16& C = KC->L;
    int id[7];
    for (int k = 0; k < 7; ++k) id[k] = ix[k * nx + e];
    for (int lat = 0; lat < 2; ++lat) {
        const bool isg = lat == 1;
        const u16* __restrict__ v = (isg ? KC->s.g : KC->s.f) + (long long)q * C.N;
        float u[7];
        for (int k = 0; k < 7; ++k) u[k] = id[k] >= 0 ? dec<BF>(KC->ct, v[id[k]], q, isg) : 0.0f;
        float* o = xs + ((long long)(lat * 4) * NQ + q) * nx + e;
        o[0] = u[0];
        for (int d = 0; d < 3; ++d) {
            const float u0 = u[0], um = u[1 + 2 * d], up = u[2 + 2 * d];
            const float cen = 0.5f * (up - um);
            const float forw = 2.0f * (up - u0);
            const float back = 2.0f * (u0 - um);
            const float slp = (forw * back >= 0.f) ? fminf(fabsf(forw), fabsf(back)) : 0.f;
            o[(long long)(1 + d) * NQ * nx] = cen;
            // the ratio is exactly 1 unless slp < |cen|: divide only there
            if (cen != 0.f && slp < fabsf(cen)) {
                const float r = slp / fabsf(cen);
                if (r < 1.0f) atomicMin((int*)&al[(lat * 3 + d) * nx + e], __float_as_int(r));
            }
        }
    }
}

// 3. one thread per fine ghost cell: u0 + sum_d off_d (alpha_d slope_d)
template <bool BF>
__global__ void k_xfill16(const LowpK* __restrict__ KF, const GhostCell* __restrict__ gl,
                          const int* __restrict__ slot, long long n, const float* __restrict__ xs,
                          const float* __restrict__ al, long long nx, u16* __restrict__ fg, u16* __restrict__ gg)
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
    const long long sl = slot[e];
    for (int lat = 0; lat < 2; ++lat) {
        const bool isg = lat == 1;
        u16* __restrict__ out = isg ? gg : fg;
        const float a0 = al[(lat * 3 + 0) * nx + sl], a1 = al[(lat * 3 + 1) * nx + sl],
                    a2 = al[(lat * 3 + 2) * nx + sl];
        const float* __restrict__ x = xs + (long long)(lat * 4) * NQ * nx + sl;
#pragma unroll 3
        for (int q = 0; q < NQ; ++q) {
            const float u0 = x[(long long)q * nx];
            const float cx = x[(long long)(NQ + q) * nx];
            const float cy = x[(long long)(2 * NQ + q) * nx];
            const float cz = x[(long long)(3 * NQ + q) * nx];
            out[q * F.NG + gi] = enc<BF>(KF->ct, u0 + off[0] * (a0 * cx) + off[1] * (a1 * cy) + off[2] * (a2 * cz),
                                         q, isg);
        }
    }
}

// streamed value of a runtime direction (the ghost stream's general entries)
template <bool BF>
__device__ __noinline__ float pull16_rt(int q, const LowpK* __restrict__ K, int b, int x, int y, int z,
                                        uint8_t tflag, int which)
{
    switch (q) {
#define MBG_PRT16(qq) \
    case qq: return pull16_slow<qq, BF>(K, b, x, y, z, tflag, which);
        MBG_UNROLL27(MBG_PRT16)
#undef MBG_PRT16
    }
    return -1.0f;
}

// coalescence: FP64 masked average of the 8 fine children into the override
// buffer (advance) or the coarse state (initial average_down); one thread per
// (coarse cell, direction), blockIdx.y the direction
// exact FP32 -> FP64 widening with integer operations (IEEE-754 binary32 to
// binary64: rebias the exponent by 1023 - 127 = 896, widen the fraction);
// zero, subnormal and non-finite inputs take the hardware conversion.  The
// FP64 pipe of GB300 issues 2 operations per SM per clock, so the
// coalescence keeps it for the sums alone.
__device__ __forceinline__ double widen_exact(float v)
{
    const unsigned u = __float_as_uint(v);
    const unsigned ex = (u >> 23) & 0xFFu;
    if (ex == 0u || ex == 0xFFu) return (double)v;
    const unsigned long long bits = ((unsigned long long)(u >> 31) << 63) |
                                    ((unsigned long long)(ex + 896u) << 52) |
                                    ((unsigned long long)(u & 0x7FFFFFu) << 29);
    return __longlong_as_double((long long)bits);
}

// The sum of the eight children of one (coarse cell, direction, lattice) as
// a fixed-point integer: with every exponent within 26 of the largest, the
// FP64 sum of the eight values is exact (24-bit significands spread over at
// most 26 + 24 bits, plus 3 bits of carry, fit FP64's 53), so the integer sum
// rounded once to FP32 is exactly the FP64 sum rounded to FP32.  Returns
// false (caller takes the FP64 adds) for a wider spread, a zero, a
// subnormal, an infinity or a NaN.
__device__ __forceinline__ bool sum8_exact(const float (&v)[8], float& out)
{
    unsigned emax = 0u, emin = 0xFFu;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const unsigned e = (__float_as_uint(v[k]) >> 23) & 0xFFu;
        emax = max(emax, e);
        emin = min(emin, e);
    }
    if (emin == 0u || emax == 0xFFu || emax - emin > 26u || emax < 60u) return false;
    long long acc = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const unsigned u = __float_as_uint(v[k]);
        const long long m = (long long)((u & 0x7FFFFFu) | 0x800000u) << (36u - (emax - ((u >> 23) & 0xFFu)));
        acc += (u >> 31) ? -m : m;
    }
    // value = acc * 2^(emax - 150 - 36); the power of two is a normal float
    // (emax >= 60) and the product of the rounded sum by it is exact
    out = __ll2float_rn(acc) * __uint_as_float((emax - 59u) << 23);
    return true;
}

template <bool BF>
__global__ void __launch_bounds__(128) k_coalesce16(const LowpK* __restrict__ KC, const LowpK* __restrict__ KF,
                                                    const CoalesceCell* __restrict__ cl, long long n,
                                                    u16* __restrict__ fo, u16* __restrict__ go, int into_state)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (e >= n) return;
    const LV16& C = KC->L;
    const LV16& F = KF->L;
    const CoalesceCell cc = cl[e];
    const DevBox& O = C.box[cc.cbox];
    const DevBox& A = F.box[cc.fbox];
    const long long cell = O.voff + val_lin(O, cc.cx, cc.cy, cc.cz);
    // the eight children's codes of both lattices, child k = 4 kz + 2 ky + kx;
    // fixed offsets when all eight are valid cells of box A (the common case),
    // each x pair one aligned word (fine boxes sit on even cells, the padded
    // layout puts valid cell 0 of a box on an even index)
    u16 code[2][8];
    if (cc.fx >= 0 && cc.fy >= 0 && cc.fz >= 0 && cc.fx + 1 < A.n[0] && cc.fy + 1 < A.n[1] && cc.fz + 1 < A.n[2]) {
        const long long b = (long long)q * F.N + A.voff + val_lin(A, cc.fx, cc.fy, cc.fz);
        const int sy = A.sy, sz = A.sz;
        const u16* __restrict__ f = KF->s.f + b;
        const u16* __restrict__ g = KF->s.g + b;
        if ((b & 1) == 0) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int off = (r >> 1) * sz + (r & 1) * sy;
                const unsigned wf = __ldg(reinterpret_cast<const unsigned*>(f + off));
                const unsigned wg = __ldg(reinterpret_cast<const unsigned*>(g + off));
                code[0][2 * r] = (u16)(wf & 0xFFFFu);
                code[0][2 * r + 1] = (u16)(wf >> 16);
                code[1][2 * r] = (u16)(wg & 0xFFFFu);
                code[1][2 * r + 1] = (u16)(wg >> 16);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int off = (k >> 2) * sz + ((k >> 1) & 1) * sy + (k & 1);
                code[0][k] = __ldg(f + off);
                code[1][k] = __ldg(g + off);
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int x = cc.fx + (k & 1), y = cc.fy + ((k >> 1) & 1), z = cc.fz + (k >> 2);
            code[0][k] = fab_value(F, A, x, y, z, q, KF->s.f, KF->s.fg);
            code[1][k] = fab_value(F, A, x, y, z, q, KF->s.g, KF->s.gg);
        }
    }
    // the mask test |v - (-1)| > SMALL_NUM on the FP32 decoded value; the sum
    // exact (sum8_exact) or in FP64, children in the reference's loop order
    // (z, y, x)
    const float small_num = (float)(2.220446049250313e-16 * 1e10);
#pragma unroll
    for (int lat = 0; lat < 2; ++lat) {
        const bool isg = lat == 1;
        float fv[8];
        bool all = true;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            fv[k] = dec<BF>(KF->ct, code[lat][k], q, isg);
            all = all && fabsf(fv[k] + 1.0f) > small_num;
        }
        // all eight children unmasked is the common case: sum / 8 is exact,
        // and a power-of-two scaling commutes with the rounding to FP32 (the
        // values are far from the FP32 range limits), so it is applied after
        float s8;
        u16 r;
        if (all && sum8_exact(fv, s8)) {
            r = enc<BF>(KC->ct, s8 * 0.125f, q, isg);
        } else {
            double sum = 0.0;
            int vol = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (fabsf(fv[k] + 1.0f) > small_num) { sum += widen_exact(fv[k]); ++vol; }
            if (vol > 0) r = enc<BF>(KC->ct, vol == 8 ? __double2float_rn(sum) * 0.125f : (float)(sum / (double)vol), q, isg);
            else if (into_state) r = (isg ? KC->s.g : KC->s.f)[q * C.N + cell];
            else r = NOOVR16;   // the step takes the cell's own streamed value
        }
        (isg ? go : fo)[q * C.N + cell] = r;
    }
}

// FP64 staging ([q][valid cell] in host cell order) <-> 16-bit padded state;
// one thread per valid cell of a tile
template <bool BF>
__global__ void k_encode16(const LowpK* __restrict__ K, const Tile* __restrict__ tiles, const double* __restrict__ src,
                           long long NV, u16* __restrict__ dst, int isg)
{
    const LV16& L = K->L;
    const Tile t = tiles[blockIdx.x];
    const DevBox& B = L.box[t.box];
    const long long c = (long long)t.start + threadIdx.x;
    const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
    if (c >= vol) return;
    const int x = (int)(c % B.n[0]), y = (int)((c / B.n[0]) % B.n[1]), z = (int)(c / ((long long)B.n[0] * B.n[1]));
    const long long pc = B.voff + val_lin(B, x, y, z), hc = B.hoff + c;
    for (int q = 0; q < NQ; ++q) dst[q * L.N + pc] = enc<BF>(K->ct, (float)src[q * NV + hc], q, isg != 0);
}
template <bool BF>
__global__ void k_decode16(const LowpK* __restrict__ K, const Tile* __restrict__ tiles, const u16* __restrict__ src,
                           long long NV, double* __restrict__ dst, int isg)
{
    const LV16& L = K->L;
    const Tile t = tiles[blockIdx.x];
    const DevBox& B = L.box[t.box];
    const long long c = (long long)t.start + threadIdx.x;
    const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
    if (c >= vol) return;
    const int x = (int)(c % B.n[0]), y = (int)((c / B.n[0]) % B.n[1]), z = (int)(c / ((long long)B.n[0] * B.n[1]));
    const long long pc = B.voff + val_lin(B, x, y, z), hc = B.hoff + c;
    for (int q = 0; q < NQ; ++q) dst[q * NV + hc] = (double)dec<BF>(K->ct, src[q * L.N + pc], q, isg != 0);
}

// a [q][n] array (a level's ghost fabs) decoded to FP64, value by value
template <bool BF>
__global__ void k_decode_flat16(const LowpK* __restrict__ K, const u16* __restrict__ src, long long n,
                                double* __restrict__ dst, int isg)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * NQ) return;
    dst[i] = (double)dec<BF>(K->ct, src[i], (int)(i / n), isg != 0);
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
    const int x = (int)(c % B.n[0]), y = (int)((c / B.n[0]) % B.n[1]), z = (int)(c / ((long long)B.n[0] * B.n[1]));
    const uint8_t tf = flag_at(L, B, x, y, z);
    double* o = out19 + B.hoff * 19 + c;
    if (!(tf & FL_FLUID)) {
        for (int k = 0; k < 19; ++k) o[k * vol] = 0.0;
        return;
    }
    const long long cell = B.voff + val_lin(B, x, y, z);
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

// running FP32 sum carried as hi + lo: TwoSum (Knuth, TAOCP vol. 2,
// 4.2.2) gives the rounding error of each addition exactly, and lo collects
// those errors, so hi + lo holds the sum to about 2^-48 relative.  The
// explicit-rounding intrinsics keep the compiler from contracting or
// reordering the error terms.
struct Sum2f {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float b)
    {
        const float s = __fadd_rn(hi, b);
        const float bb = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
        hi = s;
        lo = __fadd_rn(lo, e);
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// conserved totals of the decoded stored state (the quantities of
// mbg_fp64_out.cu::k_conserved): the per-cell sums of the 27 decoded FP32
// values in FP32 TwoSum arithmetic (GB300's FP64 pipe made the FP64 per-cell
// sums the kernel's bound), the cross-cell sums in FP64
template <bool BF>
__global__ void __launch_bounds__(TILE_CELLS) k_conserved16(const LowpK* __restrict__ K, const Tile* tiles, double dV,
                                                            double* out5)
{
    __shared__ double red[5][TILE_CELLS];
    const LV16& L = K->L;
    const Tile t0 = tiles[blockIdx.x];
    const DevBox& B = L.box[t0.box];
    int x, y, z;
    double v[5] = {0, 0, 0, 0, 0};
    if (tile_cell(B, t0, x, y, z)) {
        const uint8_t tf = flag_at(L, B, x, y, z);
        if ((tf & FL_FLUID) && !(tf & FL_COV)) {
            const long long cell = B.voff + val_lin(B, x, y, z);
            Sum2f rho, mu, mv, mw, tre;
#define MBG_CN16(q)                                                                           \
    {                                                                                         \
        constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);                               \
        const float fq = dec<BF>(K->ct, K->s.f[q * L.N + cell], q, false);                    \
        rho.add(fq);                                                                          \
        if constexpr (ex != 0) mu.add(ex > 0 ? fq : -fq);                                     \
        if constexpr (ey != 0) mv.add(ey > 0 ? fq : -fq);                                     \
        if constexpr (ez != 0) mw.add(ez > 0 ? fq : -fq);                                     \
        tre.add(dec<BF>(K->ct, K->s.g[q * L.N + cell], q, true));                             \
    }
            MBG_UNROLL27(MBG_CN16)
#undef MBG_CN16
            const double ms = K->ph.mesh_speed;
            v[0] = rho.value() * dV;
            v[1] = mu.value() * ms * dV;
            v[2] = mv.value() * ms * dV;
            v[3] = mw.value() * ms * dV;
            v[4] = tre.value() * dV;
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

// ---- launchers ---------------------------------------------------------------
template <bool BF>
void Lowp16<BF>::halo(const LowpK* k, const HaloCell* h, long long n, cudaStream_t s)
{
    if (n > 0) k_halo16<BF><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(k, h, n);
}
template <bool BF>
void Lowp16<BF>::halo_copy(const LowpK* k, const HaloCopy* hc, long long n, cudaStream_t s)
{
    if (n > 0) k_halo_copy16<BF><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(k, hc, n);
}
template <bool BF>
void Lowp16<BF>::halo_periodic(const LowpK* k, const HaloCell* h, long long n, cudaStream_t s)
{
    if (n > 0) k_halo_periodic16<BF><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(k, h, n);
}
template <bool BF>
void Lowp16<BF>::fused(const LowpK* k, const CodecTab& ct, const Lattice<float>& lat, const FusedTile* t, int ntiles,
                       int grid, cudaStream_t s)
{
    if (ntiles > 0) k_fused<BF><<<grid, FT_THREADS, 0, s>>>(k, ct, lat, t, ntiles);
}
template <bool BF>
int Lowp16<BF>::fused_blocks_per_sm()
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fused<BF>, FT_THREADS, 0) != cudaSuccess) nb = 1;
    return nb > 0 ? nb : 1;
}
// Q_corr pad face cells held by another box: a copy of that box's value
template <bool BF>
__global__ void k_qpad_copy(const long long* __restrict__ dst, const long long* __restrict__ src, long long n,
                            float* __restrict__ qs)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) qs[dst[e]] = qs[src[e]];
}

template <bool BF>
int Lowp16<BF>::two_pass(const LowpK* k, const CodecTab& ct, const Lattice<float>& lat, const Tile* tiles,
                         int ntiles, const PairLists& pl, const QPad& qpad, float* qs, const QPtrs& qp, int tight,
                         cudaStream_t s)
{
    int n = 0;
    const bool any_pair = pl.npair + pl.npair_ovr + pl.npair_eb > 0;
    const CodecPair cp = any_pair ? make_codec_pair(ct) : CodecPair{};
    if (pl.npair > 0) { k_qcorr16p<BF, false, false><<<pl.npair, TILE_CELLS, 0, s>>>(k, cp, pl.pair, qs, qp); ++n; }
    if (pl.npair_ovr > 0) {
        k_qcorr16p<BF, true, false><<<pl.npair_ovr, TILE_CELLS, 0, s>>>(k, cp, pl.pair_ovr, qs, qp);
        ++n;
    }
    if (pl.npair_eb > 0) {
        k_qcorr16p<BF, false, true><<<pl.npair_eb, TILE_CELLS, 0, s>>>(k, cp, pl.pair_eb, qs, qp);
        ++n;
    }
    if (ntiles > 0) { k_qcorr16<BF><<<ntiles, TILE_CELLS, 0, s>>>(k, ct, tiles, qs, qp); ++n; }
    if (n == 0) return 0;
    if (qpad.ncopy > 0) {
        k_qpad_copy<BF><<<(unsigned)((qpad.ncopy + 255) / 256), 256, 0, s>>>(qpad.dst, qpad.src, qpad.ncopy, qs);
        ++n;
    }
    if (qpad.nghost > 0) {
        k_qhalo16<BF><<<(unsigned)((qpad.nghost + 127) / 128), 128, 0, s>>>(k, qpad.ghost, qpad.nghost, qs);
        ++n;
    }
    if (pl.npair > 0) {
        k_collide16p<BF, false, false><<<pl.npair, TILE_CELLS, 0, s>>>(k, cp, lat, pl.pair, qs, qp);
        ++n;
    }
    if (pl.npair_ovr > 0) {
        k_collide16p<BF, true, false><<<pl.npair_ovr, TILE_CELLS, 0, s>>>(k, cp, lat, pl.pair_ovr, qs, qp);
        ++n;
    }
    if (pl.npair_eb > 0) {
        k_collide16p<BF, false, true><<<pl.npair_eb, TILE_CELLS, 0, s>>>(k, cp, lat, pl.pair_eb, qs, qp);
        ++n;
    }
    // register cap: 5 resident blocks per SM, or 6 with tight
    if (ntiles > 0) {
        if (tight) k_collide16<BF, 6><<<ntiles, TILE_CELLS, 0, s>>>(k, ct, lat, tiles, qs, qp);
        else k_collide16<BF, 5><<<ntiles, TILE_CELLS, 0, s>>>(k, ct, lat, tiles, qs, qp);
        ++n;
    }
    return n;
}
template <bool BF>
void Lowp16<BF>::ghost_stream(const LowpK* k, const GhostCell* gl, long long n, cudaStream_t s)
{
    if (n > 0) k_ghost_stream16<BF><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(k, gl, n);
}
template <bool BF>
void Lowp16<BF>::ghost_slots(const LowpK* k, const NbrSlot* T, const int* off, const int lg[3], const GhostCell* gl,
                             long long n, float* qs, cudaStream_t s)
{
    if (n > 0)
        k_ghost_stream16s<BF><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(k, T, off, lg[0], lg[1], lg[2], gl, n, qs);
}
template <bool BF>
void Lowp16<BF>::ghost_gather(const LowpK* k, const long long* dst, const long long* src, long long n,
                              const GhostCell* gl, const int* gcell, const int* gq, long long ngen, cudaStream_t s)
{
    if (n > 0) k_ghost_gather16<BF><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(k, dst, src, n);
    if (ngen > 0) k_ghost_general16<BF><<<(unsigned)((ngen + 127) / 128), 128, 0, s>>>(k, gl, gcell, gq, ngen);
}
template <bool BF>
void Lowp16<BF>::explode(const LowpK* kf, const LowpK* kc, const ExplodePlan& xp, u16* fg, u16* gg, cudaStream_t s)
{
    if (xp.n <= 0 || xp.nx <= 0) return;
    const unsigned bx = (unsigned)((xp.nx + 127) / 128);
    k_xindex16<BF><<<bx, 128, 0, s>>>(kc, xp.xc, xp.nx, xp.ix, xp.al);
    k_xslope16<BF><<<dim3(bx, NQ), 128, 0, s>>>(kc, xp.ix, xp.nx, xp.xs, xp.al);
    k_xfill16<BF><<<(unsigned)((xp.n + 127) / 128), 128, 0, s>>>(kf, xp.gl, xp.slot, xp.n, xp.xs, xp.al, xp.nx, fg,
                                                                  gg);
}
template <bool BF>
void Lowp16<BF>::coalesce(const LowpK* kc, const LowpK* kf, const CoalesceCell* cl, long long n, u16* fo, u16* go,
                          int into_state, cudaStream_t s)
{
    const dim3 grid((unsigned)((n + 127) / 128), NQ);
    if (n > 0) k_coalesce16<BF><<<grid, 128, 0, s>>>(kc, kf, cl, n, fo, go, into_state);
}
template <bool BF>
void Lowp16<BF>::encode(const LowpK* k, const Tile* tiles, int ntiles, const double* src, long long NV, u16* dst,
                        int isg, cudaStream_t s)
{
    if (ntiles > 0) k_encode16<BF><<<ntiles, TILE_CELLS, 0, s>>>(k, tiles, src, NV, dst, isg);
}
template <bool BF>
void Lowp16<BF>::decode(const LowpK* k, const Tile* tiles, int ntiles, const u16* src, long long NV, double* dst,
                        int isg, cudaStream_t s)
{
    if (ntiles > 0) k_decode16<BF><<<ntiles, TILE_CELLS, 0, s>>>(k, tiles, src, NV, dst, isg);
}
template <bool BF>
void Lowp16<BF>::decode_flat(const LowpK* k, const u16* src, long long n, double* dst, int isg, cudaStream_t s)
{
    if (n > 0) k_decode_flat16<BF><<<(unsigned)((n * NQ + 255) / 256), 256, 0, s>>>(k, src, n, dst, isg);
}
template <bool BF>
void Lowp16<BF>::conserved(const LowpK* k, const Tile* tiles, int ntiles, double dV, double* out5, cudaStream_t s)
{
    if (ntiles > 0) k_conserved16<BF><<<ntiles, TILE_CELLS, 0, s>>>(k, tiles, dV, out5);
}
template <bool BF>
void Lowp16<BF>::macro(const LowpK* k, const CodecTab& ct, const Tile* tiles, int ntiles, double* out19,
                       cudaStream_t s)
{
    if (ntiles > 0) k_macro16<BF><<<ntiles, TILE_CELLS, 0, s>>>(k, ct, tiles, out19);
}

}  // namespace mbg
