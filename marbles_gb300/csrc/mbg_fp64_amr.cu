// mbg_fp64_amr.cu -- FP64 level-to-level transfers: explosion of the coarse
// level into a fine level's ghost shell and coalescence of the fine level onto
// the coarse level.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "mbg_fp64.cuh"

namespace mbg {

// ---- explosion: conservative linear interpolation of the coarse level ------
// (AMReX cell_cons_interp as called at Source/FillPatchOps.H:124-128: MC
// slopes, one limiter factor per direction shared by all 27 components)

// storage index (without the component offset) of coarse cell p0 + s e_d, or
// -1 where no coarse box holds it
__device__ __forceinline__ long long crse_index(const LV& C, const int p0[3], int d, int s)
{
    int p[3] = {p0[0], p0[1], p0[2]};
    p[d] += s;
    wrap_pos(C, p);
    const int o = owner_of(C, p);
    if (o < 0) return -1;  // plans reject fine levels whose stencil leaves the coarse level
    const DevBox& O = C.box[o];
    return O.voff + val_lin(O, p[0] - O.lo[0], p[1] - O.lo[1], p[2] - O.lo[2]);
}

// The slopes and the limiter depend only on the coarse cell, so they are
// computed once per coarse cell under the ghost shell (a slot), not once per
// fine child; each child then evaluates the same expression as before.
//
// 1. the 7 coarse storage indices of each slot (centre, -/+ x, y, z; -1 where
//    no coarse box holds the cell); limiter reset to 1
__global__ void k_xindex(LV C, const XSlot* __restrict__ xc, long long nx, int* __restrict__ ix,
                         double* __restrict__ al)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nx) return;
    const XSlot c = xc[e];
    const int cp[3] = {c.x, c.y, c.z};
    ix[e] = (int)crse_index(C, cp, 0, 0);
    for (int d = 0; d < 3; ++d) {
        ix[(1 + 2 * d) * nx + e] = (int)crse_index(C, cp, d, -1);
        ix[(2 + 2 * d) * nx + e] = (int)crse_index(C, cp, d, 1);
    }
    for (int k = 0; k < 6; ++k) al[k * nx + e] = 1.0;
}

// 2. per (slot, direction): value, centred slopes, and each axis' limiter
//    ratio folded into the slot's minimum (non-negative doubles order like
//    their bit patterns, so an integer atomicMin is exact and order-free,
//    as fmin is)
__global__ void k_xslope(LV C, const int* __restrict__ ix, long long nx, const double* __restrict__ fc,
                         const double* __restrict__ gc_, double* __restrict__ xs, double* __restrict__ al)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (e >= nx) return;
    int id[7];
    for (int k = 0; k < 7; ++k) id[k] = ix[k * nx + e];
    for (int lat = 0; lat < 2; ++lat) {
        const double* __restrict__ v = (lat ? gc_ : fc) + (long long)q * C.N;
        double u[7];
        for (int k = 0; k < 7; ++k) u[k] = id[k] >= 0 ? v[id[k]] : 0.0;
        double* o = xs + ((long long)(lat * 4) * NQ + q) * nx + e;
        o[0] = u[0];
        for (int d = 0; d < 3; ++d) {
            const double u0 = u[0], um = u[1 + 2 * d], up = u[2 + 2 * d];
            const double cen = 0.5 * (up - um);
            const double forw = 2.0 * (up - u0);
            const double back = 2.0 * (u0 - um);
            const double slp = (forw * back >= 0.0) ? fmin(fabs(forw), fabs(back)) : 0.0;
            o[(long long)(1 + d) * NQ * nx] = cen;
            // r = min(slp, |cen|) / |cen| is exactly 1 unless slp < |cen|
            // (x / x = 1), and only r < 1 lowers the limiter: the division
            // runs only there
            if (cen != 0.0 && slp < fabs(cen)) {
                const double r = slp / fabs(cen);
                if (r < 1.0)
                    atomicMin((unsigned long long*)&al[(lat * 3 + d) * nx + e],
                              (unsigned long long)__double_as_longlong(r));
            }
        }
    }
}

// 3. one thread per fine ghost cell: u0 + sum_d off_d (alpha_d slope_d)
__global__ void k_xfill(LV F, const GhostCell* __restrict__ gl, const int* __restrict__ slot, long long n,
                        const double* __restrict__ xs, const double* __restrict__ al, long long nx,
                        double* __restrict__ fg, double* __restrict__ gg)
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
    const long long sl = slot[e];
    for (int lat = 0; lat < 2; ++lat) {
        double* __restrict__ out = lat ? gg : fg;
        const double a0 = al[(lat * 3 + 0) * nx + sl], a1 = al[(lat * 3 + 1) * nx + sl],
                     a2 = al[(lat * 3 + 2) * nx + sl];
        const double* __restrict__ x = xs + (long long)(lat * 4) * NQ * nx + sl;
        for (int q = 0; q < NQ; ++q) {
            const double u0 = x[(long long)q * nx];
            const double cx = x[(long long)(NQ + q) * nx];
            const double cy = x[(long long)(2 * NQ + q) * nx];
            const double cz = x[(long long)(3 * NQ + q) * nx];
            out[q * F.NG + gi] = u0 + off[0] * (a0 * cx) + off[1] * (a1 * cy) + off[2] * (a2 * cz);
        }
    }
}

// ---- coalescence: masked average of the 8 fine children --------------------
// (masked_avgdown, Source/Utilities.H:315-350).  into_state: write into the
// coarse state buffer directly (initial average_down, ng = 0); otherwise into
// the coarse post-stream override buffer, with the code NOOVR64 where every
// child is masked (the step then pulls the coarse cell's own streamed value).  One thread per (coarse cell, direction):
// blockIdx.y is the direction, so a warp reads one component of 32
// consecutive coarse cells' children.
// The mask test |v - (-1)| > SMALL_NUM of masked_avgdown without FP64
// arithmetic: v - (-1) is exact for v in [-2, -0.5] (Sterbenz) and at least
// 0.5 in magnitude elsewhere, so a child is masked exactly when v is NaN or
// lies in [lo, hi], lo the smallest double >= -1 - SMALL_NUM and hi the
// largest <= SMALL_NUM - 1 (both negative, found exactly on the host).  For
// negative doubles the unsigned bit pattern grows with the magnitude.
struct MaskBits {
    unsigned long long lo, hi;   // bit patterns of lo (the larger) and hi
};

__device__ __forceinline__ bool child_masked(double v, const MaskBits& mb)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const bool nan = (u & 0x7FFFFFFFFFFFFFFFULL) > 0x7FF0000000000000ULL;
    return nan || (u >= mb.hi && u <= mb.lo);
}

__global__ void k_coalesce(LV C, LV F, BCParams P, Phys64 ph, MaskBits mb, const CoalesceCell* cl, long long n,
                           const double* ff, const double* gf, const double* ffg, const double* gfg,
                           const double* fcA, const double* gcA, const double* fcAg, const double* gcAg,
                           double* fcB, double* gcB, int into_state)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (e >= n) return;
    const CoalesceCell cc = cl[e];
    const DevBox& O = C.box[cc.cbox];
    const DevBox& A = F.box[cc.fbox];
    const long long cell = O.voff + val_lin(O, cc.cx, cc.cy, cc.cz);
    const bool inA = cc.fx >= 0 && cc.fy >= 0 && cc.fz >= 0 && cc.fx + 1 < A.n[0] && cc.fy + 1 < A.n[1] &&
                     cc.fz + 1 < A.n[2];
    for (int lat = 0; lat < 2; ++lat) {
        const double* v = lat ? gf : ff;
        const double* vg = lat ? gfg : ffg;
        const double* cA = lat ? gcA : fcA;
        double s = 0.0;
        int cnt = 0;   // children kept; the reference's FP64 count 1.0, 2.0, ... exactly
        if (inA) {
            // the eight children are valid cells of box A: fixed offsets
            const double* c0 = v + (long long)q * F.N + A.voff + val_lin(A, cc.fx, cc.fy, cc.fz);
            for (int kr = 0; kr < 2; ++kr)
                for (int jr = 0; jr < 2; ++jr)
                    for (int ir = 0; ir < 2; ++ir) {
                        const double fv = c0[kr * A.sz + jr * A.sy + ir];
                        if (!child_masked(fv, mb)) { s += fv; ++cnt; }
                    }
        } else {
            for (int kr = 0; kr < 2; ++kr)
                for (int jr = 0; jr < 2; ++jr)
                    for (int ir = 0; ir < 2; ++ir) {
                        const double fv = fab_value(F, A, cc.fx + ir, cc.fy + jr, cc.fz + kr, q, v, vg);
                        if (!child_masked(fv, mb)) { s += fv; ++cnt; }
                    }
        }
        double r;
        // s / 8 and s * 0.125 are the same correctly rounded value
        if (cnt == 8) r = s * 0.125;
        else if (cnt > 0) r = s / (double)cnt;
        else if (into_state) r = cA[q * C.N + cell];
        else r = __longlong_as_double(NOOVR64);   // the step pulls the cell's own streamed value
        (lat ? gcB : fcB)[q * C.N + cell] = r;
    }
}

void launch_explode(const LevelPlan& fine, const LevelPlan& crse, const double* fc, const double* gc, double* fg,
                    double* gg, cudaStream_t s)
{
    if (fine.nghost_cells == 0 || fine.nx == 0) return;
    const unsigned bx = (unsigned)((fine.nx + 127) / 128);
    k_xindex<<<bx, 128, 0, s>>>(crse.view64, fine.xc, fine.nx, fine.xix, fine.xal);
    k_xslope<<<dim3(bx, NQ), 128, 0, s>>>(crse.view64, fine.xix, fine.nx, fc, gc, fine.xs, fine.xal);
    k_xfill<<<(unsigned)((fine.nghost_cells + 127) / 128), 128, 0, s>>>(
        fine.view64, fine.ghost_list, fine.xslot, fine.nghost_cells, fine.xs, fine.xal, fine.nx, fg, gg);
}

// lo = the smallest double >= -1 - t and hi = the largest double <= t - 1
// (t = SMALL_NUM > 0, tiny), from an exact TwoSum of each rounded sum
static MaskBits mask_bits(double t)
{
    auto two_sum = [](double a, double b, double& err) {
        const double s = a + b;
        const double bb = s - a;
        err = (a - (s - bb)) + (b - bb);
        return s;
    };
    double e;
    double lo = two_sum(-1.0, -t, e);
    if (e > 0.0) lo = std::nextafter(lo, 0.0);             // the real sum lies above the rounded one
    double hi = two_sum(t, -1.0, e);
    if (e < 0.0) hi = std::nextafter(hi, -2.0);            // the real sum lies below the rounded one
    MaskBits mb;
    std::memcpy(&mb.lo, &lo, sizeof lo);
    std::memcpy(&mb.hi, &hi, sizeof hi);
    return mb;
}

void launch_coalesce(const LevelPlan& crse, const LevelPlan& fine, const BCParams& P, const Phys64& ph,
                     const CoalesceCell* list, long long n, const double* ff, const double* gf, const double* ffg,
                     const double* gfg, const double* fcA, const double* gcA, const double* fcAg,
                     const double* gcAg, double* fcB, double* gcB, int into_state, cudaStream_t s)
{
    if (n == 0) return;
    const int th = 128;
    const dim3 grid((unsigned)((n + th - 1) / th), NQ);
    k_coalesce<<<grid, th, 0, s>>>(crse.view64, fine.view64, P, ph, mask_bits(ph.small_num), list, n, ff, gf, ffg,
                                   gfg, fcA, gcA, fcAg, gcAg, fcB, gcB, into_state);
}

// ---- regrid: every cell of a new fine level from the coarse level ----------
// (LBM::RemakeLevel / MakeNewLevelFromCoarse through FillPatchTwoLevels /
// InterpFromCoarseLevel with cell_cons_interp: per fine cell, the coarse
// parent's value, centred and MC-limited one-sided slopes, one limiter factor
// per direction over the 27 components, and the value at the child's offset)
__global__ void k_interp_level(LV F, LV C, const Tile* tiles, const double* c, double* out)
{
    int b, x, y, z;
    long long cl;
    if (!cell_of_tile(F, tiles, b, x, y, z, cl)) return;
    const DevBox& B = F.box[b];
    const int f[3] = {B.lo[0] + x, B.lo[1] + y, B.lo[2] + z};
    const int p0[3] = {f[0] >> 1, f[1] >> 1, f[2] >> 1};
    const long long i0 = crse_index(C, p0, 0, 0);
    long long ip[3], im[3];
    for (int d = 0; d < 3; ++d) {
        ip[d] = crse_index(C, p0, d, 1);
        im[d] = crse_index(C, p0, d, -1);
    }
    const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
    double* o = out + B.hoff * NQ + cl;
    if (i0 < 0 || ip[0] < 0 || ip[1] < 0 || ip[2] < 0 || im[0] < 0 || im[1] < 0 || im[2] < 0) {
        for (int n = 0; n < NQ; ++n) o[n * vol] = __longlong_as_double(0x7FF8000000000000LL);
        return;   // the host checks nesting first; a NaN marks a stencil outside the coarse level
    }
    double alpha[3] = {1.0, 1.0, 1.0};
    for (int d = 0; d < 3; ++d)
        for (int n = 0; n < NQ; ++n) {
            const double u0 = c[n * C.N + i0], up = c[n * C.N + ip[d]], um = c[n * C.N + im[d]];
            const double cen = 0.5 * (up - um);
            const double forw = 2.0 * (up - u0);
            const double back = 2.0 * (u0 - um);
            const double slp = (forw * back >= 0.0) ? fmin(fabs(forw), fabs(back)) : 0.0;
            if (cen != 0.0) alpha[d] = fmin(alpha[d], fmin(slp, fabs(cen)) / fabs(cen));
        }
    double off[3];
    for (int d = 0; d < 3; ++d) off[d] = ((f[d] - 2 * p0[d]) + 0.5) / 2.0 - 0.5;
    for (int n = 0; n < NQ; ++n) {
        const double u0 = c[n * C.N + i0];
        double cen[3];
        for (int d = 0; d < 3; ++d) cen[d] = 0.5 * (c[n * C.N + ip[d]] - c[n * C.N + im[d]]);
        o[n * vol] = u0 + off[0] * (alpha[0] * cen[0]) + off[1] * (alpha[1] * cen[1]) + off[2] * (alpha[2] * cen[2]);
    }
}

void launch_interp_level(const LevelPlan& fine, const LevelPlan& crse, const double* c, double* out, cudaStream_t s)
{
    if (fine.ntiles > 0) k_interp_level<<<fine.ntiles, TILE_CELLS, 0, s>>>(fine.view64, crse.view64, fine.tiles, c, out);
}

}  // namespace mbg
