// mbg_level.cuh -- device view of one AMR level and the pull form of the
// reference's stream with its ghost-cell semantics.
//
// Layout in HBM (per level):
//   * populations of valid cells, component-major over the whole level:
//       v[q * N + voff(box) + k * sz + j * sy + i]
//     The FP64 form stores valid cells only (sy = nx, sz = nx ny, each box
//     contiguous); the 16-bit form pads every box by one cell on each side
//     (sy = nx + 2, sz = (nx + 2)(ny + 2)) and fills the pad with the
//     streamed values that cross the box faces.
//   * for fine levels, a private ghost fab per box (the box grown by 3),
//     used only at cells no valid box of the level covers (the coarse-fine
//     ghost shell):  vg[q * NG + goff(box) + ((k+3)(ny+6) + (j+3))(nx+6) + (i+3)]
//   * flags: one byte per cell of each grown box (bit 0 is_fluid, bit 1
//     eb_boundary, bit 2 "overwritten by coalescence" on coarse levels)
//   * an owner map on a grid of G^3-cell bins (G = gcd of all box corners),
//     giving the box whose valid region holds a bin, or -1.
//
// The reference streams by pushing into a temporary preset to -1
// (Source/LBM.cpp:558-604) and then refreshes ghost cells from neighbouring
// boxes (FillBoundary) and from the physical-BC functor (Source/BC.H:345-471,
// Source/FillPatchOps.H:75-132).  streamed() below returns, for a target
// cell and direction, exactly the value that push + ghost refresh leaves
// there, reading the previous state directly:
//   * target solid                                  -> -1
//   * source outside the target box's grown fab     -> -1
//   * source solid (half-way bounce-back)           -> f(target, opp(q))
//   * source outside the domain (non-periodic side) -> physical-BC value
//   * otherwise the source's value, taken from the owning box's valid cells
//     (periodic images included) or, where no box covers the source, from
//     the target box's own ghost fab.
#pragma once

#include "mbg_physics.cuh"

namespace mbg {

enum : uint8_t { FL_FLUID = 1, FL_EBB = 2, FL_OVR = 4 };

struct DevBox {
    int lo[3];
    int n[3];
    int sy, sz;       // strides of the box's cell array along y and z
    long long voff;   // storage index of the box's valid cell (0,0,0)
    long long hoff;   // first valid cell of the box in host (level cell) order
    long long foff;   // first cell of the box's grown flag fab
    long long goff;   // first cell of the box's grown ghost fab (-1: none)
    int all_fluid;    // no solid cell anywhere in the grown fab
    int vfluid;       // every cell of the box grown by one is fluid
    int phys;         // index of the box's physical parameters (batched domains)
    int own_domain;   // the box is a periodic domain of its own (batched domains)
};

// boundary conditions of the domain (level 0 only)
struct BCParams {
    int bc[6];        // bc_lo[0..2], bc_hi[0..2]
    int velbc;        // MBG_VBC_*
    int vbc_dir, vbc_nd, vbc_td;
    double u_ref, rho0, temp, gamma, Rg;
    double prob_lo[3], prob_hi[3], dx[3];
};

template <class S>
struct LevelView {
    const DevBox* box;
    int nbox;
    int dlo[3], dhi[3];
    int per[3];
    const int* omap;
    int G[3], nb[3];
    long long N;      // valid cells of the level (component stride)
    long long NG;     // ghost-fab cells of the level (component stride)
    const uint8_t* flags;
};

__device__ __forceinline__ long long fab_lin(const DevBox& B, int x, int y, int z)
{
    return ((long long)(z + 3) * (B.n[1] + 6) + (y + 3)) * (B.n[0] + 6) + (x + 3);
}
// storage offset of box-local (x,y,z) from the box's valid origin; with
// unpadded strides (sy = nx, sz = nx ny) this is the valid-cell order
__device__ __forceinline__ long long val_lin(const DevBox& B, int x, int y, int z)
{
    return (long long)z * B.sz + (long long)y * B.sy + x;
}

template <class S>
__device__ __forceinline__ uint8_t flag_at(const LevelView<S>& L, const DevBox& B, int x, int y, int z)
{
    return L.flags[B.foff + fab_lin(B, x, y, z)];
}

template <class S>
__device__ __forceinline__ bool in_valid(const DevBox& B, int x, int y, int z)
{
    return (unsigned)x < (unsigned)B.n[0] && (unsigned)y < (unsigned)B.n[1] && (unsigned)z < (unsigned)B.n[2];
}

// wrap a global position periodically; false if outside a non-periodic side
template <class S>
__device__ __forceinline__ bool wrap_pos(const LevelView<S>& L, int p[3])
{
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (p[d] < L.dlo[d] || p[d] > L.dhi[d]) {
            if (!L.per[d]) return false;
            const int len = L.dhi[d] - L.dlo[d] + 1;
            int r = (p[d] - L.dlo[d]) % len;
            if (r < 0) r += len;
            p[d] = L.dlo[d] + r;
        }
    }
    return true;
}

template <class S>
__device__ __forceinline__ int owner_of(const LevelView<S>& L, const int p[3])
{
    if (p[0] < L.dlo[0] || p[1] < L.dlo[1] || p[2] < L.dlo[2] || p[0] > L.dhi[0] || p[1] > L.dhi[1] ||
        p[2] > L.dhi[2])
        return -1;
    const int bi = (p[0] - L.dlo[0]) / L.G[0];
    const int bj = (p[1] - L.dlo[1]) / L.G[1];
    const int bk = (p[2] - L.dlo[2]) / L.G[2];
    return L.omap[((long long)bk * L.nb[1] + bj) * L.nb[0] + bi];
}

template <class S>
__device__ __forceinline__ bool outside_nonperiodic(const LevelView<S>& L, const int p[3])
{
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (!L.per[d] && (p[d] < L.dlo[d] || p[d] > L.dhi[d])) return true;
    return false;
}

// raw storage value of the -1 sentinel (16-bit forms reserve a NaN code)
template <class S>
__device__ __forceinline__ S sentinel_raw() { return (S)-1.0; }
template <>
__device__ __forceinline__ uint16_t sentinel_raw<uint16_t>() { return (uint16_t)0xFFFFu; }

// Value of a component array at box-local position (x,y,z) of box B's fab
// (valid, covered ghost or uncovered ghost).  The position must not lie
// outside a non-periodic side of the domain.
template <class S>
__device__ __forceinline__ S fab_value(const LevelView<S>& L, const DevBox& B, int x, int y, int z, int q,
                                       const S* v, const S* vg)
{
    if (in_valid<S>(B, x, y, z)) return v[q * L.N + B.voff + val_lin(B, x, y, z)];
    int p[3] = {B.lo[0] + x, B.lo[1] + y, B.lo[2] + z};
    wrap_pos(L, p);
    const int o = owner_of(L, p);
    if (o >= 0) {
        const DevBox& O = L.box[o];
        return v[q * L.N + O.voff + val_lin(O, p[0] - O.lo[0], p[1] - O.lo[1], p[2] - O.lo[2])];
    }
    if (B.goff < 0 || vg == nullptr) return sentinel_raw<S>();  // no storage there (plans exclude this case)
    return vg[q * L.NG + B.goff + fab_lin(B, x, y, z)];
}

// velocity-BC functor (Source/VelocityBC.H:13-199) at ghost position p
__device__ inline void vel_bc_state(const BCParams& P, const int dhi[3], const int p[3], double& rho, double vel[3],
                                    double& Rg, double& temp, double& gamma)
{
    switch (P.velbc) {
    case 1:  // Constant
        rho = P.rho0; vel[P.vbc_dir] = P.u_ref; Rg = P.Rg; temp = P.temp; gamma = P.gamma;
        break;
    case 2: {  // Channel
        rho = P.rho0;
        const double c1 = p[1] * (dhi[1] - p[1]);
        const double c2 = p[2] * (dhi[2] - p[2]);
        const double d = (double)(dhi[1] + 1);
        vel[0] = 16.0 * P.u_ref * c1 * c2 / (d * d * d * d);
        Rg = P.Rg; temp = P.temp; gamma = P.gamma;
    } break;
    case 3: {  // Parabolic
        rho = P.rho0;
        const int nd = P.vbc_nd, td = P.vbc_td;
        const double height = P.prob_hi[nd] - P.prob_lo[nd];
        const double x = P.prob_lo[nd] + (p[nd] + 0.5) * P.dx[nd];
        vel[td] = 4.0 * P.u_ref * x * (height - x) / (height * height);
        Rg = P.Rg; temp = P.temp; gamma = P.gamma;
    } break;
    default:
        break;
    }
}

// Physical-BC value of direction q at ghost cell s (box-local, outside a
// non-periodic side), as left by the reference's functor at the start of
// the step.  Faces are applied in the functor's loop order; the last
// non-periodic side that s lies outside of decides.  Outflow reads the
// next cell inward, which may itself be a ghost on another side (edges and
// corners): the loop then continues from that cell.
template <int q, class S, class R, class Dec>
__device__ R bc_value(const LevelView<S>& L, const BCParams& P, const DevBox& B, int sx, int sy, int sz,
                      bool is_g, const S* v, const S* vg, const Lattice<double>& lat, const Dec& dec)
{
    constexpr int bq = opp(q), mx = mirror(q, 0), my = mirror(q, 1), mz = mirror(q, 2);
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    int s[3] = {sx, sy, sz};
    for (int depth = 0; depth < 3; ++depth) {
        // the functor writes direction q only if s + e_q is in the box's valid region
        if (!in_valid<S>(B, s[0] + ex, s[1] + ey, s[2] + ez)) return (R)-1.0;
        int face = -1, ndir = 0;
        for (int idir = 0; idir < 3; ++idir) {
            const int g = B.lo[idir] + s[idir];
            if (g < L.dlo[idir] && P.bc[idir] != 0) { face = idir; ndir = 1; }
            if (g > L.dhi[idir] && P.bc[idir + 3] != 0) { face = idir + 3; ndir = -1; }
        }
        if (face < 0) return (R)-1.0;
        const int idir = face % 3;
        const int bc = P.bc[face];
        const int tx = s[0] + ex, ty = s[1] + ey, tz = s[2] + ez;
        switch (bc) {
        case 1:  // no-slip: data(iv + ev, bounce(q))
            return dec(fab_value(L, B, tx, ty, tz, bq, v, vg), bq);
        case 6: return dec(fab_value(L, B, tx, ty, tz, mx, v, vg), mx);
        case 7: return dec(fab_value(L, B, tx, ty, tz, my, v, vg), my);
        case 8: return dec(fab_value(L, B, tx, ty, tz, mz, v, vg), mz);
        case 2: {  // velocity
            int gp[3] = {B.lo[0] + s[0], B.lo[1] + s[1], B.lo[2] + s[2]};
            double vel[3] = {0.0, 0.0, 0.0}, Rg = 1.0, temp = 1.0 / 3.0, gamma = 5.0 / 3.0, rho = 0.0;
            vel_bc_state(P, L.dhi, gp, rho, vel, Rg, temp, gamma);
            if (is_g) return (R)eq_g_plain<double>(q, rho, vel, Rg, temp, gamma, lat);
            return (R)eq_f_plain<double>(q, rho, vel, Rg * temp);
        }
        case 3: {  // pressure (Source/BC.H:222-321, dispatched at 421-446)
            int gp[3] = {B.lo[0] + s[0], B.lo[1] + s[1], B.lo[2] + s[2]};
            double vel[3] = {0.0, 0.0, 0.0}, Rg = 1.0, temp = 1.0 / 3.0, gamma = 5.0 / 3.0, rho_bc = 1.0;
            vel_bc_state(P, L.dhi, gp, rho_bc, vel, Rg, temp, gamma);
            double vb[3] = {0.0, 0.0, 0.0};
            if (is_g) {
                // the energy lattice uses the fixed outlet density 1 (BC.H:438-441)
                const double rho_bcout = 1.0;
                vb[idir] = ndir * (1.0 - (rho_bcout) / rho_bc);
                return (R)eq_g_plain<double>(q, rho_bc, vb, Rg, temp, gamma, lat);
            }
            // density leaving through the face and tangential to it, from the
            // populations of the interior cell's neighbours that point back
            // across the face or along it, in direction order
            double rho_out = 0.0, rho_tan = 0.0;
            for (int qq = 0; qq < NQ; ++qq) {
                const int bq2 = opp(qq);
                const int ei = idir == 0 ? ev_x(bq2) : (idir == 1 ? ev_y(bq2) : ev_z(bq2));
                if (ei != -ndir && ei != 0) continue;
                const double val =
                    (double)dec(fab_value(L, B, tx + ev_x(qq), ty + ev_y(qq), tz + ev_z(qq), bq2, v, vg), bq2);
                if (ei == -ndir) rho_out += 2.0 * val;
                else rho_tan += 1.0 * val;
            }
            vb[idir] = ndir * (1.0 - (rho_out + rho_tan) / rho_bc);
            return (R)eq_f_plain<double>(q, rho_bc, vb, Rg * temp);
        }
        case 5: {  // outflow: data(iv + ndir e_idir, q)
            s[idir] += ndir;
            int gp[3] = {B.lo[0] + s[0], B.lo[1] + s[1], B.lo[2] + s[2]};
            if (!outside_nonperiodic(L, gp)) return dec(fab_value(L, B, s[0], s[1], s[2], q, v, vg), q);
            continue;
        }
        default:
            return (R)-1.0;
        }
    }
    return (R)-1.0;
}

}  // namespace mbg
