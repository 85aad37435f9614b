// mbg_physics.cuh -- D3Q27 lattice and the energyD3Q27 collision, as device
// functions templated on the arithmetic type.
//
// The lattice order, weights and bounce maps are those of
// Source/Stencil.H:49-167 (NREL/marbles).  Every formula keeps the operand
// order of the reference expression it restates (cited per function), so
// that an FP64 build without FMA contraction reproduces the reference's
// rounding.  Loops over the 27 directions are unrolled at compile time and
// terms whose lattice factor is 0 are dropped; with factors of +-1 the
// remaining adds are the same IEEE operations as the reference's
// "acc += e * f" with e in {-1, 0, 1}.
#pragma once

#include <cstdint>
#include <type_traits>

namespace mbg {

constexpr int NQ = 27;

// Source/Stencil.H:49-79, direction q -> (ex, ey, ez)
__host__ __device__ constexpr int ev_x(int q)
{
    constexpr int t[NQ] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1,
                           0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
    return t[q];
}
__host__ __device__ constexpr int ev_y(int q)
{
    constexpr int t[NQ] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0,
                           1, -1, 1, -1, 1, -1, -1, 1, -1, 1, 1, -1};
    return t[q];
}
__host__ __device__ constexpr int ev_z(int q)
{
    constexpr int t[NQ] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1,
                           1, -1, -1, 1, 1, -1, 1, -1, -1, 1, -1, 1};
    return t[q];
}
__host__ __device__ constexpr int ev_c(int q, int d) { return d == 0 ? ev_x(q) : d == 1 ? ev_y(q) : ev_z(q); }

__host__ __device__ constexpr int find_dir(int a, int b, int c)
{
    for (int q = 0; q < NQ; ++q)
        if (ev_x(q) == a && ev_y(q) == b && ev_z(q) == c) return q;
    return -1;
}
// Source/Stencil.H:125-167: full inversion and single-axis mirrors
__host__ __device__ constexpr int opp(int q) { return find_dir(-ev_x(q), -ev_y(q), -ev_z(q)); }
__host__ __device__ constexpr int mirror(int q, int d)
{
    return d == 0 ? find_dir(-ev_x(q), ev_y(q), ev_z(q))
         : d == 1 ? find_dir(ev_x(q), -ev_y(q), ev_z(q))
                  : find_dir(ev_x(q), ev_y(q), -ev_z(q));
}
__host__ __device__ constexpr int ev_norm1(int q)
{
    return (ev_x(q) != 0) + (ev_y(q) != 0) + (ev_z(q) != 0);
}

// M(q) for q = 0 .. 26 in order, with q a literal: the unrolled direction
// loops of the kernels (plain expansion, nothing captured)
#define MBG_UNROLL27(M) M(0) M(1) M(2) M(3) M(4) M(5) M(6) M(7) M(8) M(9) M(10) M(11) M(12) M(13) M(14) \
    M(15) M(16) M(17) M(18) M(19) M(20) M(21) M(22) M(23) M(24) M(25) M(26)

template <int Q, int N, class F>
__device__ __forceinline__ void static_for(F&& f)
{
    if constexpr (Q < N) {
        f(std::integral_constant<int, Q>{});
        static_for<Q + 1, N>(f);
    }
}

// Lattice constants computed on the host with the reference's expressions
// (Source/Stencil.H:81-90) and passed to kernels by value.
template <class R>
struct Lattice {
    R w[NQ];
    R theta0;          // Stencil::THETA0 = 1/3
    R one_bystheta0;   // 1 / (s * theta0) with s = 1 (Utilities.H:113)
    R cth[2];          // (e*e - theta0) for e*e = 0, 1
};

template <class R>
inline Lattice<R> make_lattice()
{
    Lattice<R> L{};
    const double WSC1 = 2.0 / 27.0, WFCC1 = 1.0 / 54.0, WBCC1 = 1.0 / 216.0;
    const double WO = 1.0 - (6.0 * (WSC1) + 12.0 * (WFCC1) + 8.0 * (WBCC1));
    for (int q = 0; q < NQ; ++q) {
        const int s = ev_norm1(q);
        L.w[q] = (R)(s == 0 ? WO : s == 1 ? WSC1 : s == 2 ? WFCC1 : WBCC1);
    }
    const R th = (R)(1.0 / 3.0);
    L.theta0 = th;
    const R stheta0 = (R)1.0 * th;
    L.one_bystheta0 = (R)1.0 / stheta0;
    L.cth[0] = (R)0 - th;
    L.cth[1] = (R)1 - th;
    return L;
}

// Macroscopic state of one cell (the components of Source/Constants.H)
template <class R>
struct Macro {
    R rho, u, v, w, two_rho_e;
    R pxx, pyy, pzz, pxy, pxz, pyz;
    R qx, qy, qz;
    R temp;
    R qcx, qcy, qcz;
};

// Accumulates the moments of Source/LBM.cpp:841-862 in direction order.
template <class R>
struct MomentAcc {
    R rho = 0, u = 0, v = 0, w = 0;
    R pxx = 0, pyy = 0, pzz = 0, pxy = 0, pxz = 0, pyz = 0;
    R tre = 0, qx = 0, qy = 0, qz = 0;

    template <int q>
    __device__ __forceinline__ void add(R fq, R gq)
    {
        constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
        rho += fq;
        if constexpr (ex == 1) u += fq; else if constexpr (ex == -1) u -= fq;
        if constexpr (ey == 1) v += fq; else if constexpr (ey == -1) v -= fq;
        if constexpr (ez == 1) w += fq; else if constexpr (ez == -1) w -= fq;
        if constexpr (ex != 0) pxx += fq;
        if constexpr (ey != 0) pyy += fq;
        if constexpr (ex * ey == 1) pxy += fq; else if constexpr (ex * ey == -1) pxy -= fq;
        if constexpr (ez != 0) pzz += fq;
        if constexpr (ex * ez == 1) pxz += fq; else if constexpr (ex * ez == -1) pxz -= fq;
        if constexpr (ey * ez == 1) pyz += fq; else if constexpr (ey * ez == -1) pyz -= fq;
        tre += gq;
        if constexpr (ex == 1) qx += gq; else if constexpr (ex == -1) qx -= gq;
        if constexpr (ey == 1) qy += gq; else if constexpr (ey == -1) qy -= gq;
        if constexpr (ez == 1) qz += gq; else if constexpr (ez == -1) qz -= gq;
    }

    // Source/LBM.cpp:863-903 and Utilities.H:189-210
    __device__ __forceinline__ Macro<R> finish(R mesh_speed, R Rg, R cv) const
    {
        Macro<R> m;
        m.rho = rho;
        R uu = u, vv = v, ww = w;
        uu *= mesh_speed / rho;
        vv *= mesh_speed / rho;
        ww *= mesh_speed / rho;
        m.u = uu; m.v = vv; m.w = ww;
        m.pxx = pxx; m.pyy = pyy; m.pzz = pzz; m.pxy = pxy; m.pxz = pxz; m.pyz = pyz;
        m.two_rho_e = tre; m.qx = qx; m.qy = qy; m.qz = qz;
        const R t = ((R)0.50 / cv) * ((tre / rho) - (uu * uu + vv * vv + ww * ww));
        m.temp = t;
        m.qcx = rho * uu * (((R)1.0 - (R)3.0 * Rg * t) - uu * uu);
        m.qcy = rho * vv * (((R)1.0 - (R)3.0 * Rg * t) - vv * vv);
        m.qcz = rho * ww * (((R)1.0 - (R)3.0 * Rg * t) - ww * ww);
        return m;
    }
};

// Per-cell data of the equilibria: the product-form f_eq
// (Utilities.H:42-63) factored over the three values of each axis, and the
// Grad-expansion g_eq (Utilities.H:65-163) with its direction-independent
// coefficients precomputed.
template <class R>
struct Equilibrium {
    R rf[3][3];        // rho * phi_x[ex] * phi_y[ey], index e+1
    R phz[3];          // phi_z[ez]
    R grho;            // 2 rho E
    R a1[3];           // a1x, a1y, a1z
    R A1[2], A2[2], A4[2];  // (e*e - theta0) * a2xx / a2yy / a2zz
    R t3, t5, t6;      // 2 a2xy, 2 a2xz, 2 a2yz

    __device__ __forceinline__ static R phi(int e, R u, R p)
    {
        // ev * 0.5 * vel + |ev| * (1.50 * p - 1.0) - p + 1.0
        if (e == 0) return -p + (R)1.0;
        const R a = (e == 1 ? (R)0.5 : (R)-0.5) * u;
        return a + ((R)1.50 * p - (R)1.0) - p + (R)1.0;
    }

    template <int q>
    __device__ __forceinline__ R feq() const
    {
        constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
        return rf[ex + 1][ey + 1] * phz[ez + 1];
    }

    template <int q, class LT>
    __device__ __forceinline__ R geq(const LT& lat) const
    {
        constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
        R f = grho;
        if constexpr (ex == 1) f = f + a1[0]; else if constexpr (ex == -1) f = f + (-a1[0]);
        if constexpr (ey == 1) f = f + a1[1]; else if constexpr (ey == -1) f = f + (-a1[1]);
        if constexpr (ez == 1) f = f + a1[2]; else if constexpr (ez == -1) f = f + (-a1[2]);
        R s = A1[ex * ex] + A2[ey * ey];
        if constexpr (ex * ey == 1) s = s + t3; else if constexpr (ex * ey == -1) s = s + (-t3);
        s = s + A4[ez * ez];
        if constexpr (ex * ez == 1) s = s + t5; else if constexpr (ex * ez == -1) s = s + (-t5);
        if constexpr (ey * ez == 1) s = s + t6; else if constexpr (ey * ez == -1) s = s + (-t6);
        f += (R)0.5 * s;
        f *= lat.w[q];
        return f;
    }
};

// Source/LBM.cpp:646-760 for one fluid cell; returns omega (LBM.cpp:787-790)
template <class R, class LT>
__device__ __forceinline__ R build_equilibrium(const Macro<R>& m, R dqx, R dqy, R dqz, R nu, R alpha, R dt,
                                               R Rg, R cv, const LT& lat, Equilibrium<R>& E)
{
    const R rho = m.rho;
    const R vel0 = m.u, vel1 = m.v, vel2 = m.w;
    const R temperature = m.temp;
    const R omega = (R)1.0 / (nu / (Rg * temperature * dt) + (R)0.5);
    const R omega_one = (R)1.0 / (alpha / (Rg * temperature * dt) + (R)0.5);
    const R omega_one_by_omega = omega_one / omega;
    const R omega_corr = ((R)2.0 - omega) / ((R)2.0 * omega * rho);
    const R pxx_ext = vel0 * vel0 + Rg * temperature + dt * (omega_corr)*dqx;
    const R pyy_ext = vel1 * vel1 + Rg * temperature + dt * (omega_corr)*dqy;
    const R pzz_ext = vel2 * vel2 + Rg * temperature + dt * (omega_corr)*dqz;

    R phx[3], phy[3];
#pragma unroll
    for (int e = -1; e <= 1; ++e) {
        phx[e + 1] = Equilibrium<R>::phi(e, vel0, pxx_ext);
        phy[e + 1] = Equilibrium<R>::phi(e, vel1, pyy_ext);
        E.phz[e + 1] = Equilibrium<R>::phi(e, vel2, pzz_ext);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const R rx = rho * phx[a];
#pragma unroll
        for (int b = 0; b < 3; ++b) E.rf[a][b] = rx * phy[b];
    }

    // get_equilibrium_moments (Utilities.H:245-277)
    const R two_rho_e = m.two_rho_e;
    const R energy = two_rho_e / ((R)2.0 * rho);
    const R tmp = ((R)0.50 / cv) * ((two_rho_e / rho) - (vel0 * vel0 + vel1 * vel1 + vel2 * vel2));
    const R p = rho * Rg * tmp;
    const R h = energy + (p / rho);
    R qx_eq = (R)2.0 * rho * vel0 * h;
    R qy_eq = (R)2.0 * rho * vel1 * h;
    R qz_eq = (R)2.0 * rho * vel2 * h;
    const R rxx = (R)2.0 * rho * vel0 * vel0 * (h + (p / rho)) + (R)2.0 * p * h;
    const R ryy = (R)2.0 * rho * vel1 * vel1 * (h + (p / rho)) + (R)2.0 * p * h;
    const R rzz = (R)2.0 * rho * vel2 * vel2 * (h + (p / rho)) + (R)2.0 * p * h;
    const R rxy = (R)2.0 * rho * vel0 * vel1 * (h + (p / rho)) + (R)0;
    const R rxz = (R)2.0 * rho * vel0 * vel2 * (h + (p / rho)) + (R)0;
    const R ryz = (R)2.0 * rho * vel1 * vel2 * (h + (p / rho)) + (R)0;

    qx_eq *= omega_one_by_omega;
    qy_eq *= omega_one_by_omega;
    qz_eq *= omega_one_by_omega;
    qx_eq += ((R)1.0 - omega_one_by_omega) *
             (m.qx - (R)2.0 * vel0 * m.pxx - (R)2.0 * vel1 * m.pxy - (R)2.0 * vel2 * m.pxz - vel0 * dt * dqx);
    qy_eq += ((R)1.0 - omega_one_by_omega) *
             (m.qy - (R)2.0 * vel0 * m.pxy - (R)2.0 * vel1 * m.pyy - (R)2.0 * vel2 * m.pyz - vel1 * dt * dqy);
    qz_eq += ((R)1.0 - omega_one_by_omega) *
             (m.qz - (R)2.0 * vel0 * m.pxz - (R)2.0 * vel1 * m.pyz - (R)2.0 * vel2 * m.pzz - vel2 * dt * dqz);

    // set_extended_grad_expansion_generic with frame velocity 0, s = 1
    const R k = lat.one_bystheta0;
    const R th = lat.theta0;
    E.grho = two_rho_e;
    E.a1[0] = qx_eq * k;
    E.a1[1] = qy_eq * k;
    E.a1[2] = qz_eq * k;
    const R a2xx = (rxx - two_rho_e * th) * k * k;
    const R a2yy = (ryy - two_rho_e * th) * k * k;
    const R a2zz = (rzz - two_rho_e * th) * k * k;
    const R a2xy = rxy * k * k;
    const R a2xz = rxz * k * k;
    const R a2yz = ryz * k * k;
    E.A1[0] = lat.cth[0] * a2xx; E.A1[1] = lat.cth[1] * a2xx;
    E.A2[0] = lat.cth[0] * a2yy; E.A2[1] = lat.cth[1] * a2yy;
    E.A4[0] = lat.cth[0] * a2zz; E.A4[1] = lat.cth[1] * a2zz;
    E.t3 = (R)2.0 * a2xy;
    E.t5 = (R)2.0 * a2xz;
    E.t6 = (R)2.0 * a2yz;
    return omega;
}

// ---- boundary-condition equilibria (BC.H:143-218, IC.H:474-519) --------

// set_equilibrium_value (Utilities.H:11-40): f_eq(rho, vel, RT) for q
template <class R>
__host__ __device__ inline R eq_f_plain(int q, R rho, const R vel[3], R rt)
{
    const int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    const R pxx = vel[0] * vel[0] + rt;
    const R pyy = vel[1] * vel[1] + rt;
    const R pzz = vel[2] * vel[2] + rt;
    const R phix = ex * (R)0.5 * vel[0] + (R)(ex < 0 ? -ex : ex) * ((R)1.50 * pxx - (R)1.0) - pxx + (R)1.0;
    const R phiy = ey * (R)0.5 * vel[1] + (R)(ey < 0 ? -ey : ey) * ((R)1.50 * pyy - (R)1.0) - pyy + (R)1.0;
    const R phiz = ez * (R)0.5 * vel[2] + (R)(ez < 0 ? -ez : ez) * ((R)1.50 * pzz - (R)1.0) - pzz + (R)1.0;
    return rho * phix * phiy * phiz;
}

// Grad-expansion g_eq of (rho, vel, T) through get_energy and
// get_equilibrium_moments (BC.H:143-190 / IC.H:499-516)
template <class R>
__host__ __device__ inline R eq_g_plain(int q, R rho, const R vel[3], R Rg, R temperature, R gamma,
                                        const Lattice<R>& lat)
{
    const int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    const R cv = Rg / (gamma - (R)1.0);
    const R two_rho_e = rho * ((R)2.0 * cv * temperature + (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]));
    const R energy = two_rho_e / ((R)2.0 * rho);
    const R tmp = ((R)0.50 / cv) * ((two_rho_e / rho) - (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]));
    const R p = rho * Rg * tmp;
    const R h = energy + (p / rho);
    const R qx = (R)2.0 * rho * vel[0] * h;
    const R qy = (R)2.0 * rho * vel[1] * h;
    const R qz = (R)2.0 * rho * vel[2] * h;
    const R rxx = (R)2.0 * rho * vel[0] * vel[0] * (h + (p / rho)) + (R)2.0 * p * h;
    const R ryy = (R)2.0 * rho * vel[1] * vel[1] * (h + (p / rho)) + (R)2.0 * p * h;
    const R rzz = (R)2.0 * rho * vel[2] * vel[2] * (h + (p / rho)) + (R)2.0 * p * h;
    const R rxy = (R)2.0 * rho * vel[0] * vel[1] * (h + (p / rho)) + (R)0;
    const R rxz = (R)2.0 * rho * vel[0] * vel[2] * (h + (p / rho)) + (R)0;
    const R ryz = (R)2.0 * rho * vel[1] * vel[2] * (h + (p / rho)) + (R)0;
    const R k = lat.one_bystheta0;
    const R th = lat.theta0;
    const R a1x = qx * k, a1y = qy * k, a1z = qz * k;
    const R a2xx = (rxx - two_rho_e * th) * k * k;
    const R a2yy = (ryy - two_rho_e * th) * k * k;
    const R a2zz = (rzz - two_rho_e * th) * k * k;
    const R a2xy = rxy * k * k, a2xz = rxz * k * k, a2yz = ryz * k * k;
    R f = two_rho_e + a1x * ex + a1y * ey + a1z * ez;
    f += (R)0.5 * ((ex * ex - th) * a2xx + (ey * ey - th) * a2yy + (R)2.0 * (ex * ey - 0) * a2xy +
                   (ez * ez - th) * a2zz + (R)2.0 * (ex * ez - 0) * a2xz + (R)2.0 * (ey * ez - 0) * a2yz);
    f *= lat.w[q];
    return f;
}

}  // namespace mbg
