// mbg_adjoint.cu -- hand-written discrete adjoint of the FP64 step on one
// fully periodic box: gradient of a loss of the final temperature field with
// respect to the initial temperature field (mbg_adj_* in
// include/marbles_gb300.h).
//
// Forward.  The initial state is the equilibrium of (rho0, u0, T0(x))
// (IC.H:474-519, f = f_eq(rho, u, R T), g = the Grad g_eq); each step is the
// reference's pull-stream + collide (Source/LBM.cpp:523-807) in two passes:
// k_adj_q writes Q_corr of every cell, k_adj_step pulls, forms the moments,
// takes the q-correction gradient (one-sided at the box faces, physical
// 1/dx), builds the equilibria and relaxes.  The state is checkpointed every
// K steps.
//
// Reverse.  With s' = C(P(s)) (P the periodic pull, C the per-cell
// collision, which couples neighbours only through dQ), one reverse step is
// (the step's moment sums and dQ kept from the segment's recomputation)
//   k_adj_a1 : per cell, the transpose of the collision's Jacobian applied to
//              the adjoint of the step's output: adjoints of the 14 moment
//              sums reached through the macro fields, omega and the
//              equilibria, and of the three dQ components;
//   k_adj_a2 : per cell, the transposed gradient stencil gives the adjoint
//              of Q_corr, which joins the moment adjoints; the adjoint of
//              each pulled population is (1 - omega) lambda_out plus its
//              share of the moment adjoints, pushed back along its direction
//              (the transpose of the pull).
// Each segment of K steps is recomputed from its checkpoint and its states
// kept, then walked backwards.  The last adjoint is mapped through the
// initial-condition equilibria to dL/dT0 (derivatives with respect to T0 by a
// one-direction dual number through the same equilibrium functions).
// Everything is FP64, the adjoint accumulated over time included.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/marbles_gb300.h"
#include "mbg_kernels.h"

void mbg_set_global_error(const std::string& msg);

namespace mbg {

struct AdjBox {
    int n[3];
    long long N;
};

// workspace fields per cell (component-major [k][N])
enum { WS_LA = 0, WS_LDQ = 14, WS_OMEGA = 17, WS_RHO = 18, WS_J = 19, WS_TRE = 22, WS_N = 23 };

__device__ __forceinline__ bool adj_cell(const AdjBox& b, int& x, int& y, int& z, long long& c)
{
    c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= b.N) return false;
    x = (int)(c % b.n[0]);
    const long long r = c / b.n[0];
    y = (int)(r % b.n[1]);
    z = (int)(r / b.n[1]);
    return true;
}

__device__ __forceinline__ int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

__device__ __forceinline__ long long lin(const AdjBox& b, int x, int y, int z)
{
    return ((long long)z * b.n[1] + y) * b.n[0] + x;
}

// index of the periodic neighbour (x + dx, y + dy, z + dz)
__device__ __forceinline__ long long nbr(const AdjBox& b, int x, int y, int z, int dx, int dy, int dz)
{
    return lin(b, wrapi(x + dx, b.n[0]), wrapi(y + dy, b.n[1]), wrapi(z + dz, b.n[2]));
}

__device__ __forceinline__ MomentAcc<double> pulled_moments(const AdjBox& b, int x, int y, int z, const double* f,
                                                            const double* g, double* pf, double* pg)
{
    MomentAcc<double> acc;
#define MBG_AP(q)                                                                  \
    {                                                                              \
        const long long s = nbr(b, x, y, z, -ev_x(q), -ev_y(q), -ev_z(q));         \
        const double fq = f[q * b.N + s], gq = g[q * b.N + s];                     \
        if (pf) { pf[q] = fq; pg[q] = gq; }                                        \
        acc.template add<q>(fq, gq);                                               \
    }
    MBG_UNROLL27(MBG_AP)
#undef MBG_AP
    return acc;
}

// q-correction gradient along d at cell (x,y,z) from Q_corr of the
// neighbours (Utilities.H:279-312; one-sided at the box faces)
__device__ __forceinline__ double dq_axis(const AdjBox& b, const double* Q, int x, int y, int z, int d, double idx)
{
    int p[3] = {x, y, z};
    const int c = p[d], n = b.n[d];
    const bool p_out = c + 1 >= n, m_out = c - 1 < 0;
    const long long i0 = lin(b, x, y, z);
    int pp[3] = {x, y, z}, pm[3] = {x, y, z};
    pp[d] += 1;
    pm[d] -= 1;
    const double* Qd = Q + d * b.N;
    double vp = 0.0, vc = 0.0, vm = 0.0;
    if (p_out && m_out) {
    } else if (p_out) {
        vc = Qd[i0];
        vm = -Qd[lin(b, pm[0], pm[1], pm[2])];
    } else if (m_out) {
        vp = Qd[lin(b, pp[0], pp[1], pp[2])];
        vc = -Qd[i0];
    } else {
        vp = 0.5 * Qd[lin(b, pp[0], pp[1], pp[2])];
        vm = -0.5 * Qd[lin(b, pm[0], pm[1], pm[2])];
    }
    return (vp + vc + vm) * idx;
}

// Reverse of the macro fields (MomentAcc::finish): adjoints of rho, U and T
// (and a direct adjoint of 2 rho E) onto the moment sums rho, j, 2 rho E.
__device__ __forceinline__ void macro_reverse(const MomentAcc<double>& acc, const Phys64& ph, double lrho,
                                              const double lU[3], double lT, double ltre, double la[14])
{
    const double rho = acc.rho, tre = acc.tre;
    const double s = ph.mesh_speed / rho;
    const double U[3] = {acc.u * s, acc.v * s, acc.w * s};
    const double c = 0.50 / ph.cv;
    double lUt[3];
    for (int a = 0; a < 3; ++a) lUt[a] = lU[a] - c * 2.0 * U[a] * lT;
    ltre += c / rho * lT;
    lrho += -c * tre / (rho * rho) * lT;
    for (int a = 0; a < 3; ++a) lrho += -U[a] / rho * lUt[a];
    la[0] += lrho;
    la[1] += s * lUt[0];
    la[2] += s * lUt[1];
    la[3] += s * lUt[2];
    la[10] += ltre;
}

// Transpose of one cell's collision Jacobian (Source/LBM.cpp:621-807 and
// Utilities.H:42-277 read backwards).  In: the moment sums of the pulled
// values, dQ, the pulled values (re-read through P) and the adjoint of the
// outputs Lf/Lg (component stride lstride).
// Out: la[14] (adjoints of the moment sums, without the Q_corr part),
// ldq[3], omega.
// the pulled values of one cell, read again from the state when needed
struct CellPull {
    const AdjBox* b;
    int x, y, z;
    const double *f, *g;
    __device__ __forceinline__ long long src(int q) const
    {
        return q * b->N + nbr(*b, x, y, z, -ev_x(q), -ev_y(q), -ev_z(q));
    }
};

__device__ void collide_reverse(const MomentAcc<double>& acc, const double dq[3], const Phys64& ph, const CellPull& P,
                                const double* Lf, const double* Lg, long long lstride, double la[14], double ldq[3],
                                double& omega_out)
{
    const double ms = ph.mesh_speed, Rg = ph.Rg, cv = ph.cv, dt = ph.dt;
    const Lattice<double>& lat = ph.lat;
    const Macro<double> m = acc.finish(ms, Rg, cv);
    const double rho = m.rho, T = m.temp, tre = m.two_rho_e;
    const double U[3] = {m.u, m.v, m.w};
    const double Pm[3][3] = {{m.pxx, m.pxy, m.pxz}, {m.pxy, m.pyy, m.pyz}, {m.pxz, m.pyz, m.pzz}};
    const double mq[3] = {m.qx, m.qy, m.qz};
    Equilibrium<double> E;
    const double omega = build_equilibrium<double>(m, dq[0], dq[1], dq[2], ph.nu, ph.alpha, dt, Rg, cv, lat, E);
    const double omega1 = 1.0 / (ph.alpha / (Rg * T * dt) + 0.5);
    const double r = omega1 / omega;
    const double wc = (2.0 - omega) / (2.0 * omega * rho);
    double ph3[3][3];
    for (int a = 0; a < 3; ++a) {
        const double P = U[a] * U[a] + Rg * T + dt * wc * dq[a];
        for (int e = -1; e <= 1; ++e) ph3[a][e + 1] = Equilibrium<double>::phi(e, U[a], P);
    }
    const double energy = tre / (2.0 * rho);
    const double tmp = (0.50 / cv) * ((tre / rho) - (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]));
    const double p = rho * Rg * tmp;
    const double h = energy + (p / rho);
    const double G = h + (p / rho);
    double qeq[3], B[3];
    for (int a = 0; a < 3; ++a) {
        qeq[a] = 2.0 * rho * U[a] * h;
        B[a] = mq[a] - 2.0 * U[0] * Pm[a][0] - 2.0 * U[1] * Pm[a][1] - 2.0 * U[2] * Pm[a][2] - U[a] * dt * dq[a];
    }

    // ---- outputs -> equilibria, omega ----
    double lw = 0.0;
    double lrf[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, lphz[3] = {0, 0, 0};
    double lgrho = 0.0, la1[3] = {0, 0, 0}, la2d[3] = {0, 0, 0}, la2o[3] = {0, 0, 0};
    // per direction, with compile-time lattice vectors (no int-to-double work)
#define MBG_REV(q)                                                                                   \
    {                                                                                                \
        constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);                                      \
        const double feq = E.rf[ex + 1][ey + 1] * E.phz[ez + 1];                                     \
        const double geq = E.template geq<q>(lat);                                                   \
        const long long si = P.src(q);                                                               \
        const double lfq = Lf[q * lstride], lgq = Lg[q * lstride];                                   \
        lw += lfq * (feq - P.f[si]) + lgq * (geq - P.g[si]);                                         \
        const double lfe = omega * lfq;                                                              \
        lrf[ex + 1][ey + 1] += lfe * E.phz[ez + 1];                                                  \
        lphz[ez + 1] += lfe * E.rf[ex + 1][ey + 1];                                                  \
        const double wl = lat.w[q] * (omega * lgq);                                                  \
        lgrho += wl;                                                                                 \
        if constexpr (ex == 1) la1[0] += wl; else if constexpr (ex == -1) la1[0] -= wl;              \
        if constexpr (ey == 1) la1[1] += wl; else if constexpr (ey == -1) la1[1] -= wl;              \
        if constexpr (ez == 1) la1[2] += wl; else if constexpr (ez == -1) la1[2] -= wl;              \
        if constexpr (ex != 0) wd1[0] += wl; else wd0[0] += wl;                                      \
        if constexpr (ey != 0) wd1[1] += wl; else wd0[1] += wl;                                      \
        if constexpr (ez != 0) wd1[2] += wl; else wd0[2] += wl;                                      \
        if constexpr (ex * ey == 1) la2o[0] += wl; else if constexpr (ex * ey == -1) la2o[0] -= wl;  \
        if constexpr (ex * ez == 1) la2o[1] += wl; else if constexpr (ex * ez == -1) la2o[1] -= wl;  \
        if constexpr (ey * ez == 1) la2o[2] += wl; else if constexpr (ey * ez == -1) la2o[2] -= wl;  \
    }
    double wd0[3] = {0, 0, 0}, wd1[3] = {0, 0, 0};
    MBG_UNROLL27(MBG_REV)
#undef MBG_REV
    for (int a = 0; a < 3; ++a) la2d[a] = 0.5 * (lat.cth[0] * wd0[a] + lat.cth[1] * wd1[a]);
    // ---- product-form f_eq ----
    double lrho = 0.0, lU[3] = {0, 0, 0}, lT = 0.0, ltre = 0.0, lwc = 0.0;
    double lph[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            lrho += lrf[a][c] * ph3[0][a] * ph3[1][c];
            lph[0][a] += lrf[a][c] * rho * ph3[1][c];
            lph[1][c] += lrf[a][c] * rho * ph3[0][a];
        }
    for (int c = 0; c < 3; ++c) lph[2][c] = lphz[c];
    for (int a = 0; a < 3; ++a) {
        // phi(+-1) = +-u/2 + P/2, phi(0) = 1 - P
        lU[a] += 0.5 * (lph[a][2] - lph[a][0]);
        const double lP = -lph[a][1] + 0.5 * (lph[a][0] + lph[a][2]);
        // P = u^2 + R T + dt omega_corr dq
        lU[a] += 2.0 * U[a] * lP;
        lT += Rg * lP;
        lwc += dt * dq[a] * lP;
        ldq[a] = dt * wc * lP;
    }
    // ---- Grad-expansion g_eq ----
    ltre += lgrho;
    const double k = lat.one_bystheta0, th = lat.theta0;
    double lqf[3], lrd[3], lro[3];
    for (int a = 0; a < 3; ++a) {
        lqf[a] = k * la1[a];
        lrd[a] = k * k * la2d[a];
        ltre += -th * k * k * la2d[a];
        lro[a] = k * k * la2o[a];
    }
    double lr = 0.0, lh = 0.0, lG = 0.0, lp = 0.0, lmq[3] = {0, 0, 0};
    double lPm[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < 3; ++a) {
        const double lqeq = r * lqf[a];
        lr += (qeq[a] - B[a]) * lqf[a];
        const double lB = (1.0 - r) * lqf[a];
        lmq[a] += lB;
        for (int c = 0; c < 3; ++c) {
            lU[c] += -2.0 * Pm[a][c] * lB;
            lPm[a][c] += -2.0 * U[c] * lB;
        }
        lU[a] += -dt * dq[a] * lB;
        ldq[a] += -U[a] * dt * lB;
        // q_eq = 2 rho u h
        lrho += 2.0 * U[a] * h * lqeq;
        lU[a] += 2.0 * rho * h * lqeq;
        lh += 2.0 * rho * U[a] * lqeq;
        // r_aa = 2 rho u^2 G + 2 p h
        lrho += 2.0 * U[a] * U[a] * G * lrd[a];
        lU[a] += 4.0 * rho * U[a] * G * lrd[a];
        lG += 2.0 * rho * U[a] * U[a] * lrd[a];
        lp += 2.0 * h * lrd[a];
        lh += 2.0 * p * lrd[a];
    }
    const int oa[3] = {0, 0, 1}, ob[3] = {1, 2, 2};   // xy, xz, yz
    for (int i = 0; i < 3; ++i) {
        const int a = oa[i], c = ob[i];
        lrho += 2.0 * U[a] * U[c] * G * lro[i];
        lU[a] += 2.0 * rho * U[c] * G * lro[i];
        lU[c] += 2.0 * rho * U[a] * G * lro[i];
        lG += 2.0 * rho * U[a] * U[c] * lro[i];
    }
    // G = h + p / rho;  h = energy + p / rho
    lh += lG;
    lp += lG / rho;
    lrho += -p / (rho * rho) * lG;
    const double lenergy = lh;
    lp += lh / rho;
    lrho += -p / (rho * rho) * lh;
    // p = rho R tmp;  energy = 2 rho E / (2 rho);  tmp = (0.5 / cv)(2 rho E / rho - u^2)
    lrho += Rg * tmp * lp;
    const double ltmp = rho * Rg * lp;
    ltre += lenergy / (2.0 * rho);
    lrho += -tre / (2.0 * rho * rho) * lenergy;
    ltre += (0.50 / cv) / rho * ltmp;
    lrho += -(0.50 / cv) * tre / (rho * rho) * ltmp;
    for (int a = 0; a < 3; ++a) lU[a] += -(0.50 / cv) * 2.0 * U[a] * ltmp;
    // ---- relaxation rates ----
    // omega_corr = (2 - omega) / (2 omega rho)
    lw += -lwc / (omega * omega * rho);
    lrho += -wc / rho * lwc;
    // r = omega1 / omega
    const double lw1 = lr / omega;
    lw += -lr * omega1 / (omega * omega);
    // omega = 1 / (nu / (R T dt) + 1/2): d omega / dT = omega^2 nu / (R dt T^2)
    lT += lw * omega * omega * (ph.nu / (Rg * dt)) / (T * T);
    lT += lw1 * omega1 * omega1 * (ph.alpha / (Rg * dt)) / (T * T);
    // ---- onto the moment sums ----
    for (int i = 0; i < 14; ++i) la[i] = 0.0;
    macro_reverse(acc, ph, lrho, lU, lT, ltre, la);
    la[4] += lPm[0][0];
    la[5] += lPm[1][1];
    la[6] += lPm[2][2];
    la[7] += lPm[0][1] + lPm[1][0];
    la[8] += lPm[0][2] + lPm[2][0];
    la[9] += lPm[1][2] + lPm[2][1];
    la[11] += lmq[0];
    la[12] += lmq[1];
    la[13] += lmq[2];
    omega_out = omega;
}

// ---- forward kernels -----------------------------------------------------
__global__ void k_adj_q(AdjBox b, Phys64 ph, const double* f, const double* g, double* Q)
{
    int x, y, z;
    long long c;
    if (!adj_cell(b, x, y, z, c)) return;
    const Macro<double> m = pulled_moments(b, x, y, z, f, g, nullptr, nullptr).finish(ph.mesh_speed, ph.Rg, ph.cv);
    Q[c] = m.qcx;
    Q[b.N + c] = m.qcy;
    Q[2 * b.N + c] = m.qcz;
}

// fields a reverse step reads from its forward step: the 14 moment sums of
// the pulled values and dQ (component-major [k][N])
enum { MOM_N = 17 };

__global__ void k_adj_step(AdjBox b, Phys64 ph, const double* f, const double* g, const double* Q, double* fo,
                           double* go, double* mom)
{
    int x, y, z;
    long long c;
    if (!adj_cell(b, x, y, z, c)) return;
    const MomentAcc<double> acc = pulled_moments(b, x, y, z, f, g, nullptr, nullptr);
    const Macro<double> m = acc.finish(ph.mesh_speed, ph.Rg, ph.cv);
    const double dqx = dq_axis(b, Q, x, y, z, 0, ph.idx[0]);
    const double dqy = dq_axis(b, Q, x, y, z, 1, ph.idx[1]);
    const double dqz = dq_axis(b, Q, x, y, z, 2, ph.idx[2]);
    if (mom) {
        const double v[MOM_N] = {acc.rho, acc.u, acc.v, acc.w, acc.pxx, acc.pyy, acc.pzz, acc.pxy, acc.pxz,
                                 acc.pyz, acc.tre, acc.qx, acc.qy, acc.qz, dqx, dqy, dqz};
        for (int k = 0; k < MOM_N; ++k) mom[k * b.N + c] = v[k];
    }
    Equilibrium<double> E;
    const double omega = build_equilibrium<double>(m, dqx, dqy, dqz, ph.nu, ph.alpha, ph.dt, ph.Rg, ph.cv, ph.lat, E);
#define MBG_AS(q)                                                                                       \
    {                                                                                                   \
        const long long s = nbr(b, x, y, z, -ev_x(q), -ev_y(q), -ev_z(q));                              \
        const double fq = f[q * b.N + s], gq = g[q * b.N + s];                                          \
        fo[q * b.N + c] = fq + omega * (E.template feq<q>() - fq);                                      \
        go[q * b.N + c] = gq + omega * (E.template geq<q>(ph.lat) - gq);                                \
    }
    MBG_UNROLL27(MBG_AS)
#undef MBG_AS
}

// one-direction dual number (value, derivative) for the derivative of the
// initial-condition equilibria with respect to the temperature
struct Dual1 {
    double v, d;
    __host__ __device__ Dual1(double a = 0.0, double b = 0.0) : v(a), d(b) {}
    __host__ __device__ Dual1& operator+=(Dual1 o)
    {
        v += o.v;
        d += o.d;
        return *this;
    }
    __host__ __device__ Dual1& operator*=(Dual1 o)
    {
        d = d * o.v + v * o.d;
        v *= o.v;
        return *this;
    }
};
__host__ __device__ inline Dual1 operator+(Dual1 a, Dual1 b) { return Dual1(a.v + b.v, a.d + b.d); }
__host__ __device__ inline Dual1 operator-(Dual1 a, Dual1 b) { return Dual1(a.v - b.v, a.d - b.d); }
__host__ __device__ inline Dual1 operator-(Dual1 a) { return Dual1(-a.v, -a.d); }
__host__ __device__ inline Dual1 operator*(Dual1 a, Dual1 b) { return Dual1(a.v * b.v, a.d * b.v + a.v * b.d); }
__host__ __device__ inline Dual1 operator/(Dual1 a, Dual1 b)
{
    return Dual1(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v));
}
__host__ __device__ inline Dual1 operator*(double a, Dual1 b) { return Dual1(a * b.v, a * b.d); }
__host__ __device__ inline Dual1 operator*(int a, Dual1 b) { return Dual1(a * b.v, a * b.d); }

__global__ void k_adj_ic(AdjBox b, Phys64 ph, double gamma, double rho0, double u0x, double u0y, double u0z,
                         const double* T0, double* f, double* g)
{
    int x, y, z;
    long long c;
    if (!adj_cell(b, x, y, z, c)) return;
    const double vel[3] = {u0x, u0y, u0z};
    const double T = T0[c];
    for (int q = 0; q < NQ; ++q) {
        f[q * b.N + c] = eq_f_plain<double>(q, rho0, vel, ph.Rg * T);
        g[q * b.N + c] = eq_g_plain<double>(q, rho0, vel, ph.Rg, T, gamma, ph.lat);
    }
}

// dL/dT0 = sum_q lambda_f d f_eq / dT + lambda_g d g_eq / dT
__global__ void k_adj_ic_grad(AdjBox b, Phys64 ph, double gamma, double rho0, double u0x, double u0y, double u0z,
                              const double* T0, const double* lf, const double* lg, double* dT)
{
    int x, y, z;
    long long c;
    if (!adj_cell(b, x, y, z, c)) return;
    const Dual1 vel[3] = {Dual1(u0x), Dual1(u0y), Dual1(u0z)};
    const Dual1 T(T0[c], 1.0);
    Lattice<Dual1> lat;
    for (int q = 0; q < NQ; ++q) lat.w[q] = Dual1(ph.lat.w[q]);
    lat.theta0 = Dual1(ph.lat.theta0);
    lat.one_bystheta0 = Dual1(ph.lat.one_bystheta0);
    lat.cth[0] = Dual1(ph.lat.cth[0]);
    lat.cth[1] = Dual1(ph.lat.cth[1]);
    double s = 0.0;
    for (int q = 0; q < NQ; ++q) {
        const Dual1 fe = eq_f_plain<Dual1>(q, Dual1(rho0), vel, Dual1(ph.Rg) * T);
        const Dual1 ge = eq_g_plain<Dual1>(q, Dual1(rho0), vel, Dual1(ph.Rg), T, Dual1(gamma), lat);
        s += lf[q * b.N + c] * fe.d + lg[q * b.N + c] * ge.d;
    }
    dT[c] = s;
}

// temperature of the stored state (no stream), and the adjoint of the
// state from an adjoint of that temperature field
__global__ void k_adj_temp(AdjBox b, Phys64 ph, const double* f, const double* g, double* T)
{
    int x, y, z;
    long long c;
    if (!adj_cell(b, x, y, z, c)) return;
    MomentAcc<double> acc;
#define MBG_AT(q) acc.template add<q>(f[q * b.N + c], g[q * b.N + c]);
    MBG_UNROLL27(MBG_AT)
#undef MBG_AT
    T[c] = acc.finish(ph.mesh_speed, ph.Rg, ph.cv).temp;
}

// adjoint of one population from the adjoints of the moment sums (the
// transpose of MomentAcc::add), compile-time lattice vector
template <int q>
__device__ __forceinline__ void moments_to_pop(const double la[14], double& lf, double& lg)
{
    constexpr int ex = ev_x(q), ey = ev_y(q), ez = ev_z(q);
    double f = la[0], g = la[10];
    if constexpr (ex == 1) { f += la[1]; g += la[11]; } else if constexpr (ex == -1) { f -= la[1]; g -= la[11]; }
    if constexpr (ey == 1) { f += la[2]; g += la[12]; } else if constexpr (ey == -1) { f -= la[2]; g -= la[12]; }
    if constexpr (ez == 1) { f += la[3]; g += la[13]; } else if constexpr (ez == -1) { f -= la[3]; g -= la[13]; }
    if constexpr (ex != 0) f += la[4];
    if constexpr (ey != 0) f += la[5];
    if constexpr (ez != 0) f += la[6];
    if constexpr (ex * ey == 1) f += la[7]; else if constexpr (ex * ey == -1) f -= la[7];
    if constexpr (ex * ez == 1) f += la[8]; else if constexpr (ex * ez == -1) f -= la[8];
    if constexpr (ey * ez == 1) f += la[9]; else if constexpr (ey * ez == -1) f -= la[9];
    lf = f;
    lg = g;
}

__global__ void k_adj_seed(AdjBox b, Phys64 ph, const double* f, const double* g, const double* dLdT, double* lf,
                           double* lg)
{
    int x, y, z;
    long long c;
    if (!adj_cell(b, x, y, z, c)) return;
    MomentAcc<double> acc;
#define MBG_AS2(q) acc.template add<q>(f[q * b.N + c], g[q * b.N + c]);
    MBG_UNROLL27(MBG_AS2)
#undef MBG_AS2
    double la[14] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const double lU[3] = {0, 0, 0};
    macro_reverse(acc, ph, 0.0, lU, dLdT[c], 0.0, la);
#define MBG_SEEDQ(q) moments_to_pop<q>(la, lf[q * b.N + c], lg[q * b.N + c]);
    MBG_UNROLL27(MBG_SEEDQ)
#undef MBG_SEEDQ
}

// ---- reverse kernels -----------------------------------------------------
__global__ void __launch_bounds__(128) k_adj_a1(AdjBox b, Phys64 ph, const double* f, const double* g,
                                                const double* mom, const double* lf, const double* lg, double* ws)
{
    int x, y, z;
    long long c;
    if (!adj_cell(b, x, y, z, c)) return;
    MomentAcc<double> acc;
    acc.rho = mom[c];
    acc.u = mom[b.N + c];
    acc.v = mom[2 * b.N + c];
    acc.w = mom[3 * b.N + c];
    acc.pxx = mom[4 * b.N + c];
    acc.pyy = mom[5 * b.N + c];
    acc.pzz = mom[6 * b.N + c];
    acc.pxy = mom[7 * b.N + c];
    acc.pxz = mom[8 * b.N + c];
    acc.pyz = mom[9 * b.N + c];
    acc.tre = mom[10 * b.N + c];
    acc.qx = mom[11 * b.N + c];
    acc.qy = mom[12 * b.N + c];
    acc.qz = mom[13 * b.N + c];
    const double dq[3] = {mom[14 * b.N + c], mom[15 * b.N + c], mom[16 * b.N + c]};
    double la[14], ldq[3], omega;
    collide_reverse(acc, dq, ph, CellPull{&b, x, y, z, f, g}, lf + c, lg + c, b.N, la, ldq, omega);
    for (int i = 0; i < 14; ++i) ws[(WS_LA + i) * b.N + c] = la[i];
    for (int d = 0; d < 3; ++d) ws[(WS_LDQ + d) * b.N + c] = ldq[d];
    ws[WS_OMEGA * b.N + c] = omega;
    ws[WS_RHO * b.N + c] = acc.rho;
    ws[(WS_J + 0) * b.N + c] = acc.u;
    ws[(WS_J + 1) * b.N + c] = acc.v;
    ws[(WS_J + 2) * b.N + c] = acc.w;
    ws[WS_TRE * b.N + c] = acc.tre;
}

// transpose of the gradient stencil: adjoint of Q_corr_d at cell y
__device__ __forceinline__ double lq_axis(const AdjBox& b, const double* ws, int x, int y, int z, int d, double idx)
{
    const int p[3] = {x, y, z};
    const int cd = p[d], n = b.n[d];
    const double* L = ws + (WS_LDQ + d) * b.N;
    double s = 0.0;
    int q[3] = {x, y, z};
    if (cd - 1 >= 0) {   // from x = y - e: Q(y) is its plus neighbour
        q[d] = cd - 1;
        const double lx = L[lin(b, q[0], q[1], q[2])];
        s += (cd - 2 >= 0 ? 0.5 : 1.0) * idx * lx;
    }
    if (cd + 1 < n) {    // from x = y + e: Q(y) is its minus neighbour
        q[d] = cd + 1;
        const double lx = L[lin(b, q[0], q[1], q[2])];
        s += (cd + 2 < n ? -0.5 : -1.0) * idx * lx;
    }
    // from x = y itself, one-sided at a face
    const bool p_out = cd + 1 >= n, m_out = cd - 1 < 0;
    const double ly = L[lin(b, x, y, z)];
    if (p_out && !m_out) s += idx * ly;
    else if (m_out && !p_out) s += -idx * ly;
    return s;
}

__global__ void k_adj_a2(AdjBox b, Phys64 ph, const double* ws, const double* lf, const double* lg, double* lfo,
                         double* lgo)
{
    int x, y, z;
    long long c;
    if (!adj_cell(b, x, y, z, c)) return;
    MomentAcc<double> acc;
    acc.rho = ws[WS_RHO * b.N + c];
    acc.u = ws[(WS_J + 0) * b.N + c];
    acc.v = ws[(WS_J + 1) * b.N + c];
    acc.w = ws[(WS_J + 2) * b.N + c];
    acc.tre = ws[WS_TRE * b.N + c];
    double la[14];
    for (int i = 0; i < 14; ++i) la[i] = ws[(WS_LA + i) * b.N + c];
    // Q_corr_a = rho u_a ((1 - 3 R T) - u_a^2)
    const double rho = acc.rho, s = ph.mesh_speed / rho;
    const double U[3] = {acc.u * s, acc.v * s, acc.w * s};
    const double T = (0.50 / ph.cv) * ((acc.tre / rho) - (U[0] * U[0] + U[1] * U[1] + U[2] * U[2]));
    double lrho = 0.0, lU[3], lT = 0.0;
    for (int a = 0; a < 3; ++a) {
        const double lQ = lq_axis(b, ws, x, y, z, a, ph.idx[a]);
        const double base = (1.0 - 3.0 * ph.Rg * T) - U[a] * U[a];
        lrho += U[a] * base * lQ;
        lU[a] = rho * (base - 2.0 * U[a] * U[a]) * lQ;
        lT += rho * U[a] * (-3.0 * ph.Rg) * lQ;
    }
    macro_reverse(acc, ph, lrho, lU, lT, 0.0, la);
    const double om = 1.0 - ws[WS_OMEGA * b.N + c];
    // p(x, q) = s(x - e_q, q): push each adjoint back to its source
#define MBG_PUSH(q)                                                                \
    {                                                                              \
        double mf, mg;                                                             \
        moments_to_pop<q>(la, mf, mg);                                             \
        const long long t = nbr(b, x, y, z, -ev_x(q), -ev_y(q), -ev_z(q));         \
        lfo[q * b.N + t] = om * lf[q * b.N + c] + mf;                              \
        lgo[q * b.N + t] = om * lg[q * b.N + c] + mg;                              \
    }
    MBG_UNROLL27(MBG_PUSH)
#undef MBG_PUSH
}

}  // namespace mbg

using namespace mbg;

struct mbg_adj {
    mbg_params p{};
    Phys64 ph{};
    AdjBox b{};
    cudaStream_t s = nullptr;
    bool own_stream = false;
    std::string err;
    std::vector<void*> allocs;
    double *f[2] = {nullptr, nullptr}, *g[2] = {nullptr, nullptr};
    double* Q = nullptr;
    double* ws = nullptr;
    double *lf[2] = {nullptr, nullptr}, *lg[2] = {nullptr, nullptr};
    double *T0 = nullptr, *Tx = nullptr;
    std::vector<double*> ckpt;    // checkpoints, [f | g] each
    std::vector<double*> seg;     // states of the segment being reversed
    std::vector<double*> segm;    // their forward moments and dQ (MOM_N fields)
    double* tmpo = nullptr;       // throw-away output of the last state's forward step
    int cur = 0;
    int nsteps = -1, K = 0;
    long long launches = 0;
    double rho0 = 1.0, u0[3] = {0, 0, 0};
};

static mbg_status afail(mbg_adj* a, mbg_status st, const std::string& m)
{
    if (a) a->err = m;
    return st;
}

#define ACUDA(call)                                                                                           \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess) return afail(a, MBG_ECUDA, std::string(#call ": ") + cudaGetErrorString(e_));   \
    } while (0)

static mbg_status aalloc(mbg_adj* a, double** p, size_t count)
{
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(double));
    if (e != cudaSuccess)
        return afail(a, e == cudaErrorMemoryAllocation ? MBG_ENOMEM : MBG_ECUDA,
                     std::string("cudaMalloc (adjoint): ") + cudaGetErrorString(e));
    a->allocs.push_back(*p);
    return MBG_OK;
}

static unsigned nblk(const mbg_adj* a) { return (unsigned)((a->b.N + 127) / 128); }

static void fwd_step(mbg_adj* a, const double* f, const double* g, double* fo, double* go, double* mom = nullptr)
{
    k_adj_q<<<nblk(a), 128, 0, a->s>>>(a->b, a->ph, f, g, a->Q);
    k_adj_step<<<nblk(a), 128, 0, a->s>>>(a->b, a->ph, f, g, a->Q, fo, go, mom);
    a->launches += 2;
}

extern "C" {

mbg_status mbg_adj_create(const mbg_params* p, double rho0, const double u0[3], void* stream, mbg_adj** out)
{
    if (!p || !out) {
        mbg_set_global_error("mbg_adj_create: null argument");
        return MBG_EINVAL;
    }
    *out = nullptr;
    for (int d = 0; d < 3; ++d) {
        if (!p->is_periodic[d] || p->n_cell[d] < 3 || !(p->prob_hi[d] > p->prob_lo[d])) {
            mbg_set_global_error("mbg_adj_create: the adjoint runs on one fully periodic box of >= 3 cells per axis");
            return MBG_EINVAL;
        }
    }
    if (p->precision != MBG_FP64) {
        mbg_set_global_error("mbg_adj_create: the adjoint is FP64 (precision MBG_FP64)");
        return MBG_EINVAL;
    }
    mbg_adj* a = new mbg_adj();
    a->p = *p;
    a->rho0 = rho0;
    for (int d = 0; d < 3; ++d) a->u0[d] = u0 ? u0[d] : 0.0;
    for (int d = 0; d < 3; ++d) a->b.n[d] = p->n_cell[d];
    a->b.N = (long long)p->n_cell[0] * p->n_cell[1] * p->n_cell[2];
    Phys64& ph = a->ph;
    ph.mesh_speed = p->dx_outer / p->dt_outer;
    ph.Rg = 28.96 / p->m_bar;
    ph.cv = ph.Rg / (p->adiabatic_exponent - 1.0);
    ph.nu = p->nu;
    ph.alpha = p->alpha;
    ph.dt = p->dt_outer;
    for (int d = 0; d < 3; ++d) ph.idx[d] = 1.0 / ((p->prob_hi[d] - p->prob_lo[d]) / p->n_cell[d]);
    ph.small_num = 2.220446049250313e-16 * 1e10;
    ph.lat = make_lattice<double>();
    if (stream) {
        a->s = (cudaStream_t)stream;
    } else if (cudaStreamCreateWithFlags(&a->s, cudaStreamNonBlocking) != cudaSuccess) {
        delete a;
        mbg_set_global_error("mbg_adj_create: cudaStreamCreate failed");
        return MBG_ECUDA;
    } else {
        a->own_stream = true;
    }
    const size_t N = (size_t)a->b.N;
    mbg_status st = MBG_OK;
    for (int i = 0; i < 2 && st == MBG_OK; ++i) {
        if ((st = aalloc(a, &a->f[i], N * NQ)) != MBG_OK) break;
        if ((st = aalloc(a, &a->g[i], N * NQ)) != MBG_OK) break;
        if ((st = aalloc(a, &a->lf[i], N * NQ)) != MBG_OK) break;
        st = aalloc(a, &a->lg[i], N * NQ);
    }
    if (st == MBG_OK) st = aalloc(a, &a->Q, N * 3);
    if (st == MBG_OK) st = aalloc(a, &a->ws, N * WS_N);
    if (st == MBG_OK) st = aalloc(a, &a->T0, N);
    if (st == MBG_OK) st = aalloc(a, &a->Tx, N);
    if (st != MBG_OK) {
        mbg_set_global_error(a->err);
        mbg_adj_destroy(a);
        return st;
    }
    *out = a;
    return MBG_OK;
}

mbg_status mbg_adj_forward(mbg_adj* a, const double* T0, int nsteps, int K, double* T_final)
{
    if (!a || !T0 || !T_final || nsteps < 0 || K < 1) return MBG_EINVAL;
    const size_t N = (size_t)a->b.N;
    const size_t sb = N * NQ * sizeof(double);
    const int nck = (nsteps + K - 1) / K;
    // checkpoint storage (kept across calls with the same count)
    while ((int)a->ckpt.size() < nck) {
        double* c = nullptr;
        mbg_status st = aalloc(a, &c, 2 * N * NQ);
        if (st != MBG_OK) return st;
        a->ckpt.push_back(c);
    }
    ACUDA(cudaMemcpyAsync(a->T0, T0, N * sizeof(double), cudaMemcpyHostToDevice, a->s));
    k_adj_ic<<<nblk(a), 128, 0, a->s>>>(a->b, a->ph, a->p.adiabatic_exponent, a->rho0, a->u0[0], a->u0[1],
                                         a->u0[2], a->T0, a->f[0], a->g[0]);
    a->launches++;
    a->cur = 0;
    for (int n = 0; n < nsteps; ++n) {
        if (n % K == 0) {
            double* c = a->ckpt[n / K];
            ACUDA(cudaMemcpyAsync(c, a->f[a->cur], sb, cudaMemcpyDeviceToDevice, a->s));
            ACUDA(cudaMemcpyAsync(c + N * NQ, a->g[a->cur], sb, cudaMemcpyDeviceToDevice, a->s));
        }
        fwd_step(a, a->f[a->cur], a->g[a->cur], a->f[1 - a->cur], a->g[1 - a->cur]);
        a->cur = 1 - a->cur;
    }
    k_adj_temp<<<nblk(a), 128, 0, a->s>>>(a->b, a->ph, a->f[a->cur], a->g[a->cur], a->Tx);
    a->launches++;
    ACUDA(cudaMemcpyAsync(T_final, a->Tx, N * sizeof(double), cudaMemcpyDeviceToHost, a->s));
    ACUDA(cudaStreamSynchronize(a->s));
    a->nsteps = nsteps;
    a->K = K;
    return MBG_OK;
}

mbg_status mbg_adj_backward(mbg_adj* a, const double* dL_dTfinal, double* dL_dT0)
{
    if (!a || !dL_dTfinal || !dL_dT0) return MBG_EINVAL;
    if (a->nsteps < 0) return afail(a, MBG_ESTATE, "mbg_adj_backward: no forward run to differentiate");
    const size_t N = (size_t)a->b.N;
    const int K = a->K, nsteps = a->nsteps;
    // segment states
    while ((int)a->seg.size() < K) {
        double *c = nullptr, *cm = nullptr;
        mbg_status st = aalloc(a, &c, 2 * N * NQ);
        if (st == MBG_OK) st = aalloc(a, &cm, (size_t)MOM_N * N);
        if (st != MBG_OK) return st;
        a->seg.push_back(c);
        a->segm.push_back(cm);
    }
    if (!a->tmpo) {
        mbg_status st = aalloc(a, &a->tmpo, 2 * N * NQ);
        if (st != MBG_OK) return st;
    }
    // adjoint of the final state from dL/dT_final
    ACUDA(cudaMemcpyAsync(a->Tx, dL_dTfinal, N * sizeof(double), cudaMemcpyHostToDevice, a->s));
    k_adj_seed<<<nblk(a), 128, 0, a->s>>>(a->b, a->ph, a->f[a->cur], a->g[a->cur], a->Tx, a->lf[0], a->lg[0]);
    a->launches++;
    int lc = 0;
    const int nck = (nsteps + K - 1) / K;
    for (int ci = nck - 1; ci >= 0; --ci) {
        const int n0 = ci * K, n1 = std::min(nsteps, n0 + K);
        // recompute the segment's states from its checkpoint
        ACUDA(cudaMemcpyAsync(a->seg[0], a->ckpt[ci], 2 * N * NQ * sizeof(double), cudaMemcpyDeviceToDevice, a->s));
        // (keeping each step's moments and dQ, which the reverse steps read;
        // the last state's step runs into a throw-away output for them)
        for (int i = 1; i < n1 - n0; ++i)
            fwd_step(a, a->seg[i - 1], a->seg[i - 1] + N * NQ, a->seg[i], a->seg[i] + N * NQ, a->segm[i - 1]);
        {
            const double* fl = a->seg[n1 - n0 - 1];
            fwd_step(a, fl, fl + N * NQ, a->tmpo, a->tmpo + N * NQ, a->segm[n1 - n0 - 1]);
        }
        for (int n = n1 - 1; n >= n0; --n) {
            const double* f = a->seg[n - n0];
            const double* g = f + N * NQ;
            k_adj_a1<<<nblk(a), 128, 0, a->s>>>(a->b, a->ph, f, g, a->segm[n - n0], a->lf[lc], a->lg[lc], a->ws);
            k_adj_a2<<<nblk(a), 128, 0, a->s>>>(a->b, a->ph, a->ws, a->lf[lc], a->lg[lc], a->lf[1 - lc],
                                                 a->lg[1 - lc]);
            a->launches += 2;
            lc = 1 - lc;
        }
    }
    k_adj_ic_grad<<<nblk(a), 128, 0, a->s>>>(a->b, a->ph, a->p.adiabatic_exponent, a->rho0, a->u0[0], a->u0[1],
                                              a->u0[2], a->T0, a->lf[lc], a->lg[lc], a->Tx);
    a->launches++;
    ACUDA(cudaMemcpyAsync(dL_dT0, a->Tx, N * sizeof(double), cudaMemcpyDeviceToHost, a->s));
    ACUDA(cudaStreamSynchronize(a->s));
    return MBG_OK;
}

long long mbg_adj_launch_count(const mbg_adj* a) { return a ? a->launches : 0; }

void* mbg_adj_stream(const mbg_adj* a) { return a ? (void*)a->s : nullptr; }

const char* mbg_adj_last_error(const mbg_adj* a) { return a ? a->err.c_str() : ""; }

void mbg_adj_destroy(mbg_adj* a)
{
    if (!a) return;
    if (a->s) cudaStreamSynchronize(a->s);
    for (void* p : a->allocs) cudaFree(p);
    if (a->own_stream && a->s) cudaStreamDestroy(a->s);
    delete a;
}

}  // extern "C"
