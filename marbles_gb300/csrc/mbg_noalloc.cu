// mbg_noalloc.cu -- FP64 step of one periodic box without any device
// allocation (mbg_step_box_noalloc in include/marbles_gb300.h).
//
// Who needs it: a host code that has handed the whole GPU to its own memory
// arena (AMReX-based solvers such as MARBLES reserve most of device memory up
// front) cannot let a library call cudaMalloc behind its back -- the call can
// fail with out-of-memory in the middle of a run -- and cudaMalloc / cudaFree
// can synchronise the device, which a caller that queues its whole time loop
// asynchronously on its own stream cannot accept.  Such a caller passes its
// own input and output populations; the only other memory the step needs,
// the macro-field scratch between its two passes, is the fixed array below,
// part of the library's device image.
//
// The array holds MBG_NOALLOC_MAX_CELLS cells x 18 FP64 fields (4.5 MiB) on
// every GPU that loads the library, until the process exits.  All calls share
// it: two calls whose kernels overlap on the GPU (different streams, or
// different host threads on one device) race on it and must be serialised by
// the caller.  Each call rewrites every scratch entry it later reads, so
// nothing needs clearing between calls.
//
// Every call looks up the array's device address on the current device
// (cudaGetSymbolAddress, a host-side lookup with no device work) instead of
// caching it, so that a context torn down and re-created by cudaDeviceReset
// never leaves a stale address behind.  The first call on a device may load
// the library's device code; make that first call outside any stream capture.
#include <cstdio>
#include <string>

#include "../../include/marbles_gb300.h"
#include "mbg_kernels.h"

namespace mbg {

constexpr long long NOALLOC_MAX_CELLS = MBG_NOALLOC_MAX_CELLS;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_MAX_CELLS * MD_NCOMP];

struct BoxDims {
    int n[3];
    long long N;
};

__device__ __forceinline__ long long nx_lin(const BoxDims& b, int x, int y, int z)
{
    return ((long long)z * b.n[1] + y) * b.n[0] + x;
}

// pulled value of direction q at (x, y, z): the periodic source of the box
template <int q>
__device__ __forceinline__ double na_pull(const BoxDims& b, int x, int y, int z, const double* v)
{
    int sx = x - ev_x(q), sy = y - ev_y(q), sz = z - ev_z(q);
    sx += (sx < 0) ? b.n[0] : (sx >= b.n[0] ? -b.n[0] : 0);
    sy += (sy < 0) ? b.n[1] : (sy >= b.n[1] ? -b.n[1] : 0);
    sz += (sz < 0) ? b.n[2] : (sz >= b.n[2] ? -b.n[2] : 0);
    return v[q * b.N + nx_lin(b, sx, sy, sz)];
}

__device__ __forceinline__ bool na_cell(const BoxDims& b, int& x, int& y, int& z, long long& c)
{
    c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= b.N) return false;
    x = (int)(c % b.n[0]);
    const long long r = c / b.n[0];
    y = (int)(r % b.n[1]);
    z = (int)(r / b.n[1]);
    return true;
}

__global__ void __launch_bounds__(TILE_CELLS) k_na_moments(BoxDims b, Phys64 ph, const double* f, const double* g,
                                                           double* md)
{
    int x, y, z;
    long long c;
    if (!na_cell(b, x, y, z, c)) return;
    MomentAcc<double> acc;
#define MBG_NAM(q) acc.template add<q>(na_pull<q>(b, x, y, z, f), na_pull<q>(b, x, y, z, g));
    MBG_UNROLL27(MBG_NAM)
#undef MBG_NAM
    const Macro<double> m = acc.finish(ph.mesh_speed, ph.Rg, ph.cv);
    const long long N = b.N;
    md[MD_RHO * N + c] = m.rho;
    md[MD_U * N + c] = m.u;
    md[MD_V * N + c] = m.v;
    md[MD_W * N + c] = m.w;
    md[MD_TRE * N + c] = m.two_rho_e;
    md[MD_PXX * N + c] = m.pxx;
    md[MD_PYY * N + c] = m.pyy;
    md[MD_PZZ * N + c] = m.pzz;
    md[MD_PXY * N + c] = m.pxy;
    md[MD_PXZ * N + c] = m.pxz;
    md[MD_PYZ * N + c] = m.pyz;
    md[MD_QX * N + c] = m.qx;
    md[MD_QY * N + c] = m.qy;
    md[MD_QZ * N + c] = m.qz;
    md[MD_T * N + c] = m.temp;
    md[MD_QCX * N + c] = m.qcx;
    md[MD_QCY * N + c] = m.qcy;
    md[MD_QCZ * N + c] = m.qcz;
}

// gradient() of Source/Utilities.H:279-312 along d; the domain is the box,
// so neighbours across a face are absent (one-sided difference there)
__device__ __forceinline__ double na_grad(const BoxDims& b, int x, int y, int z, int d, double idx,
                                          const double* md)
{
    const int p[3] = {x, y, z};
    const bool p_out = p[d] + 1 >= b.n[d];
    const bool m_out = p[d] - 1 < 0;
    int pp[3] = {x, y, z}, pm[3] = {x, y, z};
    pp[d] += 1;
    pm[d] -= 1;
    const double* qc = md + (MD_QCX + d) * b.N;
    double vp = 0.0, vc = 0.0, vm = 0.0;
    if (p_out && m_out) {
        vp = 0.0; vc = 0.0; vm = 0.0;
    } else if (p_out) {
        vp = 0.0;
        vc = qc[nx_lin(b, x, y, z)];
        vm = -qc[nx_lin(b, pm[0], pm[1], pm[2])];
    } else if (m_out) {
        vp = qc[nx_lin(b, pp[0], pp[1], pp[2])];
        vc = -qc[nx_lin(b, x, y, z)];
        vm = 0.0;
    } else {
        vp = 0.5 * qc[nx_lin(b, pp[0], pp[1], pp[2])];
        vc = 0.0;
        vm = -0.5 * qc[nx_lin(b, pm[0], pm[1], pm[2])];
    }
    return (vp + vc + vm) * idx;
}

__global__ void __launch_bounds__(TILE_CELLS) k_na_collide(BoxDims b, Phys64 ph, const double* f, const double* g,
                                                           double* fo, double* go, const double* md)
{
    int x, y, z;
    long long c;
    if (!na_cell(b, x, y, z, c)) return;
    const long long N = b.N;
    Macro<double> m;
    m.rho = md[MD_RHO * N + c];
    m.u = md[MD_U * N + c];
    m.v = md[MD_V * N + c];
    m.w = md[MD_W * N + c];
    m.two_rho_e = md[MD_TRE * N + c];
    m.pxx = md[MD_PXX * N + c];
    m.pyy = md[MD_PYY * N + c];
    m.pzz = md[MD_PZZ * N + c];
    m.pxy = md[MD_PXY * N + c];
    m.pxz = md[MD_PXZ * N + c];
    m.pyz = md[MD_PYZ * N + c];
    m.qx = md[MD_QX * N + c];
    m.qy = md[MD_QY * N + c];
    m.qz = md[MD_QZ * N + c];
    m.temp = md[MD_T * N + c];
    const double dqx = na_grad(b, x, y, z, 0, ph.idx[0], md);
    const double dqy = na_grad(b, x, y, z, 1, ph.idx[1], md);
    const double dqz = na_grad(b, x, y, z, 2, ph.idx[2], md);
    Equilibrium<double> E;
    const double omega =
        build_equilibrium<double>(m, dqx, dqy, dqz, ph.nu, ph.alpha, ph.dt, ph.Rg, ph.cv, ph.lat, E);
#define MBG_NAF(q)                                                   \
    {                                                                \
        const double fq = na_pull<q>(b, x, y, z, f);                 \
        fo[q * N + c] = fq + omega * (E.template feq<q>() - fq);     \
    }
#define MBG_NAG(q)                                                   \
    {                                                                \
        const double gq = na_pull<q>(b, x, y, z, g);                 \
        go[q * N + c] = gq + omega * (E.template geq<q>(ph.lat) - gq); \
    }
    MBG_UNROLL27(MBG_NAF)
    MBG_UNROLL27(MBG_NAG)
#undef MBG_NAF
#undef MBG_NAG
}

}  // namespace mbg

using namespace mbg;

// error text of the last failed call (shared with mbg_last_error(NULL))
void mbg_set_global_error(const std::string& msg);

namespace {
mbg_status na_fail(const std::string& m)
{
    mbg_set_global_error("mbg_step_box_noalloc: " + m);
    return MBG_EINVAL;
}
}  // namespace

extern "C" mbg_status mbg_step_box_noalloc(const mbg_params* p, const double* f_in, const double* g_in,
                                           double* f_out, double* g_out, void* cuda_stream)
{
    if (!p || !f_in || !g_in || !f_out || !g_out) return na_fail("null argument");
    if (p->precision != MBG_FP64) return na_fail("only the FP64 form is available without allocation");
    for (int d = 0; d < 3; ++d) {
        if (!p->is_periodic[d]) return na_fail("the box must be periodic in every direction");
        if (p->n_cell[d] < 1) return na_fail("n_cell must be positive");
        if (!(p->prob_hi[d] > p->prob_lo[d])) return na_fail("prob_hi must exceed prob_lo");
    }
    // each factor is checked before the product is formed, so the product
    // cannot overflow (every n_cell[d] <= the maximum, itself < 2^21)
    for (int d = 0; d < 3; ++d)
        if (p->n_cell[d] > NOALLOC_MAX_CELLS)
            return na_fail("n_cell[" + std::to_string(d) + "] = " + std::to_string(p->n_cell[d]) +
                           " exceeds the maximum of " + std::to_string(NOALLOC_MAX_CELLS) + " cells");
    const long long N = (long long)p->n_cell[0] * p->n_cell[1] * p->n_cell[2];
    if (N > NOALLOC_MAX_CELLS)
        return na_fail("box of " + std::to_string(N) + " cells exceeds the maximum of " +
                       std::to_string(NOALLOC_MAX_CELLS) + " cells");
    if (!(p->nu > 0) || !(p->alpha > 0) || !(p->m_bar > 0) || !(p->adiabatic_exponent > 1.0) || !(p->dt_outer > 0))
        return na_fail("nu, alpha, dt_outer, m_bar must be positive and adiabatic_exponent > 1");
    if (f_out == f_in || f_out == g_in || g_out == f_in || g_out == g_in || f_out == g_out)
        return na_fail("outputs must not alias inputs or each other");
    // the scratch array's address on the current device, looked up on every
    // call (a cached address would go stale after cudaDeviceReset)
    void* scratch = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
    if (e != cudaSuccess || !scratch) {
        mbg_set_global_error(std::string("mbg_step_box_noalloc: cudaGetSymbolAddress: ") +
                             cudaGetErrorString(e));
        return MBG_ECUDA;
    }
    BoxDims b;
    for (int d = 0; d < 3; ++d) b.n[d] = p->n_cell[d];
    b.N = N;
    Phys64 ph;
    ph.mesh_speed = p->dx_outer / p->dt_outer;
    ph.Rg = 28.96 / p->m_bar;
    ph.cv = ph.Rg / (p->adiabatic_exponent - 1.0);
    ph.nu = p->nu;
    ph.alpha = p->alpha;
    ph.dt = 1.0;
    for (int d = 0; d < 3; ++d) ph.idx[d] = 1.0 / ((p->prob_hi[d] - p->prob_lo[d]) / p->n_cell[d]);
    ph.small_num = 0.0;
    ph.lat = make_lattice<double>();
    cudaStream_t s = (cudaStream_t)cuda_stream;
    const unsigned grid = (unsigned)((N + TILE_CELLS - 1) / TILE_CELLS);
    double* md = (double*)scratch;
    k_na_moments<<<grid, TILE_CELLS, 0, s>>>(b, ph, f_in, g_in, md);
    k_na_collide<<<grid, TILE_CELLS, 0, s>>>(b, ph, f_in, g_in, f_out, g_out, md);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        mbg_set_global_error(std::string("mbg_step_box_noalloc: launch: ") + cudaGetErrorString(e));
        return MBG_ECUDA;
    }
    return MBG_OK;
}
