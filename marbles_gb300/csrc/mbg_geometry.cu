// mbg_geometry.cu -- is_fluid flags of a level's boxes from the embedded
// geometry, on the GPU (mbg_geometry_flags in include/marbles_gb300.h).
//
// One thread per cell of every box grown by 3 (the layout mbg_define_level
// takes).  Component 0 (is_fluid) is the cell's classification, taken at
// the periodic image when that image lies in a box of the level (what
// FillBoundary copies there); component 1 (eb_boundary: a covered cell with
// a fluid face neighbour) is computed for cells within 2 of the box, and at
// the image for cells whose image lies in a box -- initialize_is_fluid
// (Source/LBM.cpp:1213-1262) with its two FillBoundary calls.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/marbles_gb300.h"
#include "mbg_geometry.cuh"

void mbg_set_global_error(const std::string& msg);

namespace mbg {

struct FlagLevel {
    int dhi[3];
    int per[3];
    int G[3], nb[3];
    const int* omap;
    const int* lohi;          // [box][6]
    const long long* foff;    // first grown cell of each box
    int nbox;
    double plo[3], dx[3];
};

__device__ __forceinline__ bool fl_wrap(const FlagLevel& L, int p[3])
{
    for (int d = 0; d < 3; ++d) {
        if (p[d] < 0 || p[d] > L.dhi[d]) {
            if (!L.per[d]) return false;
            const int len = L.dhi[d] + 1;
            int r = p[d] % len;
            if (r < 0) r += len;
            p[d] = r;
        }
    }
    return true;
}

__device__ __forceinline__ int fl_owner(const FlagLevel& L, const int p[3])
{
    return L.omap[((long long)(p[2] / L.G[2]) * L.nb[1] + p[1] / L.G[1]) * L.nb[0] + p[0] / L.G[0]];
}

__device__ __forceinline__ int fl_comp0(const FlagLevel& L, const GeomDesc& g, int i, int j, int k)
{
    int p[3] = {i, j, k};
    if (fl_wrap(L, p) && fl_owner(L, p) >= 0) return geom_covered(g, L.plo, L.dx, p[0], p[1], p[2]) ? 0 : 1;
    return geom_covered(g, L.plo, L.dx, i, j, k) ? 0 : 1;
}

__device__ __forceinline__ int fl_comp1(const FlagLevel& L, const GeomDesc& g, int i, int j, int k)
{
    bool all_covered = true;
    all_covered &= (fl_comp0(L, g, i - 1, j, k) == 0) && (fl_comp0(L, g, i + 1, j, k) == 0);
    all_covered &= (fl_comp0(L, g, i, j - 1, k) == 0) && (fl_comp0(L, g, i, j + 1, k) == 0);
    all_covered &= (fl_comp0(L, g, i, j, k - 1) == 0) && (fl_comp0(L, g, i, j, k + 1) == 0);
    return (all_covered || fl_comp0(L, g, i, j, k) == 1) ? 0 : 1;
}

__global__ void k_geometry_flags(FlagLevel L, GeomDesc g, long long total, uint8_t* out)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    // the box holding grown cell t (boxes in order, foff ascending)
    int lo = 0, hi = L.nbox - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (L.foff[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const int* b = L.lohi + 6 * lo;
    const int gx = b[3] - b[0] + 7, gy = b[4] - b[1] + 7;
    const long long c = t - L.foff[lo];
    const int x = (int)(c % gx), y = (int)((c / gx) % gy), z = (int)(c / ((long long)gx * gy));
    const int i = b[0] - 3 + x, j = b[1] - 3 + y, k = b[2] - 3 + z;
    if (g.type == GEOM_ALL_REGULAR) {
        out[t] = 1;
        return;
    }
    const int c0 = fl_comp0(L, g, i, j, k);
    int c1 = 0;
    int p[3] = {i, j, k};
    const bool owned = fl_wrap(L, p) && fl_owner(L, p) >= 0;
    const bool layer3 = i == b[0] - 3 || i == b[3] + 3 || j == b[1] - 3 || j == b[4] + 3 || k == b[2] - 3 ||
                        k == b[5] + 3;
    if (owned) c1 = fl_comp1(L, g, p[0], p[1], p[2]);
    else if (!layer3) c1 = fl_comp1(L, g, i, j, k);
    out[t] = (uint8_t)(c0 | (c1 << 1));
}

GeomDesc geom_from(const mbg_geometry& in)
{
    GeomDesc g;
    g.type = in.type;
    g.fluid_inside = in.has_fluid_inside;
    for (int d = 0; d < 3; ++d) {
        g.center[d] = in.center[d];
        g.lo[d] = in.lo[d];
        g.hi[d] = in.hi[d];
        g.point[d] = in.point[d];
        g.normal[d] = in.normal[d];
        g.rot_center[d] = in.rotation_center[d];
    }
    g.radius = in.radius;
    g.height = in.height;
    g.direction = in.direction;
    // Source/Geometry.cpp:150, 179: degrees to radians
    const double angle = (in.rotation_deg / 180.) * M_PI;
    g.rot_cos = std::cos(angle);
    g.rot_sin = std::sin(angle);
    g.rot_axis = in.rotation_axis;
    g.ntri = std::min(std::max(in.ntri, 0), GEOM_MAX_TRI);
    for (int t = 0; t < GEOM_MAX_TRI; ++t)
        for (int v = 0; v < 3; ++v)
            for (int d = 0; d < 2; ++d) g.tri[t][v][d] = in.tri[t][v][d];
    return g;
}

}  // namespace mbg

using namespace mbg;

namespace {
mbg_status geo_fail(const std::string& m, mbg_status st = MBG_EINVAL)
{
    mbg_set_global_error("mbg_geometry_flags: " + m);
    return st;
}
}  // namespace

extern "C" mbg_status mbg_geometry_flags(const mbg_geometry* geom, const mbg_params* p, int lev, int nbox,
                                         const int* lohi, uint8_t* flags, void* cuda_stream)
{
    if (!geom || !p || !lohi || !flags || nbox < 1 || lev < 0 || lev > 20) return geo_fail("bad argument");
    if (geom->type < GEOM_ALL_REGULAR || geom->type > GEOM_EXTRUDED_TRIANGLES) return geo_fail("unknown geometry");
    if (geom->direction < 0 || geom->direction > 2 || geom->rotation_axis < 0 || geom->rotation_axis > 2)
        return geo_fail("direction and rotation_axis must be 0, 1 or 2");
    FlagLevel L{};
    for (int d = 0; d < 3; ++d) {
        if (p->n_cell[d] < 1 || !(p->prob_hi[d] > p->prob_lo[d])) return geo_fail("bad domain");
        L.dhi[d] = (p->n_cell[d] << lev) - 1;
        L.per[d] = p->is_periodic[d] != 0;
        L.plo[d] = p->prob_lo[d];
        L.dx[d] = (p->prob_hi[d] - p->prob_lo[d]) / (p->n_cell[d] << lev);
    }
    // owner map on bins of the gcd of all box corners
    std::vector<long long> foff(nbox);
    long long total = 0;
    for (int d = 0; d < 3; ++d) {
        int g = L.dhi[d] + 1;
        for (int n = 0; n < nbox; ++n) {
            const int* b = lohi + 6 * n;
            if (b[d] < 0 || b[d + 3] < b[d] || b[d + 3] > L.dhi[d]) return geo_fail("box outside the domain");
            g = std::gcd(g, b[d]);
            g = std::gcd(g, b[d + 3] + 1);
        }
        L.G[d] = g;
        L.nb[d] = (L.dhi[d] + 1) / g;
    }
    std::vector<int> omap((size_t)L.nb[0] * L.nb[1] * L.nb[2], -1);
    for (int n = 0; n < nbox; ++n) {
        const int* b = lohi + 6 * n;
        foff[n] = total;
        total += (long long)(b[3] - b[0] + 7) * (b[4] - b[1] + 7) * (b[5] - b[2] + 7);
        for (int k = b[2] / L.G[2]; k <= b[5] / L.G[2]; ++k)
            for (int j = b[1] / L.G[1]; j <= b[4] / L.G[1]; ++j)
                for (int i = b[0] / L.G[0]; i <= b[3] / L.G[0]; ++i) {
                    int& o = omap[((size_t)k * L.nb[1] + j) * L.nb[0] + i];
                    if (o >= 0) return geo_fail("boxes overlap");
                    o = n;
                }
    }
    cudaStream_t s = (cudaStream_t)cuda_stream;
    int *d_omap = nullptr, *d_lohi = nullptr;
    long long* d_foff = nullptr;
    uint8_t* d_out = nullptr;
    auto release = [&] {
        cudaFree(d_omap);
        cudaFree(d_lohi);
        cudaFree(d_foff);
        cudaFree(d_out);
    };
    cudaError_t e = cudaMalloc(&d_omap, omap.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&d_lohi, (size_t)nbox * 6 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&d_foff, (size_t)nbox * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&d_out, (size_t)total);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_omap, omap.data(), omap.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_lohi, lohi, (size_t)nbox * 6 * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_foff, foff.data(), (size_t)nbox * sizeof(long long), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        release();
        return geo_fail(std::string("CUDA: ") + cudaGetErrorString(e),
                        e == cudaErrorMemoryAllocation ? MBG_ENOMEM : MBG_ECUDA);
    }
    L.omap = d_omap;
    L.lohi = d_lohi;
    L.foff = d_foff;
    L.nbox = nbox;
    const GeomDesc g = geom_from(*geom);
    k_geometry_flags<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(L, g, total, d_out);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(flags, d_out, (size_t)total, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    release();
    if (e != cudaSuccess) return geo_fail(std::string("CUDA: ") + cudaGetErrorString(e), MBG_ECUDA);
    return MBG_OK;
}
