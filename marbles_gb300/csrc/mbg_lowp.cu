// mbg_lowp.cu -- host side of the FP32-arithmetic / 16-bit-storage form of the
// level step: storage codec, padded layout, tiles, constant blocks and the
// order of the kernels (mbg_lowp_kern.cuh) in one level advance.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <unordered_map>

#include "mbg_lowp_types.cuh"

namespace mbg {

// launch through the instantiation of the level's storage format
#define LOWP16(bf, fn, ...) ((bf) ? Lowp16<true>::fn(__VA_ARGS__) : Lowp16<false>::fn(__VA_ARGS__))

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct LowpDev {
    CodecTab ct;
    Lattice<float> lat;
    LowpK hk[2];                 // host copies, indexed by the source parity
    bool uploaded = false;
    bool with_override = false;
    LowpK* dk = nullptr;         // device copies [2]
    DevBox* box16 = nullptr;     // the level's boxes in the padded layout
    // step variants (FUSED_ZC): fused tile lists of variants 1 and 2
    FusedTile* ftiles[2] = {nullptr, nullptr};
    int nftiles[2] = {0, 0};
    int variant = 0;
    double variant_ms[4] = {0, 0, 0, 0};   // tuner's timings (0: not timed)
    float* qs = nullptr;         // Q_corr of the two-pass step, [3][N]
    QPad qpad;                   // Q_corr of the pad (qpad_plan)
    // variant 0: the tile classes of step_tiles; each device list holds room
    // for every tile of its kind, so that lowp_retile only copies
    Tile* ptiles = nullptr;
    int nptiles = 0;
    Tile* potiles = nullptr;
    int nootiles = 0;
    Tile* petiles = nullptr;
    int neetiles = 0;
    Tile* ctiles = nullptr;
    int nctiles = 0;
    unsigned* nmask = nullptr;   // neighbour masks (neighbour_masks), or null
    std::vector<DevBox> box16h;  // host copy of box16
    HaloCopy* hcopy = nullptr;   // pad fill: per pad cell, the directions and the cell copied (halo_plan)
    long long ngather = 0;
    HaloCell* general = nullptr; // pad cells that need the general kernel (physical BCs)
    long long ngeneral = 0;
    NbrSlot* gslots = nullptr;   // ghost stream: ghost-shell slot tables (ghost_slots16), the ghost
    int* gslot_off = nullptr;    // cells that copy through them, the other ghost cells (gathered)
    int gslot_lg[3] = {0, 0, 0};
    GhostCell* ghost_fast = nullptr;
    long long nghost_fast = 0;
    GhostCell* ghost_rest = nullptr;
    long long nghost_rest = 0;
    long long* sdst = nullptr;   // ghost stream by gather (ghost_plan over the other ghost cells)
    long long* ssrc = nullptr;
    long long nsgather = 0;
    int* scell = nullptr;        // ghost stream entries for the general kernel
    int* sq = nullptr;
    long long nsgen = 0;
    long long nhalo = 0;         // pad cells of the level (the pad fill runs when there are any)
    u16* fo = nullptr;           // coalescence override buffers
    u16* go = nullptr;
    ExplodePlan xp{};            // explosion into this (fine) level's ghost fabs
};

static LowpDev* dev_of(LowpLevel& L) { return (LowpDev*)L.impl; }

static LevelView<u16> view16(const LevelPlan& plan, const LowpLevel& L)
{
    const LevelView<double>& v = plan.view64;
    LevelView<u16> w;
    w.box = ((const LowpDev*)L.impl)->box16;
    w.nbox = v.nbox;
    for (int d = 0; d < 3; ++d) {
        w.dlo[d] = v.dlo[d];
        w.dhi[d] = v.dhi[d];
        w.per[d] = v.per[d];
        w.G[d] = v.G[d];
        w.nb[d] = v.nb[d];
    }
    w.omap = v.omap;
    w.N = L.N;
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

Phys32 phys32(const mbg_params& p, double dt, const double idx[3])
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

// codec of the storage: the equilibria at the reference state and the scales
CodecTab make_codec(const mbg_params& p)
{
    CodecTab ct;
    const Lattice<double> lat64 = make_lattice<double>();
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
        ct.frest[q] = (float)fr;
        ct.grest[q] = (float)gr;
        ct.fsc[q] = (float)fs;
        ct.gsc[q] = (float)gs;
        ct.fisc[q] = (float)(1.0 / fs);
        ct.gisc[q] = (float)(1.0 / gs);
    }
    return ct;
}

// padded boxes: strides, storage offsets; returns the padded cell count
long long pad_boxes(std::vector<DevBox>& box)
{
    long long np = 0;
    for (DevBox& B : box) {
        const long long px = B.n[0] + 2, py = B.n[1] + 2, pz = B.n[2] + 2;
        B.sy = (int)px;
        B.sz = (int)(px * py);
        // valid cell (0,0,0) at an even index, so that the cell pairs (x even)
        // of a box with an even x extent are 4-byte aligned
        if ((np + B.sz + B.sy + 1) & 1) ++np;
        B.voff = np + B.sz + B.sy + 1;
        np += px * py * pz;
    }
    // an even component stride keeps that alignment in every component
    return np + (np & 1);
}

static void upload_tiles(LowpDev* D, const StepTiles& t, cudaStream_t s)
{
    D->nptiles = (int)t.pair.size();
    D->nootiles = (int)t.pair_ovr.size();
    D->neetiles = (int)t.pair_eb.size();
    D->nctiles = (int)t.cell.size();
    if (!t.pair.empty()) cudaMemcpyAsync(D->ptiles, t.pair.data(), t.pair.size() * sizeof(Tile), cudaMemcpyHostToDevice, s);
    if (!t.pair_ovr.empty())
        cudaMemcpyAsync(D->potiles, t.pair_ovr.data(), t.pair_ovr.size() * sizeof(Tile), cudaMemcpyHostToDevice, s);
    if (!t.pair_eb.empty())
        cudaMemcpyAsync(D->petiles, t.pair_eb.data(), t.pair_eb.size() * sizeof(Tile), cudaMemcpyHostToDevice, s);
    if (!t.cell.empty()) cudaMemcpyAsync(D->ctiles, t.cell.data(), t.cell.size() * sizeof(Tile), cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);   // the host vectors end with the caller
}

StepTiles step_tiles(const std::vector<DevBox>& box, const std::vector<uint8_t>* flags)
{
    StepTiles t;
    for (size_t n = 0; n < box.size(); ++n) {
        const DevBox& B = box[n];
        const long long vol = (long long)B.n[0] * B.n[1] * B.n[2];
        const bool pairs = B.n[0] % 2 == 0 && B.voff % 2 == 0;
        if (!pairs) {
            for (long long s = 0; s < vol; s += TILE_CELLS) t.cell.push_back(Tile{(int)n, (int)s});
            continue;
        }
        for (long long s = 0; s < vol; s += PAIR_CELLS) {
            bool ovr = false;
            for (long long c = s; c < std::min(vol, s + PAIR_CELLS) && flags && !ovr; ++c) {
                const int x = (int)(c % B.n[0]), y = (int)((c / B.n[0]) % B.n[1]), z = (int)(c / B.n[0] / B.n[1]);
                const long long fi = B.foff + ((long long)(z + 3) * (B.n[1] + 6) + (y + 3)) * (B.n[0] + 6) + (x + 3);
                ovr = (*flags)[fi] & FL_OVR;
            }
            if (B.vfluid) {
                (ovr ? t.pair_ovr : t.pair).push_back(Tile{(int)n, (int)s});
            } else if (!ovr) {
                t.pair_eb.push_back(Tile{(int)n, (int)s});
            } else {
                // overwritten cells next to solids: the per-cell kernels
                for (long long c = s; c < std::min(vol, s + PAIR_CELLS); c += TILE_CELLS)
                    t.cell.push_back(Tile{(int)n, (int)c});
            }
        }
    }
    return t;
}

// per valid cell of the boxes holding solid cells: bit q where the fluid
// cell's source x - e_q is solid, bit NMASK_FLUID where the cell is fluid
static std::vector<unsigned> neighbour_masks(const std::vector<DevBox>& box, const std::vector<uint8_t>& fl,
                                             long long N)
{
    std::vector<unsigned> m((size_t)N, 0u);
    for (const DevBox& B : box) {
        if (B.vfluid) continue;
        auto f = [&](int x, int y, int z) {
            return fl[B.foff + ((long long)(z + 3) * (B.n[1] + 6) + (y + 3)) * (B.n[0] + 6) + (x + 3)] & FL_FLUID;
        };
        for (int z = 0; z < B.n[2]; ++z)
            for (int y = 0; y < B.n[1]; ++y)
                for (int x = 0; x < B.n[0]; ++x) {
                    if (!f(x, y, z)) continue;
                    unsigned w = 1u << NMASK_FLUID;
                    for (int q = 0; q < NQ; ++q)
                        if (!f(x - ev_x(q), y - ev_y(q), z - ev_z(q))) w |= 1u << q;
                    m[B.voff + (long long)z * B.sz + (long long)y * B.sy + x] = w;
                }
    }
    return m;
}

// the step's tile lists again after the level's flags gained or lost cells
// overwritten by coalescence (a finer level defined or dropped); the device
// lists were sized at set-up for every class
void lowp_retile(LowpLevel& L, const std::vector<uint8_t>& flags, cudaStream_t s)
{
    LowpDev* D = dev_of(L);
    if (!D) return;
    upload_tiles(D, step_tiles(D->box16h, &flags), s);
}

// every pad cell of every box, faces first, then edges, then corners, so that
// neighbouring threads share the set of directions they fill
std::vector<HaloCell> halo_cells(const std::vector<DevBox>& box)
{
    std::vector<HaloCell> out;
    for (int nz = 1; nz <= 3; ++nz)
        for (size_t b = 0; b < box.size(); ++b)
            for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        if ((dx != 0) + (dy != 0) + (dz != 0) != nz) continue;
                        const int d[3] = {dx, dy, dz};
                        int lo[3], hi[3];
                        for (int a = 0; a < 3; ++a) {
                            lo[a] = d[a] < 0 ? -1 : d[a] > 0 ? box[b].n[a] : 0;
                            hi[a] = d[a] < 0 ? -1 : d[a] > 0 ? box[b].n[a] : box[b].n[a] - 1;
                        }
                        for (int z = lo[2]; z <= hi[2]; ++z)
                            for (int y = lo[1]; y <= hi[1]; ++y)
                                for (int x = lo[0]; x <= hi[0]; ++x)
                                    out.push_back(HaloCell{(int)b, (short)x, (short)y, (short)z, 0});
                    }
    return out;
}


// fused-step tiles: tile width the smallest of 8, 16, 32 that covers the box
// (32 for wider boxes), runs of zc planes
std::vector<FusedTile> fused_tiles(const std::vector<DevBox>& box, int zc)
{
    std::vector<FusedTile> tiles;
    for (size_t n = 0; n < box.size(); ++n) {
        const int lgw = box[n].n[0] <= 8 ? 3 : box[n].n[0] <= 16 ? 4 : 5;
        const int tw = 1 << lgw, th = FT_THREADS / tw;
        for (int z0 = 0; z0 < box[n].n[2]; z0 += zc)
            for (int y0 = 0; y0 < box[n].n[1]; y0 += th)
                for (int x0 = 0; x0 < box[n].n[0]; x0 += tw)
                    tiles.push_back(FusedTile{(int)n, (short)x0, (short)y0, (short)z0,
                                              (short)std::min(box[n].n[2], z0 + zc), (short)lgw, 0});
    }
    return tiles;
}

// Q_corr pad plan: the face cells of every box's pad inside the domain box
// that hold fluid (edges and corners are on no gradient stencil, cells
// outside the domain box are read by no one-sided gradient, solid ones by
// no gradient at all; their zeros from set-up stay), each a copy from the
// owning box's valid cell or, on the coarse-fine shell, a ghost entry.
static void qpad_plan(const std::vector<DevBox>& box, const std::vector<HaloCell>& halo, long long N,
                      const LevelHost& h, std::vector<long long>& dst, std::vector<long long>& src,
                      std::vector<HaloCell>& ghost)
{
    auto fab = [](const DevBox& B, int x, int y, int z) {
        return ((long long)(z + 3) * (B.n[1] + 6) + (y + 3)) * (B.n[0] + 6) + (x + 3);
    };
    const std::vector<uint8_t>& fl = *h.flags;
    for (const HaloCell& c : halo) {
        const DevBox& B = box[c.box];
        const int out0 = c.x < 0 || c.x >= B.n[0], out1 = c.y < 0 || c.y >= B.n[1], out2 = c.z < 0 || c.z >= B.n[2];
        if (out0 + out1 + out2 != 1) continue;
        const int d = out0 ? 0 : out1 ? 1 : 2;
        const int gp[3] = {B.lo[0] + c.x, B.lo[1] + c.y, B.lo[2] + c.z};
        bool inside = true;
        for (int a = 0; a < 3; ++a) inside = inside && gp[a] >= h.dlo[a] && gp[a] <= h.dhi[a];
        if (!inside || !(fl[B.foff + fab(B, c.x, c.y, c.z)] & FL_FLUID)) continue;
        const int bi = (gp[0] - h.dlo[0]) / h.G[0], bj = (gp[1] - h.dlo[1]) / h.G[1], bk = (gp[2] - h.dlo[2]) / h.G[2];
        const int o = (*h.omap)[((size_t)bk * h.nb[1] + bj) * h.nb[0] + bi];
        if (o >= 0) {
            const DevBox& O = box[o];
            dst.push_back((long long)d * N + B.voff + (long long)c.z * B.sz + (long long)c.y * B.sy + c.x);
            src.push_back((long long)d * N + O.voff + (long long)(gp[2] - O.lo[2]) * O.sz +
                          (long long)(gp[1] - O.lo[1]) * O.sy + (gp[0] - O.lo[0]));
        } else if (B.goff >= 0) {
            ghost.push_back(c);
        }
    }
}

// Pad fill plan: per pad cell, the directions q whose pull from the pad cell
// lands on a fluid cell of the box (the pad cell fluid too: a solid source
// bounces back in the step), and the storage index within one component the
// values are copied from -- a valid cell of the owning box (periodic images
// resolved), or the box's own ghost fab as -index - 1.  Every direction of a
// pad cell copies from the same cell.  Pad cells outside a non-periodic side
// (physical BC) go to a separate list filled by the general kernel.
static void halo_plan(const std::vector<DevBox>& box, const std::vector<HaloCell>& halo, const LevelHost& h,
                      std::vector<HaloCopy>& copies, std::vector<HaloCell>& general)
{
    auto fab = [](const DevBox& B, int x, int y, int z) {
        return ((long long)(z + 3) * (B.n[1] + 6) + (y + 3)) * (B.n[0] + 6) + (x + 3);
    };
    const std::vector<uint8_t>& fl = *h.flags;
    for (const HaloCell& c : halo) {
        const DevBox& B = box[c.box];
        if (!(fl[B.foff + fab(B, c.x, c.y, c.z)] & FL_FLUID)) continue;   // bounce-back in the step
        unsigned qmask = 0u;
        for (int q = 0; q < NQ; ++q) {
            const int tx = c.x + ev_x(q), ty = c.y + ev_y(q), tz = c.z + ev_z(q);
            if (tx < 0 || ty < 0 || tz < 0 || tx >= B.n[0] || ty >= B.n[1] || tz >= B.n[2]) continue;
            if (fl[B.foff + fab(B, tx, ty, tz)] & FL_FLUID) qmask |= 1u << q;   // a collided target
        }
        if (!qmask) continue;
        int gp[3] = {B.lo[0] + c.x, B.lo[1] + c.y, B.lo[2] + c.z};
        bool out = false;
        for (int d = 0; d < 3; ++d) {
            if (gp[d] < h.dlo[d] || gp[d] > h.dhi[d]) {
                if (!h.per[d]) { out = true; break; }
                const int len = h.dhi[d] - h.dlo[d] + 1;
                gp[d] = h.dlo[d] + (((gp[d] - h.dlo[d]) % len) + len) % len;
            }
        }
        if (out) {
            general.push_back(c);
            continue;
        }
        const int bi = (gp[0] - h.dlo[0]) / h.G[0], bj = (gp[1] - h.dlo[1]) / h.G[1], bk = (gp[2] - h.dlo[2]) / h.G[2];
        const int o = (*h.omap)[((size_t)bk * h.nb[1] + bj) * h.nb[0] + bi];
        HaloCopy hc;
        hc.dst = B.voff + (long long)c.z * B.sz + (long long)c.y * B.sy + c.x;
        hc.qmask = qmask;
        hc.pad = 0;
        if (o >= 0) {
            const DevBox& O = box[o];
            hc.src = O.voff + (long long)(gp[2] - O.lo[2]) * O.sz + (long long)(gp[1] - O.lo[1]) * O.sy +
                     (gp[0] - O.lo[0]);
        } else if (B.goff >= 0) {
            hc.src = -(B.goff + fab(B, c.x, c.y, c.z)) - 1;
        } else {
            general.push_back(c);
            continue;
        }
        copies.push_back(hc);
    }
}

// Ghost-stream plan: for every uncovered ghost cell and direction, the
// streamed value as a copy -- from a valid cell of the owning box (src >= 0,
// q N + index), from the box's own ghost fab (src = -(q NG + index) - 2) --
// or the -1 sentinel (src = -1).  Bounce-back from a solid source (a value
// of the opposite direction, re-encoded) and physical BCs go to the general
// list as (ghost-cell index, direction).
// Ghost-shell slot tables on the padded layout (chunks 3 cells wide at the
// box faces, grain 2^lg inside): each chunk of the box grown by 3 maps to
// one box's valid cells at a fixed offset or to the box's own ghost fab;
// ok[n] when every chunk of box n does.  The ghost stream of an all-fluid
// box with a table is then a copy through it (k_ghost_stream16s).
static void ghost_slots16(const std::vector<DevBox>& box, const LevelHost& h, const int lg[3],
                          std::vector<NbrSlot>& out, std::vector<int>& off, std::vector<char>& ok)
{
    const int w = 3;
    const int nbox = (int)box.size();
    out.clear();
    off.assign(nbox, -1);
    ok.assign(nbox, 0);
    auto owner = [&](int p[3]) -> int {
        for (int d = 0; d < 3; ++d) {
            if (p[d] < h.dlo[d] || p[d] > h.dhi[d]) {
                if (!h.per[d]) return -2;
                const int len = h.dhi[d] - h.dlo[d] + 1;
                p[d] = h.dlo[d] + (((p[d] - h.dlo[d]) % len) + len) % len;
            }
        }
        const int bi = (p[0] - h.dlo[0]) / h.G[0], bj = (p[1] - h.dlo[1]) / h.G[1], bk = (p[2] - h.dlo[2]) / h.G[2];
        return (*h.omap)[((size_t)bk * h.nb[1] + bj) * h.nb[0] + bi];
    };
    for (int n = 0; n < nbox; ++n) {
        const DevBox& B = box[n];
        if (!B.all_fluid || B.goff < 0) continue;
        int tc[3];
        for (int d = 0; d < 3; ++d) tc[d] = ((B.n[d] + (1 << lg[d]) - 1) >> lg[d]) + 2;
        const long long T = (long long)tc[0] * tc[1] * tc[2];
        if (T > SLOT_TABLE_MAX) continue;
        const size_t t0 = out.size();
        out.resize(t0 + (size_t)T, NbrSlot{0, 0, 0, -1, 0});
        bool all = true;
        for (int cz = 0; cz < tc[2] && all; ++cz)
            for (int cy = 0; cy < tc[1] && all; ++cy)
                for (int cx = 0; cx < tc[0] && all; ++cx) {
                    const int c3[3] = {cx, cy, cz};
                    NbrSlot& S = out[t0 + cx + (size_t)tc[0] * (cy + (size_t)tc[1] * cz)];
                    int rlo[3], rhi[3];
                    bool inside = true;
                    for (int d = 0; d < 3; ++d) {
                        if (c3[d] == 0) { rlo[d] = -w; rhi[d] = -1; }
                        else if (c3[d] == tc[d] - 1) { rlo[d] = B.n[d]; rhi[d] = B.n[d] + w - 1; }
                        else { rlo[d] = (c3[d] - 1) << lg[d]; rhi[d] = std::min(c3[d] << lg[d], B.n[d]) - 1; }
                        inside = inside && c3[d] > 0 && c3[d] < tc[d] - 1;
                    }
                    if (inside) {
                        S.base = B.voff;
                        S.sy = B.sy;
                        S.sz = B.sz;
                        S.ghost = 0;
                        continue;
                    }
                    int own = -3, dl0[3] = {0, 0, 0};
                    for (int z = rlo[2]; z <= rhi[2] && all; ++z)
                        for (int y = rlo[1]; y <= rhi[1] && all; ++y)
                            for (int x = rlo[0]; x <= rhi[0] && all; ++x) {
                                int p[3] = {B.lo[0] + x, B.lo[1] + y, B.lo[2] + z};
                                const int o = owner(p);
                                if (o == -2) { all = false; break; }
                                int dl[3] = {0, 0, 0};
                                if (o >= 0) {
                                    dl[0] = p[0] - box[o].lo[0] - x;
                                    dl[1] = p[1] - box[o].lo[1] - y;
                                    dl[2] = p[2] - box[o].lo[2] - z;
                                }
                                if (own == -3) {
                                    own = o;
                                    for (int d = 0; d < 3; ++d) dl0[d] = dl[d];
                                } else if (o != own || dl[0] != dl0[0] || dl[1] != dl0[1] || dl[2] != dl0[2]) {
                                    all = false;
                                }
                            }
                    if (!all) break;
                    if (own >= 0) {
                        const DevBox& O = box[own];
                        S.base = O.voff + (long long)dl0[2] * O.sz + (long long)dl0[1] * O.sy + dl0[0];
                        S.sy = O.sy;
                        S.sz = O.sz;
                        S.ghost = 0;
                    } else {
                        const int gx = B.n[0] + 6, gy = B.n[1] + 6;
                        S.base = B.goff + 3LL * gy * gx + 3LL * gx + 3;
                        S.sy = gx;
                        S.sz = gx * gy;
                        S.ghost = 1;
                    }
                }
        if (!all) {
            out.resize(t0);
            continue;
        }
        off[n] = (int)t0;
        ok[n] = 1;
    }
}

static void ghost_plan(const std::vector<DevBox>& box, const std::vector<GhostCell>& gl, long long N, long long NG,
                       const LevelHost& h, std::vector<long long>& dst, std::vector<long long>& src,
                       std::vector<int>& gen_cell, std::vector<int>& gen_q)
{
    auto fab = [](const DevBox& B, int x, int y, int z) {
        return ((long long)(z + 3) * (B.n[1] + 6) + (y + 3)) * (B.n[0] + 6) + (x + 3);
    };
    const std::vector<uint8_t>& fl = *h.flags;
    for (size_t e = 0; e < gl.size(); ++e) {
        const GhostCell& c = gl[e];
        const DevBox& B = box[c.box];
        const long long gi = B.goff + fab(B, c.x, c.y, c.z);
        const uint8_t tf = fl[B.foff + fab(B, c.x, c.y, c.z)];
        for (int q = 0; q < NQ; ++q) {
            const long long d = (long long)q * NG + gi;
            const int sx = c.x - ev_x(q), sy = c.y - ev_y(q), sz = c.z - ev_z(q);
            if (!(tf & FL_FLUID) || sx < -3 || sy < -3 || sz < -3 || sx > B.n[0] + 2 || sy > B.n[1] + 2 ||
                sz > B.n[2] + 2) {
                dst.push_back(d);
                src.push_back(-1);
                continue;
            }
            if (!(fl[B.foff + fab(B, sx, sy, sz)] & FL_FLUID)) {
                gen_cell.push_back((int)e);
                gen_q.push_back(q);
                continue;
            }
            int gp[3] = {B.lo[0] + sx, B.lo[1] + sy, B.lo[2] + sz};
            bool out = false;
            for (int a = 0; a < 3; ++a) {
                if (gp[a] < h.dlo[a] || gp[a] > h.dhi[a]) {
                    if (!h.per[a]) { out = true; break; }
                    const int len = h.dhi[a] - h.dlo[a] + 1;
                    gp[a] = h.dlo[a] + (((gp[a] - h.dlo[a]) % len) + len) % len;
                }
            }
            if (out) {
                gen_cell.push_back((int)e);
                gen_q.push_back(q);
                continue;
            }
            long long sidx = -1;
            if (sx >= 0 && sy >= 0 && sz >= 0 && sx < B.n[0] && sy < B.n[1] && sz < B.n[2]) {
                sidx = (long long)q * N + B.voff + (long long)sz * B.sz + (long long)sy * B.sy + sx;
            } else {
                const int bi = (gp[0] - h.dlo[0]) / h.G[0], bj = (gp[1] - h.dlo[1]) / h.G[1],
                          bk = (gp[2] - h.dlo[2]) / h.G[2];
                const int o = (*h.omap)[((size_t)bk * h.nb[1] + bj) * h.nb[0] + bi];
                if (o >= 0) {
                    const DevBox& O = box[o];
                    sidx = (long long)q * N + O.voff + (long long)(gp[2] - O.lo[2]) * O.sz +
                           (long long)(gp[1] - O.lo[1]) * O.sy + (gp[0] - O.lo[0]);
                } else if (B.goff >= 0) {
                    sidx = -((long long)q * NG + B.goff + fab(B, sx, sy, sz)) - 2;
                }
            }
            dst.push_back(d);
            src.push_back(sidx);
        }
    }
}

// explosion plan: the distinct coarse cells under the uncovered ghost cells,
// numbered in order of first use so that neighbouring ghost cells read
// neighbouring slots
void explode_plan(const std::vector<DevBox>& box, const std::vector<GhostCell>& ghosts, const LevelHost& h,
                  std::vector<XSlot>& xc, std::vector<int>& slot)
{
    auto floor2 = [](int v) { return v >= 0 ? v / 2 : -((1 - v) / 2); };
    std::unordered_map<long long, int> id;
    slot.reserve(ghosts.size());
    for (const GhostCell& g : ghosts) {
        const DevBox& B = box[g.box];
        int fp[3] = {B.lo[0] + g.x, B.lo[1] + g.y, B.lo[2] + g.z};
        // the device's wrap_pos: periodic sides wrap, up to the first side
        // that is outside and not periodic
        for (int d = 0; d < 3; ++d) {
            if (fp[d] >= h.dlo[d] && fp[d] <= h.dhi[d]) continue;
            if (!h.per[d]) break;
            const int len = h.dhi[d] - h.dlo[d] + 1;
            fp[d] = h.dlo[d] + (((fp[d] - h.dlo[d]) % len) + len) % len;
        }
        const XSlot c{floor2(fp[0]), floor2(fp[1]), floor2(fp[2]), 0};
        const long long key = ((long long)(c.z + 32768) * 65536 + (c.y + 32768)) * 65536 + (c.x + 32768);
        auto it = id.find(key);
        if (it == id.end()) {
            it = id.emplace(key, (int)xc.size()).first;
            xc.push_back(c);
        }
        slot.push_back(it->second);
    }
}

// order a gather plan by destination: component-major destinations make
// consecutive entries write consecutive cells of one component (the plans are
// built cell by cell, which spreads a warp's 2-byte stores over 27 components)
static void sort_plan(std::vector<long long>& dst, std::vector<long long>& src)
{
    std::vector<std::pair<long long, long long>> e(dst.size());
    for (size_t i = 0; i < dst.size(); ++i) e[i] = {dst[i], src[i]};
    std::sort(e.begin(), e.end());
    for (size_t i = 0; i < e.size(); ++i) {
        dst[i] = e[i].first;
        src[i] = e[i].second;
    }
}

mbg_status lowp_define(const mbg_params& p, const LevelPlan& plan, const std::vector<DevBox>& hbox, long long N,
                       long long NG, double dt, const double idx[3], const LevelHost& host, LowpLevel& L,
                       std::string& err)
{
    L.precision = p.precision;
    L.NV = N;
    L.NG = NG;
    L.ph = phys32(p, dt, idx);
    auto* D = new LowpDev();
    L.impl = D;
    D->ct = make_codec(p);
    D->lat = make_lattice<float>();
    std::vector<DevBox> box = hbox;
    for (size_t n = 0; n < box.size(); ++n) box[n].hoff = hbox[n].voff;
    L.N = pad_boxes(box);
    if (L.N >= (1LL << 31)) {
        err = "16-bit form: a level holds more than 2^31 padded cells";
        return MBG_EINVAL;
    }
    const std::vector<HaloCell> halo = halo_cells(box);
    std::vector<HaloCopy> hcopy;
    std::vector<HaloCell> general;
    halo_plan(box, halo, host, hcopy, general);
    std::vector<long long> sdst, ssrc;
    std::vector<int> scell, sq;
    std::vector<NbrSlot> gsl;
    std::vector<int> gsl_off;
    std::vector<GhostCell> gfast, grest;
    std::vector<char> gok(box.size(), 0);
    if (host.ghosts && NG > 0) {
        ghost_slots16(box, host, plan.slot_lg, gsl, gsl_off, gok);
        for (const GhostCell& gc : *host.ghosts) (gok[gc.box] ? gfast : grest).push_back(gc);
        ghost_plan(box, grest, L.N, NG, host, sdst, ssrc, scell, sq);
    }
    sort_plan(sdst, ssrc);
    D->nhalo = (long long)halo.size();
    std::vector<long long> qdst, qsrc;
    std::vector<HaloCell> qghost;
    qpad_plan(box, halo, L.N, host, qdst, qsrc, qghost);
    // the ghost stream of boxes with a ghost-shell table writes the Q_corr
    // of their coarse-fine pad face cells itself
    qghost.erase(std::remove_if(qghost.begin(), qghost.end(), [&](const HaloCell& c) { return gok[c.box] != 0; }),
                 qghost.end());
    mbg_status st;
    if ((st = lalloc(L, (void**)&D->box16, box.size() * sizeof(DevBox), err)) != MBG_OK) return st;
    for (int v = 0; v < 2; ++v) {
        const std::vector<FusedTile> tiles = fused_tiles(box, FUSED_ZC[v]);
        D->nftiles[v] = (int)tiles.size();
        if ((st = lalloc(L, (void**)&D->ftiles[v], tiles.size() * sizeof(FusedTile), err)) != MBG_OK) return st;
        cudaMemcpy(D->ftiles[v], tiles.data(), tiles.size() * sizeof(FusedTile), cudaMemcpyHostToDevice);
    }
    {
        const StepTiles t = step_tiles(box, host.flags);
        const size_t cap = t.pair.size() + t.pair_ovr.size() + t.pair_eb.size();   // pair tiles of any class
        size_t ccap = 0;                                                         // every cell per-cell
        for (const DevBox& B : box) ccap += ((size_t)B.n[0] * B.n[1] * B.n[2] + TILE_CELLS - 1) / TILE_CELLS;
        if ((st = lalloc(L, (void**)&D->ptiles, cap * sizeof(Tile), err)) != MBG_OK) return st;
        if ((st = lalloc(L, (void**)&D->potiles, cap * sizeof(Tile), err)) != MBG_OK) return st;
        if ((st = lalloc(L, (void**)&D->petiles, cap * sizeof(Tile), err)) != MBG_OK) return st;
        if ((st = lalloc(L, (void**)&D->ctiles, ccap * sizeof(Tile), err)) != MBG_OK) return st;
        upload_tiles(D, t, 0);
        D->box16h = box;
        bool any_eb = false;
        for (const DevBox& B : box) any_eb = any_eb || !B.vfluid;
        if (any_eb) {
            const std::vector<unsigned> m = neighbour_masks(box, *host.flags, L.N);
            if ((st = lalloc(L, (void**)&D->nmask, m.size() * sizeof(unsigned), err)) != MBG_OK) return st;
            cudaMemcpy(D->nmask, m.data(), m.size() * sizeof(unsigned), cudaMemcpyHostToDevice);
        }
    }
    {
        long long* qd = nullptr;
        long long* qsr = nullptr;
        HaloCell* qg = nullptr;
        if ((st = lalloc(L, (void**)&qd, qdst.size() * sizeof(long long), err)) != MBG_OK) return st;
        if ((st = lalloc(L, (void**)&qsr, qsrc.size() * sizeof(long long), err)) != MBG_OK) return st;
        if ((st = lalloc(L, (void**)&qg, qghost.size() * sizeof(HaloCell), err)) != MBG_OK) return st;
        cudaMemcpy(qd, qdst.data(), qdst.size() * sizeof(long long), cudaMemcpyHostToDevice);
        cudaMemcpy(qsr, qsrc.data(), qsrc.size() * sizeof(long long), cudaMemcpyHostToDevice);
        cudaMemcpy(qg, qghost.data(), qghost.size() * sizeof(HaloCell), cudaMemcpyHostToDevice);
        D->qpad.dst = qd;
        D->qpad.src = qsr;
        D->qpad.ncopy = (long long)qdst.size();
        D->qpad.ghost = qg;
        D->qpad.nghost = (long long)qghost.size();
    }
    D->ngather = (long long)hcopy.size();
    D->ngeneral = (long long)general.size();
    if ((st = lalloc(L, (void**)&D->hcopy, hcopy.size() * sizeof(HaloCopy), err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->general, general.size() * sizeof(HaloCell), err)) != MBG_OK) return st;
    cudaMemcpy(D->hcopy, hcopy.data(), hcopy.size() * sizeof(HaloCopy), cudaMemcpyHostToDevice);
    cudaMemcpy(D->general, general.data(), general.size() * sizeof(HaloCell), cudaMemcpyHostToDevice);
    D->nghost_fast = (long long)gfast.size();
    D->nghost_rest = (long long)grest.size();
    for (int d = 0; d < 3; ++d) D->gslot_lg[d] = plan.slot_lg[d];
    if ((st = lalloc(L, (void**)&D->gslots, gsl.size() * sizeof(NbrSlot), err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->gslot_off, gsl_off.size() * sizeof(int), err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->ghost_fast, gfast.size() * sizeof(GhostCell), err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->ghost_rest, grest.size() * sizeof(GhostCell), err)) != MBG_OK) return st;
    cudaMemcpy(D->gslots, gsl.data(), gsl.size() * sizeof(NbrSlot), cudaMemcpyHostToDevice);
    cudaMemcpy(D->gslot_off, gsl_off.data(), gsl_off.size() * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(D->ghost_fast, gfast.data(), gfast.size() * sizeof(GhostCell), cudaMemcpyHostToDevice);
    cudaMemcpy(D->ghost_rest, grest.data(), grest.size() * sizeof(GhostCell), cudaMemcpyHostToDevice);
    D->nsgather = (long long)sdst.size();
    D->nsgen = (long long)scell.size();
    if ((st = lalloc(L, (void**)&D->sdst, sdst.size() * sizeof(long long), err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->ssrc, ssrc.size() * sizeof(long long), err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->scell, scell.size() * sizeof(int), err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->sq, sq.size() * sizeof(int), err)) != MBG_OK) return st;
    cudaMemcpy(D->sdst, sdst.data(), sdst.size() * sizeof(long long), cudaMemcpyHostToDevice);
    cudaMemcpy(D->ssrc, ssrc.data(), ssrc.size() * sizeof(long long), cudaMemcpyHostToDevice);
    cudaMemcpy(D->scell, scell.data(), scell.size() * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(D->sq, sq.data(), sq.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (host.ghosts && NG > 0 && !host.ghosts->empty()) {
        std::vector<XSlot> xc;
        std::vector<int> slot;
        explode_plan(box, *host.ghosts, host, xc, slot);
        ExplodePlan& xp = D->xp;
        xp.n = (long long)slot.size();
        xp.nx = (long long)xc.size();
        if ((st = lalloc(L, (void**)&xp.slot, slot.size() * sizeof(int), err)) != MBG_OK) return st;
        if ((st = lalloc(L, (void**)&xp.xc, xc.size() * sizeof(XSlot), err)) != MBG_OK) return st;
        if ((st = lalloc(L, (void**)&xp.ix, (size_t)xp.nx * 7 * sizeof(int), err)) != MBG_OK) return st;
        if ((st = lalloc(L, (void**)&xp.xs, (size_t)xp.nx * 8 * NQ * sizeof(float), err)) != MBG_OK) return st;
        if ((st = lalloc(L, (void**)&xp.al, (size_t)xp.nx * 6 * sizeof(float), err)) != MBG_OK) return st;
        cudaMemcpy((void*)xp.slot, slot.data(), slot.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy((void*)xp.xc, xc.data(), xc.size() * sizeof(XSlot), cudaMemcpyHostToDevice);
    }
    cudaMemcpy(D->box16, box.data(), box.size() * sizeof(DevBox), cudaMemcpyHostToDevice);
    const size_t sb = (size_t)L.N * NQ * 2;
    for (int b = 0; b < 2; ++b) {
        if ((st = lalloc(L, &L.f[b], sb, err)) != MBG_OK) return st;
        if ((st = lalloc(L, &L.g[b], sb, err)) != MBG_OK) return st;
        cudaMemset(L.f[b], 0xFF, sb);
        cudaMemset(L.g[b], 0xFF, sb);
        if (NG > 0) {
            if ((st = lalloc(L, &L.fg[b], (size_t)NG * NQ * 2, err)) != MBG_OK) return st;
            if ((st = lalloc(L, &L.gg[b], (size_t)NG * NQ * 2, err)) != MBG_OK) return st;
            cudaMemset(L.fg[b], 0xFF, (size_t)NG * NQ * 2);
            cudaMemset(L.gg[b], 0xFF, (size_t)NG * NQ * 2);
        }
    }
    if ((st = lalloc(L, (void**)&D->fo, sb, err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->go, sb, err)) != MBG_OK) return st;
    cudaMemset(D->fo, 0xFF, sb);
    cudaMemset(D->go, 0xFF, sb);
    if ((st = lalloc(L, (void**)&D->qs, (size_t)L.N * 3 * sizeof(float), err)) != MBG_OK) return st;
    cudaMemset(D->qs, 0, (size_t)L.N * 3 * sizeof(float));
    if ((st = lalloc(L, (void**)&L.tmp, (size_t)N * NQ * sizeof(double), err)) != MBG_OK) return st;
    if ((st = lalloc(L, (void**)&D->dk, 2 * sizeof(LowpK), err)) != MBG_OK) return st;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        err = std::string("16-bit level setup: ") + cudaGetErrorString(e);
        return MBG_ECUDA;
    }
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
        k.L = view16(plan, L);
        k.P = bc;
        k.ph = L.ph;
        k.ct = D->ct;
        k.lat64 = make_lattice<double>();
        k.s = bufs(L, a);
        if (with_override) {
            k.s.fo = D->fo;
            k.s.go = D->go;
        }
        k.fA = (u16*)L.f[a];
        k.gA = (u16*)L.g[a];
        k.fB = (u16*)L.f[1 - a];
        k.gB = (u16*)L.g[1 - a];
        k.fBg = (u16*)L.fg[1 - a];
        k.gBg = (u16*)L.gg[1 - a];
        k.phys = nullptr;
        k.nmask = D->nmask;
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
    LowpDev* D = dev_of(L);
    ensure_k(L, plan, known_bc(L), D->with_override, s);
    for (int lat = 0; lat < 2; ++lat) {
        const double* src = lat ? g : f;
        if (!src) continue;
        long long off = 0;
        for (size_t n = 0; n < hbox.size(); ++n) {
            const long long vol = (long long)hbox[n].n[0] * hbox[n].n[1] * hbox[n].n[2];
            cudaError_t e = cudaMemcpy2DAsync(L.tmp + hbox[n].voff, L.NV * sizeof(double), src + off * NQ,
                                              vol * sizeof(double), vol * sizeof(double), NQ, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) { err = std::string("set_state copy: ") + cudaGetErrorString(e); return MBG_ECUDA; }
            off += vol;
        }
        u16* dst = (u16*)(lat ? L.g[L.cur] : L.f[L.cur]);
        const LowpK* k = D->dk + L.cur;
        LOWP16(L.precision == MBG_FP32C_BF16S, encode, k, plan.tiles, plan.ntiles, L.tmp, L.NV, dst, lat, s);
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { err = std::string("set_state: ") + cudaGetErrorString(e); return MBG_ECUDA; }
    return MBG_OK;
}

mbg_status lowp_get_state(LowpLevel& L, const LevelPlan& plan, const std::vector<DevBox>& hbox, double* f,
                          double* g, cudaStream_t s, std::string& err)
{
    LowpDev* D = dev_of(L);
    ensure_k(L, plan, known_bc(L), D->with_override, s);
    for (int lat = 0; lat < 2; ++lat) {
        double* dst = lat ? g : f;
        if (!dst) continue;
        const u16* src = (const u16*)(lat ? L.g[L.cur] : L.f[L.cur]);
        const LowpK* k = D->dk + L.cur;
        LOWP16(L.precision == MBG_FP32C_BF16S, decode, k, plan.tiles, plan.ntiles, src, L.NV, L.tmp, lat, s);
        long long off = 0;
        for (size_t n = 0; n < hbox.size(); ++n) {
            const long long vol = (long long)hbox[n].n[0] * hbox[n].n[1] * hbox[n].n[2];
            cudaError_t e = cudaMemcpy2DAsync(dst + off * NQ, vol * sizeof(double), L.tmp + hbox[n].voff,
                                              L.NV * sizeof(double), vol * sizeof(double), NQ, cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) { err = std::string("get_state copy: ") + cudaGetErrorString(e); return MBG_ECUDA; }
            off += vol;
        }
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { err = std::string("get_state: ") + cudaGetErrorString(e); return MBG_ECUDA; }
    }
    return MBG_OK;
}

void lowp_decode(LowpLevel& L, const LevelPlan& plan, int lat, double* dst, cudaStream_t s)
{
    LowpDev* D = dev_of(L);
    ensure_k(L, plan, known_bc(L), D->with_override, s);
    const u16* src = (const u16*)(lat ? L.g[L.cur] : L.f[L.cur]);
    const LowpK* k = D->dk + L.cur;
    LOWP16(L.precision == MBG_FP32C_BF16S, decode, k, plan.tiles, plan.ntiles, src, L.NV, dst, lat, s);
}

void lowp_decode_ghost(LowpLevel& L, const LevelPlan& plan, int lat, double* dst, cudaStream_t s)
{
    if (L.NG <= 0) return;
    LowpDev* D = dev_of(L);
    ensure_k(L, plan, known_bc(L), D->with_override, s);
    const u16* src = (const u16*)(lat ? L.gg[L.cur] : L.fg[L.cur]);
    const LowpK* k = D->dk + L.cur;
    LOWP16(L.precision == MBG_FP32C_BF16S, decode_flat, k, src, L.NG, dst, lat, s);
}

mbg_status lowp_macro(LowpLevel& L, const LevelPlan& plan, double* out19, cudaStream_t s, std::string& err)
{
    if (plan.ntiles == 0) return MBG_OK;
    LowpDev* D = dev_of(L);
    ensure_k(L, plan, known_bc(L), D->with_override, s);
    const LowpK* k = D->dk + L.cur;
    LOWP16(L.precision == MBG_FP32C_BF16S, macro, k, D->ct, plan.tiles, plan.ntiles, out19, s);
    (void)err;
    return MBG_OK;
}

void lowp_conserved(LowpLevel& L, const LevelPlan& plan, double dV, double* out5, cudaStream_t s)
{
    LowpDev* D = dev_of(L);
    ensure_k(L, plan, known_bc(L), D->with_override, s);
    LOWP16(L.precision == MBG_FP32C_BF16S, conserved, D->dk + L.cur, plan.tiles, plan.ntiles, dV, out5, s);
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
        run(LOWP_STAGE_COALESCE, [&] { LOWP16(bf, coalesce, k, kf, coal, ncoal, D->fo, D->go, 0, s); });
        ++launches;
    }
    if (D->nhalo > 0) {
        run(LOWP_STAGE_HALO, [&] {
            LOWP16(bf, halo_copy, k, D->hcopy, D->ngather, s);
            LOWP16(bf, halo, k, D->general, D->ngeneral, s);
        });
        launches += (D->ngather > 0) + (D->ngeneral > 0);
    }
    if (L.NG > 0 && plan.nghost_cells > 0) {
        run(LOWP_STAGE_GHOST_STREAM, [&] {
            LOWP16(bf, ghost_slots, k, D->gslots, D->gslot_off, D->gslot_lg, D->ghost_fast, D->nghost_fast, D->qs, s);
            LOWP16(bf, ghost_gather, k, D->sdst, D->ssrc, D->nsgather, D->ghost_rest, D->scell, D->sq, D->nsgen, s);
        });
        launches += (D->nghost_fast > 0) + (D->nsgather > 0) + (D->nsgen > 0);
    }
    if (D->variant == 0 || D->variant == 3) {
        const bool pairs = D->variant == 0;
        const Tile* ct = pairs ? D->ctiles : plan.tiles;
        const int nct = pairs ? D->nctiles : plan.ntiles;
        run(LOWP_STAGE_FUSED,
            [&] {
                const QPtrs qp = make_qptrs(L.f[A], L.g[A], L.f[1 - A], L.g[1 - A], L.N);
                PairLists pl;
                if (pairs) {
                    pl.pair = D->ptiles;
                    pl.npair = D->nptiles;
                    pl.pair_ovr = D->potiles;
                    pl.npair_ovr = D->nootiles;
                    pl.pair_eb = D->petiles;
                    pl.npair_eb = D->neetiles;
                }
                launches += LOWP16(bf, two_pass, k, D->ct, D->lat, ct, nct, pl, D->qpad, D->qs, qp, !pairs, s);
            });
    } else {
        const int v = D->variant - 1;
        run(LOWP_STAGE_FUSED,
            [&] { LOWP16(bf, fused, k, D->ct, D->lat, D->ftiles[v], D->nftiles[v], D->nftiles[v], s); });
        ++launches;
    }
    L.cur = 1 - A;
    (void)p;
    (void)dt;
    (void)idx;
    return launches;
}

int lowp_variants() { return 4; }

// Time every step variant on the level's current data and keep the fastest.
// The trials recompute the same step from the same source buffer (the
// parity is not flipped), so the state is unchanged.
mbg_status lowp_autotune(LowpLevel& L, const LevelPlan& plan, const BCParams& bc, const CoalesceCell* coal,
                         long long ncoal, const LowpLevel* fine, const LevelPlan* fplan, int reps, cudaStream_t s,
                         std::string& err)
{
    LowpDev* D = dev_of(L);
    const int keep = L.cur;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const LowpRunner run = [](int, const std::function<void()>& launch) { launch(); };
    mbg_params dummy{};
    const double idx0[3] = {0, 0, 0};
    double best = 0;
    int best_v = 0;
    for (int v = 0; v < lowp_variants(); ++v) {
        D->variant = v;
        lowp_advance(dummy, bc, L, plan, 0.0, idx0, coal, ncoal, fine, fplan, s, run);   // warm-up
        L.cur = keep;
        cudaEventRecord(a, s);
        for (int r = 0; r < reps; ++r) {
            lowp_advance(dummy, bc, L, plan, 0.0, idx0, coal, ncoal, fine, fplan, s, run);
            L.cur = keep;
        }
        cudaEventRecord(b, s);
        cudaError_t e = cudaEventSynchronize(b);
        if (e != cudaSuccess) {
            err = std::string("autotune: ") + cudaGetErrorString(e);
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            return MBG_ECUDA;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        D->variant_ms[v] = ms / reps;
        if (v == 0 || D->variant_ms[v] < best) {
            best = D->variant_ms[v];
            best_v = v;
        }
    }
    D->variant = best_v;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return MBG_OK;
}

void lowp_set_variant(LowpLevel& L, int variant) { dev_of(L)->variant = variant; }

void lowp_variant(LowpLevel& L, int* variant, double ms[4])
{
    LowpDev* D = dev_of(L);
    *variant = D->variant;
    for (int v = 0; v < 4; ++v) ms[v] = D->variant_ms[v];
}

int lowp_explode(LowpLevel& F, const LevelPlan& fplan, const LowpLevel& C, const LevelPlan& cplan, cudaStream_t s)
{
    if (fplan.nghost_cells == 0 || dev_of(F)->xp.nx == 0) return 0;
    LowpLevel& Cm = const_cast<LowpLevel&>(C);
    LowpDev* FD = dev_of(F);
    LowpDev* CD = dev_of(Cm);
    ensure_k(F, fplan, known_bc(F), FD->with_override, s);
    ensure_k(Cm, cplan, known_bc(Cm), CD->with_override, s);
    const LowpK* kf = FD->dk + F.cur;
    const LowpK* kc = CD->dk + C.cur;
    ExplodePlan xp = FD->xp;
    xp.gl = fplan.ghost_list;
    LOWP16(F.precision == MBG_FP32C_BF16S, explode, kf, kc, xp, (u16*)F.fg[F.cur], (u16*)F.gg[F.cur], s);
    return 3;
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
    LOWP16(C.precision == MBG_FP32C_BF16S, coalesce, kc, kf, list, n, (u16*)C.f[C.cur], (u16*)C.g[C.cur], 1, s);
}

void lowp_release(LowpLevel& L)
{
    for (void* p : L.allocs) cudaFree(p);
    L.allocs.clear();
    delete (LowpDev*)L.impl;
    L.impl = nullptr;
}

}  // namespace mbg

