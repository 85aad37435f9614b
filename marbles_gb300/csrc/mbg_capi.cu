// mbg_capi.cu -- the C ABI of include/marbles_gb300.h: context, level plans
// and the subcycled step (Source/LBM.cpp:398-544 restated as launches).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/marbles_gb300.h"
#include "mbg_kernels.h"
#include "mbg_lowp.h"

using namespace mbg;

namespace {

struct HBox {
    int lo[3], hi[3];
    int n(int d) const { return hi[d] - lo[d] + 1; }
    long long vol() const { return (long long)n(0) * n(1) * n(2); }
    long long gvol() const { return (long long)(n(0) + 6) * (n(1) + 6) * (n(2) + 6); }
};

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
};

struct Level {
    std::vector<HBox> boxes;
    std::vector<DevBox> hbox;
    int dlo[3], dhi[3];
    int G[3], nb[3];
    std::vector<int> omap;
    std::vector<uint8_t> hflags;
    long long N = 0, NG = 0, NF = 0;
    bool has_ghost = false;
    // device
    DevBox* d_box = nullptr;
    int* d_omap = nullptr;
    uint8_t* d_flags = nullptr;
    double* f[2] = {nullptr, nullptr};
    double* g[2] = {nullptr, nullptr};
    double* fg[2] = {nullptr, nullptr};
    double* gg[2] = {nullptr, nullptr};
    double* md = nullptr;
    double* gqc = nullptr;
    Tile* d_tiles = nullptr;
    int ntiles = 0;
    NbrSlot* d_slots = nullptr;
    int* d_slot_off = nullptr;
    NbrSlot* d_gslots = nullptr;       // FP64 ghost-shell tables (chunks 3 cells wide at the box faces)
    int* d_gslot_off = nullptr;
    GhostCell* d_ghost_fast = nullptr; // ghost cells of all-fluid boxes with a ghost-shell table
    long long nghost_fast = 0;
    GhostCell* d_ghost_gen = nullptr;  // the other ghost cells (general pull)
    long long nghost_gen = 0;
    int slot_lg[3] = {0, 0, 0};
    int slot_max = 0;
    Tile* d_fast_tiles = nullptr;
    int nfast = 0;
    Tile* d_fasteb_tiles = nullptr;
    int nfasteb = 0;
    Tile* d_fastbc_tiles = nullptr;
    int nfastbc = 0;
    Tile* d_fastebbc_tiles = nullptr;
    int nfastebbc = 0;
    Tile* d_gen_tiles = nullptr;
    int ngen = 0;
    GhostCell* d_ghost = nullptr;
    GhostCell* d_ghost1 = nullptr;
    long long nghost = 0, nghost1 = 0;
    // coalescence of the next finer level onto this one (ng = 1 and ng = 0)
    CoalesceCell* d_coal1 = nullptr;
    long long ncoal1 = 0;
    CoalesceCell* d_coal0 = nullptr;
    long long ncoal0 = 0;
    // FP64 explosion plan and scratch (fine levels)
    int* d_xslot = nullptr;
    XSlot* d_xc = nullptr;
    long long nx = 0;
    int* d_xix = nullptr;
    double* d_xs = nullptr;
    double* d_xal = nullptr;
    int cur = 0;
    double dt = 1.0;
    double dx[3], idx[3];
    // the FP64 macro scratch holds the moments the level's last collision
    // started from (false after a state upload or a remake)
    bool md_valid = false;
    // the level's entries of mbg_ctx::allocs (freed when a regrid drops it)
    size_t alloc_begin = 0, alloc_end = 0;
    LevelPlan plan;
    LowpLevel lowp;   // 16-bit storage form buffers (mbg_lowp.cu)
};

}  // namespace

// kernel classes timed by mbg_set_timing
enum { TK_MOMENTS = 0, TK_COLLIDE, TK_GHOST_STREAM, TK_GHOST_MOMENTS, TK_EXPLODE, TK_COALESCE, TK_FUSED, TK_HALO, TK_OTHER, TK_N };
static const char* TK_NAMES[TK_N] = {"k_moments", "k_collide", "k_ghost_stream", "k_ghost_moments",
                                     "k_explode", "k_coalesce", "k_lowp_step", "k_halo", "other"};

struct mbg_ctx {
    // two coarse steps captured into a CUDA graph (see mbg_step)
    cudaGraphExec_t graph = nullptr;
    std::vector<int> graph_par;
    long long graph_launches = 0;
    mbg_params p;
    bool timing = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> events;
    std::vector<cudaEvent_t> event_pool;
    long long tk_count[TK_N] = {};
    double tk_ms[TK_N] = {};
    cudaStream_t s = nullptr;
    bool own_stream = false;
    std::vector<Level> lv;
    BCParams bc;
    Lattice<double> lat;
    std::string err;
    long long launches = 0;
    double* d_red = nullptr;   // small reduction scratch
    unsigned long long* d_check = nullptr;   // mbg_check_state: two counts and the first key
    double* d_out19 = nullptr;
    size_t out19_n = 0;
    double* d_stage = nullptr;   // FP64 state transfers: one lattice of a level in host layout
    size_t stage_n = 0;
    // per-block partial sums of the EB force (3 per tile of every level)
    double* d_partial = nullptr;
    size_t partial_n = 0;
    // FP64 decode of a 16-bit level's f and g for the output kernels
    double* d_dec[2] = {nullptr, nullptr};
    size_t dec_n[2] = {0, 0};
    double* d_decg[2] = {nullptr, nullptr};   // and of its ghost fabs
    size_t decg_n[2] = {0, 0};
    std::vector<void*> allocs;
};

static void drop_graph(mbg_ctx* ctx)
{
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
}

static std::string g_create_err;

void mbg_set_global_error(const std::string& msg) { g_create_err = msg; }

#define MBG_CUDA(call)                                                                   \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);               \
            return MBG_ECUDA;                                                            \
        }                                                                                \
    } while (0)

static mbg_status fail(mbg_ctx* ctx, mbg_status st, const std::string& m)
{
    ctx->err = m;
    return st;
}

static cudaEvent_t take_event(mbg_ctx* ctx)
{
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// records an event pair around the launches issued by `launch`
template <class F>
static void timed(mbg_ctx* ctx, int k, F&& launch)
{
    if (!ctx->timing) {
        launch();
        return;
    }
    cudaEvent_t a = take_event(ctx), b = take_event(ctx);
    cudaEventRecord(a, ctx->s);
    launch();
    cudaEventRecord(b, ctx->s);
    ctx->events.push_back({k, {a, b}});
}

static void drain_events(mbg_ctx* ctx)
{
    if (ctx->events.empty()) return;
    cudaStreamSynchronize(ctx->s);
    for (auto& e : ctx->events) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e.second.first, e.second.second);
        ctx->tk_count[e.first] += 1;
        ctx->tk_ms[e.first] += ms;
        ctx->event_pool.push_back(e.second.first);
        ctx->event_pool.push_back(e.second.second);
    }
    ctx->events.clear();
}

template <class T>
static mbg_status dalloc(mbg_ctx* ctx, T** p, size_t n)
{
    *p = nullptr;
    if (n == 0) return MBG_OK;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T));
    if (e != cudaSuccess) {
        ctx->err = std::string("cudaMalloc of ") + std::to_string(n * sizeof(T)) + " bytes: " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? MBG_ENOMEM : MBG_ECUDA;
    }
    ctx->allocs.push_back(q);
    *p = (T*)q;
    return MBG_OK;
}

static Phys64 phys64(const mbg_ctx* ctx, const Level& L)
{
    Phys64 ph;
    const mbg_params& p = ctx->p;
    ph.mesh_speed = p.dx_outer / p.dt_outer;
    ph.Rg = 28.96 / p.m_bar;
    ph.cv = ph.Rg / (p.adiabatic_exponent - 1.0);
    ph.nu = p.nu;
    ph.alpha = p.alpha;
    ph.dt = L.dt;
    for (int d = 0; d < 3; ++d) ph.idx[d] = L.idx[d];
    ph.small_num = std::numeric_limits<double>::epsilon() * 1e10;
    ph.lat = ctx->lat;
    return ph;
}

static bool wrap_host(const Level& L, const int per[3], int p[3])
{
    for (int d = 0; d < 3; ++d) {
        if (p[d] < L.dlo[d] || p[d] > L.dhi[d]) {
            if (!per[d]) return false;
            const int len = L.dhi[d] - L.dlo[d] + 1;
            p[d] = L.dlo[d] + (((p[d] - L.dlo[d]) % len) + len) % len;
        }
    }
    return true;
}

static int owner_host(const Level& L, const int p[3])
{
    const int bi = (p[0] - L.dlo[0]) / L.G[0], bj = (p[1] - L.dlo[1]) / L.G[1], bk = (p[2] - L.dlo[2]) / L.G[2];
    return L.omap[((size_t)bk * L.nb[1] + bj) * L.nb[0] + bi];
}

// Neighbour-slot tables of every box (NbrSlot), the chunks below and above
// the box w cells wide (1 for the step's pulls, 3 for the pulls of the
// coarse-fine ghost shell): a chunk maps to one box when
// all its cells (after the periodic wrap) lie in that box's valid cells at
// one fixed offset, or to the box's ghost fab when none lies in a box and the
// box has one.  ok[n] is set when every chunk of box n maps (no non-periodic
// domain side within one cell, no chunk across a box edge) and its table
// fits; off[n] is the table's first slot, -1 for a box without one.
static void build_slots(const Level& L, const int* is_periodic, const int lg[3], std::vector<NbrSlot>& out,
                        std::vector<int>& off, std::vector<char>& ok, int w = 1, std::vector<char>* has_bc = nullptr)
{
    if (has_bc) has_bc->assign(L.boxes.size(), 0);
    const int nbox = (int)L.boxes.size();
    out.clear();
    off.assign(nbox, -1);
    ok.assign(nbox, 0);
    for (int n = 0; n < nbox; ++n) {
        const HBox& b = L.boxes[n];
        const DevBox& B = L.hbox[n];
        int nch[3], tc[3];
        for (int d = 0; d < 3; ++d) {
            nch[d] = (b.n(d) + (1 << lg[d]) - 1) >> lg[d];
            tc[d] = nch[d] + 2;
        }
        const long long T = (long long)tc[0] * tc[1] * tc[2];
        if (T > SLOT_TABLE_MAX) continue;
        const size_t t0 = out.size();
        out.resize(t0 + (size_t)T, NbrSlot{0, 0, 0, -1, 0});
        bool all = true;
        for (int cz = 0; cz < tc[2]; ++cz)
            for (int cy = 0; cy < tc[1]; ++cy)
                for (int cx = 0; cx < tc[0]; ++cx) {
                    const int c3[3] = {cx, cy, cz};
                    NbrSlot& S = out[t0 + cx + (size_t)tc[0] * (cy + (size_t)tc[1] * cz)];
                    int rlo[3], rhi[3];
                    bool inside = true;
                    for (int d = 0; d < 3; ++d) {
                        if (c3[d] == 0) {
                            rlo[d] = -w;
                            rhi[d] = -1;
                        } else if (c3[d] == tc[d] - 1) {
                            rlo[d] = b.n(d);
                            rhi[d] = b.n(d) + w - 1;
                        }
                        else {
                            rlo[d] = (c3[d] - 1) << lg[d];
                            rhi[d] = std::min(c3[d] << lg[d], b.n(d)) - 1;
                        }
                        inside = inside && c3[d] > 0 && c3[d] < tc[d] - 1;
                    }
                    if (inside) {   // the box itself
                        S.base = B.voff;
                        S.sy = B.sy;
                        S.sz = B.sz;
                        S.ghost = 0;
                        continue;
                    }
                    int owner = -2;         // -2: unset, -1: uncovered
                    int delta[3] = {0, 0, 0};
                    bool good = true;
                    long long outside = 0, cells = 0;
                    for (int z = rlo[2]; z <= rhi[2] && good; ++z)
                        for (int y = rlo[1]; y <= rhi[1] && good; ++y)
                            for (int x = rlo[0]; x <= rhi[0] && good; ++x) {
                                int gp[3] = {b.lo[0] + x, b.lo[1] + y, b.lo[2] + z};
                                ++cells;
                                if (!wrap_host(L, is_periodic, gp)) {
                                    ++outside;   // beyond a non-periodic side
                                    continue;
                                }
                                if (outside > 0) { good = false; break; }
                                const int o = owner_host(L, gp);
                                int dl[3] = {0, 0, 0};
                                if (o >= 0) {
                                    const int loc[3] = {gp[0] - L.boxes[o].lo[0], gp[1] - L.boxes[o].lo[1],
                                                        gp[2] - L.boxes[o].lo[2]};
                                    dl[0] = loc[0] - x; dl[1] = loc[1] - y; dl[2] = loc[2] - z;
                                }
                                if (owner == -2) {
                                    owner = o;
                                    for (int d = 0; d < 3; ++d) delta[d] = dl[d];
                                } else if (o != owner || dl[0] != delta[0] || dl[1] != delta[1] || dl[2] != delta[2]) {
                                    good = false;
                                }
                            }
                    if (good && outside > 0) {
                        // the step tables take a chunk wholly beyond a
                        // non-periodic side: its pulls are the BC's values
                        if (outside == cells && w == 1 && has_bc) {
                            S.ghost = 2;
                            (*has_bc)[n] = 1;
                        } else {
                            all = false;
                        }
                    } else if (good && owner >= 0) {
                        const DevBox& O = L.hbox[owner];
                        S.base = O.voff + (long long)delta[2] * O.sz + (long long)delta[1] * O.sy + delta[0];
                        S.sy = O.sy;
                        S.sz = O.sz;
                        S.ghost = 0;
                    } else if (good && B.goff >= 0) {
                        const int gx = B.n[0] + 6, gy = B.n[1] + 6;
                        S.base = B.goff + 3LL * gy * gx + 3LL * gx + 3;
                        S.sy = gx;
                        S.sz = gx * gy;
                        S.ghost = 1;
                    } else {
                        all = false;
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

// chunk length of the slot tables along d: the largest power of two, at most
// 32, dividing the level's owner-map grain (every box corner and length)
static int slot_lg(const Level& L, int d)
{
    int lg = 0;
    while (lg < 5 && L.G[d] % (2 << lg) == 0) ++lg;
    return lg;
}

static void refresh_plan(mbg_ctx* ctx, Level& L)
{
    LevelView<double> v;
    v.box = L.d_box;
    v.nbox = (int)L.boxes.size();
    for (int d = 0; d < 3; ++d) {
        v.dlo[d] = L.dlo[d];
        v.dhi[d] = L.dhi[d];
        v.per[d] = ctx->p.is_periodic[d];
        v.G[d] = L.G[d];
        v.nb[d] = L.nb[d];
    }
    v.omap = L.d_omap;
    v.N = L.N;
    v.NG = L.NG;
    v.flags = L.d_flags;
    L.plan.view64 = v;
    L.plan.tiles = L.d_tiles;
    L.plan.ntiles = L.ntiles;
    L.plan.slots = L.d_slots;
    L.plan.slot_off = L.d_slot_off;
    L.plan.gslots = L.d_gslots;
    L.plan.gslot_off = L.d_gslot_off;
    L.plan.ghost_fast = L.d_ghost_fast;
    L.plan.nghost_fast = L.nghost_fast;
    L.plan.ghost_gen = L.d_ghost_gen;
    L.plan.nghost_gen = L.nghost_gen;
    for (int d = 0; d < 3; ++d) L.plan.slot_lg[d] = L.slot_lg[d];
    L.plan.slot_max = L.slot_max;
    L.plan.fast_tiles = L.d_fast_tiles;
    L.plan.nfast = L.nfast;
    L.plan.fasteb_tiles = L.d_fasteb_tiles;
    L.plan.nfasteb = L.nfasteb;
    L.plan.fastbc_tiles = L.d_fastbc_tiles;
    L.plan.nfastbc = L.nfastbc;
    L.plan.fastebbc_tiles = L.d_fastebbc_tiles;
    L.plan.nfastebbc = L.nfastebbc;
    L.plan.gen_tiles = L.d_gen_tiles;
    L.plan.ngen = L.ngen;
    L.plan.ghost_list = L.d_ghost;
    L.plan.nghost_cells = L.nghost;
    L.plan.ghost_list1 = L.d_ghost1;
    L.plan.nghost1 = L.nghost1;
    L.plan.xslot = L.d_xslot;
    L.plan.xc = L.d_xc;
    L.plan.nx = L.nx;
    L.plan.xix = L.d_xix;
    L.plan.xs = L.d_xs;
    L.plan.xal = L.d_xal;
}

extern "C" {

mbg_status mbg_create(const mbg_params* params, void* cuda_stream, mbg_ctx** out)
{
    if (!params || !out) {
        g_create_err = "mbg_create: null argument";
        return MBG_EINVAL;
    }
    *out = nullptr;
    const mbg_params& p = *params;
    for (int d = 0; d < 3; ++d) {
        if (p.n_cell[d] <= 0) { g_create_err = "mbg_create: n_cell must be positive"; return MBG_EINVAL; }
        if (!(p.prob_hi[d] > p.prob_lo[d])) { g_create_err = "mbg_create: prob_hi must exceed prob_lo"; return MBG_EINVAL; }
        const int codes[] = {0, 1, 2, 3, 5, 6, 7, 8};
        for (int lh = 0; lh < 2; ++lh) {
            const int c = lh ? p.bc_hi[d] : p.bc_lo[d];
            if (std::find(std::begin(codes), std::end(codes), c) == std::end(codes)) {
                g_create_err = "mbg_create: unknown boundary-condition code " + std::to_string(c);
                return MBG_EINVAL;
            }
            if (p.is_periodic[d] && c != 0) {
                g_create_err = "mbg_create: BC is periodic in direction " + std::to_string(d) + " but bc code is not 0";
                return MBG_EINVAL;
            }
            if (!p.is_periodic[d] && c == 0) {
                g_create_err = "mbg_create: BC is interior in direction " + std::to_string(d) + " but not periodic";
                return MBG_EINVAL;
            }
            if (c == 3 && !(p.is_periodic[(d + 1) % 3] && p.is_periodic[(d + 2) % 3])) {
                // The reference's functor reads, for a pressure ghost cell, the
                // populations around the adjacent interior cell; next to a
                // non-periodic tangential side some of those are ghost cells that
                // the same functor pass rewrites, so the result depends on the
                // order the functor visits ghost cells.  With periodic
                // tangential sides every read is a valid cell or a periodic copy.
                g_create_err = "mbg_create: the pressure boundary condition (code 3) in direction " +
                               std::to_string(d) + " needs periodic tangential directions";
                return MBG_EINVAL;
            }
        }
    }
    if (!(p.nu > 0) || !(p.alpha > 0) || !(p.dt_outer > 0) || !(p.m_bar > 0) || !(p.adiabatic_exponent > 1.0)) {
        g_create_err = "mbg_create: nu, alpha, dt_outer, m_bar must be positive and adiabatic_exponent > 1";
        return MBG_EINVAL;
    }
    if (p.vbc_dir < 0 || p.vbc_dir > 2 || p.vbc_normal_dir < 0 || p.vbc_normal_dir > 2 || p.vbc_tangential_dir < 0 ||
        p.vbc_tangential_dir > 2) {
        g_create_err = "mbg_create: velocity-BC directions must be 0, 1 or 2";
        return MBG_EINVAL;
    }
    if (p.precision < 0 || p.precision > 2) {
        g_create_err = "mbg_create: unknown precision form";
        return MBG_EINVAL;
    }
    auto* ctx = new (std::nothrow) mbg_ctx();
    if (!ctx) { g_create_err = "mbg_create: out of host memory"; return MBG_ENOMEM; }
    ctx->p = p;
    if (cuda_stream) {
        ctx->s = (cudaStream_t)cuda_stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->s, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            g_create_err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
            delete ctx;
            return MBG_ECUDA;
        }
        ctx->own_stream = true;
    }
    ctx->lat = make_lattice<double>();
    BCParams& bc = ctx->bc;
    for (int d = 0; d < 3; ++d) { bc.bc[d] = p.bc_lo[d]; bc.bc[d + 3] = p.bc_hi[d]; }
    bc.velbc = p.velbc_type;
    bc.vbc_dir = p.vbc_dir;
    bc.vbc_nd = p.vbc_normal_dir;
    bc.vbc_td = p.vbc_tangential_dir;
    bc.u_ref = p.vbc_u_ref;
    bc.rho0 = p.vbc_initial_density;
    bc.temp = p.vbc_initial_temperature;
    bc.gamma = p.vbc_adiabatic_exponent;
    bc.Rg = 28.96 / p.vbc_m_bar;
    for (int d = 0; d < 3; ++d) {
        bc.prob_lo[d] = p.prob_lo[d];
        bc.prob_hi[d] = p.prob_hi[d];
        bc.dx[d] = (p.prob_hi[d] - p.prob_lo[d]) / p.n_cell[d];
    }
    if (dalloc(ctx, &ctx->d_red, 8) != MBG_OK) {
        g_create_err = ctx->err;
        mbg_destroy(ctx);
        return MBG_ENOMEM;
    }
    *out = ctx;
    return MBG_OK;
}

void mbg_destroy(mbg_ctx* ctx)
{
    if (ctx) drop_graph(ctx);
    if (!ctx) return;
    if (ctx->s) cudaStreamSynchronize(ctx->s);
    drain_events(ctx);
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    for (auto& L : ctx->lv)
        if (L.lowp.impl) lowp_release(L.lowp);
    for (void* q : ctx->allocs) cudaFree(q);
    if (ctx->own_stream && ctx->s) cudaStreamDestroy(ctx->s);
    delete ctx;
}

const char* mbg_last_error(const mbg_ctx* ctx)
{
    return ctx ? ctx->err.c_str() : g_create_err.c_str();
}

mbg_status mbg_level_cells(const mbg_ctx* ctx, int lev, long long* n)
{
    if (!ctx || !n) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)ctx->lv.size()) return MBG_ESTATE;
    *n = ctx->lv[lev].N;
    return MBG_OK;
}

long long mbg_launch_count(const mbg_ctx* ctx) { return ctx ? ctx->launches : 0; }

mbg_status mbg_define_level(mbg_ctx* ctx, int lev, int nbox, const int* lohi, const uint8_t* flags)
{
    if (ctx) drop_graph(ctx);
    if (!ctx) return MBG_EINVAL;
    if (lev != (int)ctx->lv.size()) return fail(ctx, MBG_ESTATE, "mbg_define_level: levels must be defined in order 0, 1, ...");
    if (nbox <= 0 || !lohi) return fail(ctx, MBG_EINVAL, "mbg_define_level: need at least one box");
    const mbg_params& p = ctx->p;
    const size_t alloc_begin = ctx->allocs.size();
    Level L;
    const int r = 1 << lev;
    for (int d = 0; d < 3; ++d) {
        L.dlo[d] = 0;
        L.dhi[d] = p.n_cell[d] * r - 1;
        L.dx[d] = (p.prob_hi[d] - p.prob_lo[d]) / (p.n_cell[d] * r);
        L.idx[d] = 1.0 / L.dx[d];
    }
    L.dt = 1.0;
    for (int l = 1; l <= lev; ++l) L.dt = L.dt / 2;
    L.boxes.resize(nbox);
    for (int n = 0; n < nbox; ++n) {
        HBox& b = L.boxes[n];
        for (int d = 0; d < 3; ++d) {
            b.lo[d] = lohi[6 * n + d];
            b.hi[d] = lohi[6 * n + 3 + d];
            if (b.hi[d] < b.lo[d] || b.lo[d] < L.dlo[d] || b.hi[d] > L.dhi[d])
                return fail(ctx, MBG_EINVAL, "mbg_define_level: box " + std::to_string(n) + " is empty or outside the domain");
            if (b.n(d) > 32000) return fail(ctx, MBG_EINVAL, "mbg_define_level: box too long");
        }
    }
    // owner map on gcd bins; also rejects overlapping boxes
    for (int d = 0; d < 3; ++d) {
        int g = L.dhi[d] - L.dlo[d] + 1;
        for (const auto& b : L.boxes) {
            g = std::gcd(g, b.lo[d] - L.dlo[d]);
            g = std::gcd(g, b.hi[d] + 1 - L.dlo[d]);
        }
        L.G[d] = g > 0 ? g : 1;
        L.nb[d] = (L.dhi[d] - L.dlo[d] + 1) / L.G[d];
    }
    L.omap.assign((size_t)L.nb[0] * L.nb[1] * L.nb[2], -1);
    for (int n = 0; n < nbox; ++n) {
        const HBox& b = L.boxes[n];
        for (int k = b.lo[2] / L.G[2]; k <= b.hi[2] / L.G[2]; ++k)
            for (int j = b.lo[1] / L.G[1]; j <= b.hi[1] / L.G[1]; ++j)
                for (int i = b.lo[0] / L.G[0]; i <= b.hi[0] / L.G[0]; ++i) {
                    int& o = L.omap[((size_t)k * L.nb[1] + j) * L.nb[0] + i];
                    if (o >= 0) return fail(ctx, MBG_EINVAL, "mbg_define_level: boxes overlap");
                    o = n;
                }
    }
    if (lev == 0) {
        long long cov = 0;
        for (const auto& b : L.boxes) cov += b.vol();
        long long dom = (long long)(L.dhi[0] + 1) * (L.dhi[1] + 1) * (L.dhi[2] + 1);
        if (cov != dom) return fail(ctx, MBG_EINVAL, "mbg_define_level: level 0 boxes must cover the domain");
    }
    // per-box offsets and flags
    L.hbox.resize(nbox);
    long long voff = 0, foff = 0;
    for (int n = 0; n < nbox; ++n) {
        DevBox& B = L.hbox[n];
        for (int d = 0; d < 3; ++d) { B.lo[d] = L.boxes[n].lo[d]; B.n[d] = L.boxes[n].n(d); }
        B.sy = B.n[0];
        B.sz = B.n[0] * B.n[1];
        B.voff = voff;
        B.hoff = voff;
        B.foff = foff;
        B.goff = -1;
        B.phys = 0;
        B.own_domain = 0;
        voff += L.boxes[n].vol();
        foff += L.boxes[n].gvol();
    }
    L.N = voff;
    L.NF = foff;
    L.hflags.assign(foff, FL_FLUID);
    if (flags) {
        for (long long i = 0; i < foff; ++i) L.hflags[i] = flags[i] & (FL_FLUID | FL_EBB);
    }
    for (int n = 0; n < nbox; ++n) {
        DevBox& B = L.hbox[n];
        B.all_fluid = 1;
        for (long long i = 0; i < L.boxes[n].gvol(); ++i)
            if (!(L.hflags[B.foff + i] & FL_FLUID)) { B.all_fluid = 0; break; }
        B.vfluid = 1;
        for (int z = -1; z <= B.n[2] && B.vfluid; ++z)
            for (int y = -1; y <= B.n[1] && B.vfluid; ++y)
                for (int x = -1; x <= B.n[0]; ++x)
                    if (!(L.hflags[B.foff + ((long long)(z + 3) * (B.n[1] + 6) + (y + 3)) * (B.n[0] + 6) + (x + 3)] &
                          FL_FLUID)) {
                        B.vfluid = 0;
                        break;
                    }
    }
    // coarse-fine ghost shell of fine levels
    std::vector<GhostCell> ghosts, ghosts1;
    std::vector<XSlot> xcells;   // FP64 explosion plan (staging for the copies below)
    std::vector<int> xslot;
    if (lev > 0) {
        Level& C = ctx->lv[lev - 1];
        long long goff = 0;
        for (int n = 0; n < nbox; ++n) {
            const HBox& b = L.boxes[n];
            bool any = false;
            for (int z = -3; z < b.n(2) + 3; ++z)
                for (int y = -3; y < b.n(1) + 3; ++y)
                    for (int x = -3; x < b.n(0) + 3; ++x) {
                        if (x >= 0 && y >= 0 && z >= 0 && x < b.n(0) && y < b.n(1) && z < b.n(2)) continue;
                        int gp[3] = {b.lo[0] + x, b.lo[1] + y, b.lo[2] + z};
                        if (!wrap_host(L, p.is_periodic, gp))
                            return fail(ctx, MBG_EINVAL,
                                        "mbg_define_level: fine level " + std::to_string(lev) +
                                            " reaches a non-periodic domain boundary (unsupported)");
                        if (owner_host(L, gp) >= 0) continue;
                        // the interpolation stencil must lie in the coarse level's valid cells
                        const int cp[3] = {gp[0] >> 1, gp[1] >> 1, gp[2] >> 1};
                        for (int d = 0; d < 3; ++d)
                            for (int s = -1; s <= 1; ++s) {
                                int c[3] = {cp[0], cp[1], cp[2]};
                                c[d] += s;
                                if (!wrap_host(C, p.is_periodic, c) || owner_host(C, c) < 0)
                                    return fail(ctx, MBG_EINVAL,
                                                "mbg_define_level: level " + std::to_string(lev) +
                                                    " is not properly nested in level " + std::to_string(lev - 1));
                            }
                        GhostCell gc;
                        gc.box = n;
                        gc.x = (short)x; gc.y = (short)y; gc.z = (short)z;
                        gc.layer = (short)std::max({x < 0 ? -x : x - b.n(0) + 1, y < 0 ? -y : y - b.n(1) + 1,
                                                    z < 0 ? -z : z - b.n(2) + 1, 0});
                        ghosts.push_back(gc);
                        if (gc.layer == 1) ghosts1.push_back(gc);
                        any = true;
                    }
            if (any) {
                L.hbox[n].goff = goff;
                goff += b.gvol();
            }
        }
        L.NG = goff;
        L.has_ghost = goff > 0;
        // cells of the uncovered shell also need their flags from the caller
        // coalescence lists onto the coarse level (ascending box order, the
        // last box whose grown coarsened box holds a cell wins)
        for (int ng = 0; ng <= 1; ++ng) {
            std::unordered_map<long long, int> win;
            std::vector<long long> order;
            for (int n = 0; n < nbox; ++n) {
                const HBox& b = L.boxes[n];
                if (b.lo[0] % 2 || b.lo[1] % 2 || b.lo[2] % 2 || b.n(0) % 2 || b.n(1) % 2 || b.n(2) % 2)
                    return fail(ctx, MBG_EINVAL, "mbg_define_level: fine boxes must be aligned to the ratio 2");
                for (int cz = b.lo[2] / 2 - ng; cz <= b.hi[2] / 2 + ng; ++cz)
                    for (int cy = b.lo[1] / 2 - ng; cy <= b.hi[1] / 2 + ng; ++cy)
                        for (int cx = b.lo[0] / 2 - ng; cx <= b.hi[0] / 2 + ng; ++cx) {
                            int c[3] = {cx, cy, cz};
                            if (cx < C.dlo[0] || cy < C.dlo[1] || cz < C.dlo[2] || cx > C.dhi[0] || cy > C.dhi[1] ||
                                cz > C.dhi[2] || owner_host(C, c) < 0)
                                return fail(ctx, MBG_EINVAL,
                                            "mbg_define_level: coalescence region of level " + std::to_string(lev) +
                                                " leaves the coarse level");
                            const long long key = ((long long)cz * 65536 + cy) * 65536 + cx;
                            auto it = win.find(key);
                            if (it == win.end()) { win[key] = n; order.push_back(key); }
                            else it->second = n;
                        }
            }
            std::vector<CoalesceCell> cl;
            cl.reserve(order.size());
            for (long long key : order) {
                const int cx = (int)(key % 65536), cy = (int)((key / 65536) % 65536), cz = (int)(key / 65536 / 65536);
                int c[3] = {cx, cy, cz};
                const int o = owner_host(C, c);
                // children that are valid cells of a fine box give the same
                // values whichever box is named (reads go to their owner), so
                // name that box: the kernels then read them at fixed offsets.
                // Fine boxes are aligned to the ratio, so one box holds all
                // eight.  The last-wins box stays for children in no box.
                const int child[3] = {2 * cx, 2 * cy, 2 * cz};
                const int own = owner_host(L, child);
                const int n = own >= 0 ? own : win[key];
                CoalesceCell cc;
                cc.cbox = o;
                cc.fbox = n;
                cc.cx = (short)(cx - C.boxes[o].lo[0]);
                cc.cy = (short)(cy - C.boxes[o].lo[1]);
                cc.cz = (short)(cz - C.boxes[o].lo[2]);
                cc.fx = (short)(2 * cx - L.boxes[n].lo[0]);
                cc.fy = (short)(2 * cy - L.boxes[n].lo[1]);
                cc.fz = (short)(2 * cz - L.boxes[n].lo[2]);
                cl.push_back(cc);
                // flag the coarse cell
                const DevBox& CB = C.hbox[o];
                const long long fi = CB.foff + ((long long)(cc.cz + 3) * (CB.n[1] + 6) + (cc.cy + 3)) * (CB.n[0] + 6) + (cc.cx + 3);
                C.hflags[fi] |= (uint8_t)(ng == 1 ? (uint8_t)FL_OVR : (uint8_t)FL_COV);
            }
            // cells whose children all lie in the named box first: each cell
            // appears once, so the order changes no result, and warps then
            // take the kernels' fixed-offset path together
            std::stable_partition(cl.begin(), cl.end(), [&](const CoalesceCell& cc) {
                const DevBox& A = L.hbox[cc.fbox];
                return cc.fx >= 0 && cc.fy >= 0 && cc.fz >= 0 && cc.fx + 1 < A.n[0] && cc.fy + 1 < A.n[1] &&
                       cc.fz + 1 < A.n[2];
            });
            CoalesceCell** dst = ng ? &C.d_coal1 : &C.d_coal0;
            long long* cnt = ng ? &C.ncoal1 : &C.ncoal0;
            mbg_status st = dalloc(ctx, dst, cl.size());
            if (st != MBG_OK) return st;
            if (!cl.empty())
                MBG_CUDA(cudaMemcpyAsync(*dst, cl.data(), cl.size() * sizeof(CoalesceCell), cudaMemcpyHostToDevice, ctx->s));
            *cnt = (long long)cl.size();
        }
        // re-upload the coarse flags with the coalescence bits
        MBG_CUDA(cudaMemcpyAsync(C.d_flags, C.hflags.data(), C.hflags.size(), cudaMemcpyHostToDevice, ctx->s));
        if (p.precision != MBG_FP64) lowp_retile(C.lowp, C.hflags, ctx->s);
    }
    // device allocations
    mbg_status st;
    if ((st = dalloc(ctx, &L.d_box, nbox)) != MBG_OK) return st;
    MBG_CUDA(cudaMemcpyAsync(L.d_box, L.hbox.data(), nbox * sizeof(DevBox), cudaMemcpyHostToDevice, ctx->s));
    if ((st = dalloc(ctx, &L.d_omap, L.omap.size())) != MBG_OK) return st;
    MBG_CUDA(cudaMemcpyAsync(L.d_omap, L.omap.data(), L.omap.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
    if ((st = dalloc(ctx, &L.d_flags, L.hflags.size())) != MBG_OK) return st;
    MBG_CUDA(cudaMemcpyAsync(L.d_flags, L.hflags.data(), L.hflags.size(), cudaMemcpyHostToDevice, ctx->s));
    std::vector<Tile> tiles, fast_tiles, fasteb_tiles, fastbc_tiles, fastebbc_tiles, gen_tiles;
    std::vector<NbrSlot> slots;
    std::vector<int> slot_off;
    std::vector<char> slot_ok;
    for (int d = 0; d < 3; ++d) L.slot_lg[d] = slot_lg(L, d);
    std::vector<char> slot_bc;
    build_slots(L, p.is_periodic, L.slot_lg, slots, slot_off, slot_ok, 1, &slot_bc);
    L.slot_max = 0;
    for (int n = 0; n < nbox; ++n) {
        const bool simple = slot_ok[n];
        if (simple) {
            int t = 1;
            for (int d = 0; d < 3; ++d) t *= ((L.boxes[n].n(d) + (1 << L.slot_lg[d]) - 1) >> L.slot_lg[d]) + 2;
            L.slot_max = std::max(L.slot_max, t);
        }
        std::vector<Tile>& list = !simple ? gen_tiles
                                  : slot_bc[n] ? (L.hbox[n].all_fluid ? fastbc_tiles : fastebbc_tiles)
                                               : (L.hbox[n].all_fluid ? fast_tiles : fasteb_tiles);
        for (long long s = 0; s < L.boxes[n].vol(); s += TILE_CELLS) {
            tiles.push_back(Tile{n, (int)s});
            list.push_back(Tile{n, (int)s});
        }
    }
    L.ntiles = (int)tiles.size();
    L.nfast = (int)fast_tiles.size();
    L.nfasteb = (int)fasteb_tiles.size();
    L.nfastbc = (int)fastbc_tiles.size();
    L.nfastebbc = (int)fastebbc_tiles.size();
    L.ngen = (int)gen_tiles.size();
    if ((st = dalloc(ctx, &L.d_tiles, tiles.size())) != MBG_OK) return st;
    MBG_CUDA(cudaMemcpyAsync(L.d_tiles, tiles.data(), tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, ctx->s));
    if ((st = dalloc(ctx, &L.d_fast_tiles, fast_tiles.size())) != MBG_OK) return st;
    if ((st = dalloc(ctx, &L.d_gen_tiles, gen_tiles.size())) != MBG_OK) return st;
    if ((st = dalloc(ctx, &L.d_fasteb_tiles, fasteb_tiles.size())) != MBG_OK) return st;
    if ((st = dalloc(ctx, &L.d_fastbc_tiles, fastbc_tiles.size())) != MBG_OK) return st;
    if ((st = dalloc(ctx, &L.d_fastebbc_tiles, fastebbc_tiles.size())) != MBG_OK) return st;
    if (!fastbc_tiles.empty())
        MBG_CUDA(cudaMemcpyAsync(L.d_fastbc_tiles, fastbc_tiles.data(), fastbc_tiles.size() * sizeof(Tile),
                                 cudaMemcpyHostToDevice, ctx->s));
    if (!fastebbc_tiles.empty())
        MBG_CUDA(cudaMemcpyAsync(L.d_fastebbc_tiles, fastebbc_tiles.data(), fastebbc_tiles.size() * sizeof(Tile),
                                 cudaMemcpyHostToDevice, ctx->s));
    if (!fasteb_tiles.empty())
        MBG_CUDA(cudaMemcpyAsync(L.d_fasteb_tiles, fasteb_tiles.data(), fasteb_tiles.size() * sizeof(Tile),
                                 cudaMemcpyHostToDevice, ctx->s));
    if ((st = dalloc(ctx, &L.d_slots, slots.size())) != MBG_OK) return st;
    if (!fast_tiles.empty())
        MBG_CUDA(cudaMemcpyAsync(L.d_fast_tiles, fast_tiles.data(), fast_tiles.size() * sizeof(Tile),
                                 cudaMemcpyHostToDevice, ctx->s));
    if (!gen_tiles.empty())
        MBG_CUDA(cudaMemcpyAsync(L.d_gen_tiles, gen_tiles.data(), gen_tiles.size() * sizeof(Tile),
                                 cudaMemcpyHostToDevice, ctx->s));
    if (!slots.empty())
        MBG_CUDA(cudaMemcpyAsync(L.d_slots, slots.data(), slots.size() * sizeof(NbrSlot), cudaMemcpyHostToDevice,
                                 ctx->s));
    if ((st = dalloc(ctx, &L.d_slot_off, slot_off.size())) != MBG_OK) return st;
    MBG_CUDA(cudaMemcpyAsync(L.d_slot_off, slot_off.data(), slot_off.size() * sizeof(int), cudaMemcpyHostToDevice,
                             ctx->s));
    L.nghost = (long long)ghosts.size();
    L.nghost1 = (long long)ghosts1.size();
    if ((st = dalloc(ctx, &L.d_ghost, ghosts.size())) != MBG_OK) return st;
    if ((st = dalloc(ctx, &L.d_ghost1, ghosts1.size())) != MBG_OK) return st;
    if (!ghosts.empty())
        MBG_CUDA(cudaMemcpyAsync(L.d_ghost, ghosts.data(), ghosts.size() * sizeof(GhostCell), cudaMemcpyHostToDevice, ctx->s));
    if (!ghosts1.empty())
        MBG_CUDA(cudaMemcpyAsync(L.d_ghost1, ghosts1.data(), ghosts1.size() * sizeof(GhostCell), cudaMemcpyHostToDevice, ctx->s));
    // FP64 ghost stream: cells of all-fluid boxes whose ghost-shell chunks
    // each map to one box or the ghost fab take the table pull
    std::vector<NbrSlot> gslots;
    std::vector<int> gslot_off;
    std::vector<char> gslot_ok;
    std::vector<GhostCell> gfast, ggen;
    if (lev > 0 && p.precision == MBG_FP64 && !ghosts.empty()) {
        build_slots(L, p.is_periodic, L.slot_lg, gslots, gslot_off, gslot_ok, 3);
        for (const GhostCell& gc : ghosts) (gslot_ok[gc.box] && L.hbox[gc.box].all_fluid ? gfast : ggen).push_back(gc);
        if ((st = dalloc(ctx, &L.d_gslots, gslots.size())) != MBG_OK) return st;
        if ((st = dalloc(ctx, &L.d_gslot_off, gslot_off.size())) != MBG_OK) return st;
        if ((st = dalloc(ctx, &L.d_ghost_fast, gfast.size())) != MBG_OK) return st;
        if ((st = dalloc(ctx, &L.d_ghost_gen, ggen.size())) != MBG_OK) return st;
        if (!gslots.empty())
            MBG_CUDA(cudaMemcpyAsync(L.d_gslots, gslots.data(), gslots.size() * sizeof(NbrSlot), cudaMemcpyHostToDevice,
                                     ctx->s));
        MBG_CUDA(cudaMemcpyAsync(L.d_gslot_off, gslot_off.data(), gslot_off.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, ctx->s));
        if (!gfast.empty())
            MBG_CUDA(cudaMemcpyAsync(L.d_ghost_fast, gfast.data(), gfast.size() * sizeof(GhostCell),
                                     cudaMemcpyHostToDevice, ctx->s));
        if (!ggen.empty())
            MBG_CUDA(cudaMemcpyAsync(L.d_ghost_gen, ggen.data(), ggen.size() * sizeof(GhostCell), cudaMemcpyHostToDevice,
                                     ctx->s));
    } else {
        ggen = ghosts;
        if ((st = dalloc(ctx, &L.d_ghost_gen, ggen.size())) != MBG_OK) return st;
        if (!ggen.empty())
            MBG_CUDA(cudaMemcpyAsync(L.d_ghost_gen, ggen.data(), ggen.size() * sizeof(GhostCell), cudaMemcpyHostToDevice,
                                     ctx->s));
    }
    L.nghost_fast = (long long)gfast.size();
    L.nghost_gen = (long long)ggen.size();
    if (p.precision == MBG_FP64) {
        for (int b = 0; b < 2; ++b) {
            if ((st = dalloc(ctx, &L.f[b], (size_t)L.N * NQ)) != MBG_OK) return st;
            if ((st = dalloc(ctx, &L.g[b], (size_t)L.N * NQ)) != MBG_OK) return st;
            MBG_CUDA(cudaMemsetAsync(L.f[b], 0, (size_t)L.N * NQ * sizeof(double), ctx->s));
            MBG_CUDA(cudaMemsetAsync(L.g[b], 0, (size_t)L.N * NQ * sizeof(double), ctx->s));
            if (L.NG > 0) {
                if ((st = dalloc(ctx, &L.fg[b], (size_t)L.NG * NQ)) != MBG_OK) return st;
                if ((st = dalloc(ctx, &L.gg[b], (size_t)L.NG * NQ)) != MBG_OK) return st;
                MBG_CUDA(cudaMemsetAsync(L.fg[b], 0, (size_t)L.NG * NQ * sizeof(double), ctx->s));
                MBG_CUDA(cudaMemsetAsync(L.gg[b], 0, (size_t)L.NG * NQ * sizeof(double), ctx->s));
            }
        }
        if ((st = dalloc(ctx, &L.md, (size_t)L.N * MD_NCOMP)) != MBG_OK) return st;
        MBG_CUDA(cudaMemsetAsync(L.md, 0, (size_t)L.N * MD_NCOMP * sizeof(double), ctx->s));
        if (L.NG > 0) {
            if ((st = dalloc(ctx, &L.gqc, (size_t)L.NG * 3)) != MBG_OK) return st;
            MBG_CUDA(cudaMemsetAsync(L.gqc, 0, (size_t)L.NG * 3 * sizeof(double), ctx->s));
        }
        if (!ghosts.empty()) {
            // the plan keeps coarse storage indices in 32 bits
            if (ctx->lv[lev - 1].N >= (1LL << 31))
                return fail(ctx, MBG_EINVAL, "mbg_define_level: coarse level holds more than 2^31 cells");
            LevelHost h{};
            for (int d = 0; d < 3; ++d) {
                h.dlo[d] = L.dlo[d];
                h.dhi[d] = L.dhi[d];
                h.per[d] = p.is_periodic[d];
            }
            explode_plan(L.hbox, ghosts, h, xcells, xslot);
            L.nx = (long long)xcells.size();
            if ((st = dalloc(ctx, &L.d_xslot, xslot.size())) != MBG_OK) return st;
            if ((st = dalloc(ctx, &L.d_xc, xcells.size())) != MBG_OK) return st;
            if ((st = dalloc(ctx, &L.d_xix, (size_t)L.nx * 7)) != MBG_OK) return st;
            if ((st = dalloc(ctx, &L.d_xs, (size_t)L.nx * 8 * NQ)) != MBG_OK) return st;
            if ((st = dalloc(ctx, &L.d_xal, (size_t)L.nx * 6)) != MBG_OK) return st;
            MBG_CUDA(cudaMemcpyAsync(L.d_xslot, xslot.data(), xslot.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->s));
            MBG_CUDA(cudaMemcpyAsync(L.d_xc, xcells.data(), xcells.size() * sizeof(XSlot), cudaMemcpyHostToDevice, ctx->s));
        }
    }
    // the host staging vectors above must outlive their copies
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    ctx->lv.push_back(std::move(L));
    Level& LL = ctx->lv.back();
    LL.alloc_begin = alloc_begin;
    LL.alloc_end = ctx->allocs.size();
    refresh_plan(ctx, LL);
    if (p.precision != MBG_FP64) {
        LevelHost host;
        host.flags = &LL.hflags;
        host.omap = &LL.omap;
        host.ghosts = &ghosts;
        for (int d = 0; d < 3; ++d) {
            host.dlo[d] = LL.dlo[d];
            host.dhi[d] = LL.dhi[d];
            host.G[d] = LL.G[d];
            host.nb[d] = LL.nb[d];
            host.per[d] = ctx->p.is_periodic[d];
        }
        mbg_status s2 = lowp_define(ctx->p, LL.plan, LL.hbox, LL.N, LL.NG, LL.dt, LL.idx, host, LL.lowp, ctx->err);
        if (s2 != MBG_OK) return s2;
    }
    return MBG_OK;
}

// the FP64 staging buffer, grown to one lattice of level L in host layout
// (allocated at the first transfer of a level that size, not in the step)
static mbg_status stage_buffer(mbg_ctx* ctx, const Level& L)
{
    const size_t need = (size_t)L.N * NQ;
    if (ctx->stage_n >= need) return MBG_OK;
    if (ctx->d_stage) {   // a smaller buffer of an earlier level: freed, not kept
        MBG_CUDA(cudaStreamSynchronize(ctx->s));
        for (auto& a : ctx->allocs)
            if (a == ctx->d_stage) {
                cudaFree(a);
                a = nullptr;
            }
        ctx->d_stage = nullptr;
        ctx->stage_n = 0;
    }
    mbg_status st = dalloc(ctx, &ctx->d_stage, need);
    if (st != MBG_OK) return st;
    ctx->stage_n = need;
    return MBG_OK;
}

mbg_status mbg_set_state(mbg_ctx* ctx, int lev, const double* f, const double* g)
{
    if (!ctx) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)ctx->lv.size()) return fail(ctx, MBG_ESTATE, "mbg_set_state: level not defined");
    Level& L = ctx->lv[lev];
    L.md_valid = false;
    if (ctx->p.precision != MBG_FP64) {
        mbg_status s2 = lowp_set_state(L.lowp, L.plan, L.hbox, f, g, ctx->s, ctx->err);
        ctx->launches += 2;
        return s2;
    }
    mbg_status st = stage_buffer(ctx, L);
    if (st != MBG_OK) return st;
    const size_t bytes = (size_t)L.N * NQ * sizeof(double);
    for (int lat = 0; lat < 2; ++lat) {
        const double* src = lat ? g : f;
        if (!src) continue;
        MBG_CUDA(cudaMemcpyAsync(ctx->d_stage, src, bytes, cudaMemcpyHostToDevice, ctx->s));
        launch_stage(L.plan, ctx->d_stage, lat ? L.g[L.cur] : L.f[L.cur], 1, ctx->s);
        ctx->launches++;
    }
    MBG_CUDA(cudaGetLastError());
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    return MBG_OK;
}

mbg_status mbg_get_state(mbg_ctx* ctx, int lev, double* f, double* g)
{
    if (!ctx) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)ctx->lv.size()) return fail(ctx, MBG_ESTATE, "mbg_get_state: level not defined");
    Level& L = ctx->lv[lev];
    if (ctx->p.precision != MBG_FP64) {
        mbg_status s2 = lowp_get_state(L.lowp, L.plan, L.hbox, f, g, ctx->s, ctx->err);
        ctx->launches += 2;
        return s2;
    }
    mbg_status st = stage_buffer(ctx, L);
    if (st != MBG_OK) return st;
    const size_t bytes = (size_t)L.N * NQ * sizeof(double);
    for (int lat = 0; lat < 2; ++lat) {
        double* dst = lat ? g : f;
        if (!dst) continue;
        launch_stage(L.plan, ctx->d_stage, lat ? L.g[L.cur] : L.f[L.cur], 0, ctx->s);
        ctx->launches++;
        MBG_CUDA(cudaMemcpyAsync(dst, ctx->d_stage, bytes, cudaMemcpyDeviceToHost, ctx->s));
    }
    MBG_CUDA(cudaGetLastError());
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    return MBG_OK;
}

mbg_status mbg_get_macro(mbg_ctx* ctx, int lev, double* macro)
{
    if (!ctx || !macro) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)ctx->lv.size()) return fail(ctx, MBG_ESTATE, "mbg_get_macro: level not defined");
    Level& L = ctx->lv[lev];
    const size_t need = (size_t)L.N * 19;
    if (ctx->out19_n < need) {
        mbg_status st = dalloc(ctx, &ctx->d_out19, need);
        if (st != MBG_OK) return st;
        ctx->out19_n = need;
    }
    if (ctx->p.precision != MBG_FP64) {
        mbg_status s2 = lowp_macro(L.lowp, L.plan, ctx->d_out19, ctx->s, ctx->err);
        if (s2 != MBG_OK) return s2;
    } else {
        launch_macro_local(L.plan, phys64(ctx, L), L.f[L.cur], L.g[L.cur], ctx->d_out19, ctx->s);
    }
    ctx->launches++;
    MBG_CUDA(cudaGetLastError());
    MBG_CUDA(cudaMemcpyAsync(macro, ctx->d_out19, need * sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    return MBG_OK;
}

}  // extern "C"

// ---- the step ---------------------------------------------------------------
static mbg_status explode(mbg_ctx* ctx, int lev)
{
    Level& F = ctx->lv[lev];
    Level& C = ctx->lv[lev - 1];
    if (ctx->p.precision != MBG_FP64) {
        int n = 0;
        timed(ctx, TK_EXPLODE, [&] { n = lowp_explode(F.lowp, F.plan, C.lowp, C.plan, ctx->s); });
        ctx->launches += n;
    } else {
        timed(ctx, TK_EXPLODE,
              [&] { launch_explode(F.plan, C.plan, C.f[C.cur], C.g[C.cur], F.fg[F.cur], F.gg[F.cur], ctx->s); });
        ctx->launches += F.plan.nx > 0 ? 3 : 0;
    }
    MBG_CUDA(cudaGetLastError());
    return MBG_OK;
}

static mbg_status advance(mbg_ctx* ctx, int lev)
{
    Level& L = ctx->lv[lev];
    const bool has_finer = lev + 1 < (int)ctx->lv.size();
    if (ctx->p.precision != MBG_FP64) {
        const LowpLevel* fine = has_finer ? &ctx->lv[lev + 1].lowp : nullptr;
        const LevelPlan* fplan = has_finer ? &ctx->lv[lev + 1].plan : nullptr;
        int nl = 0;
        static const int stage_tk[4] = {TK_COALESCE, TK_GHOST_STREAM, TK_FUSED, TK_HALO};
        nl = lowp_advance(ctx->p, ctx->bc, L.lowp, L.plan, L.dt, L.idx, has_finer ? L.d_coal1 : nullptr,
                          has_finer ? L.ncoal1 : 0, fine, fplan, ctx->s,
                          [&](int stage, const std::function<void()>& launch) { timed(ctx, stage_tk[stage], launch); });
        if (nl < 0) return fail(ctx, MBG_ENOMEM, "16-bit form: allocation of the coalescence buffer failed");
        ctx->launches += nl;
        MBG_CUDA(cudaGetLastError());
        return MBG_OK;
    }
    const Phys64 ph = phys64(ctx, L);
    const int A = L.cur, Bf = 1 - L.cur;
    if (has_finer) {
        Level& F = ctx->lv[lev + 1];
        timed(ctx, TK_COALESCE, [&] {
            launch_coalesce(L.plan, F.plan, ctx->bc, ph, L.d_coal1, L.ncoal1, F.f[F.cur], F.g[F.cur], F.fg[F.cur],
                            F.gg[F.cur], L.f[A], L.g[A], L.fg[A], L.gg[A], L.f[Bf], L.g[Bf], 0, ctx->s);
        });
        ctx->launches++;
    }
    if (L.NG > 0) {
        timed(ctx, TK_GHOST_STREAM, [&] {
            launch_ghost_stream(L.plan, ctx->bc, ph, L.f[A], L.g[A], L.fg[A], L.gg[A], L.fg[Bf], L.gg[Bf], ctx->s);
        });
        timed(ctx, TK_GHOST_MOMENTS, [&] {
            launch_ghost_moments(L.plan, ph, L.fg[Bf], L.gg[Bf], L.gqc, ctx->s);
        });
        ctx->launches += ghost_stream_launches(L.plan) + (L.plan.nghost1 > 0);
    }
    timed(ctx, TK_MOMENTS, [&] {
        launch_moments(L.plan, ctx->bc, ph, L.f[A], L.g[A], L.fg[A], L.gg[A], L.f[Bf], L.g[Bf], L.md, ctx->s);
    });
    timed(ctx, TK_COLLIDE, [&] {
        launch_collide(L.plan, ctx->bc, ph, L.f[A], L.g[A], L.fg[A], L.gg[A], L.f[Bf], L.g[Bf], L.md, L.gqc,
                       ctx->s);
    });
    ctx->launches += 2 * fp64_step_launches(L.plan);
    MBG_CUDA(cudaGetLastError());
    L.cur = Bf;
    L.md_valid = true;
    return MBG_OK;
}

static mbg_status time_step(mbg_ctx* ctx, int lev)
{
    mbg_status st;
    if (lev + 1 < (int)ctx->lv.size()) {
        if ((st = explode(ctx, lev + 1)) != MBG_OK) return st;
        for (int i = 1; i <= 2; ++i)
            if ((st = time_step(ctx, lev + 1)) != MBG_OK) return st;
    }
    return advance(ctx, lev);
}

extern "C" {

// buffer parities of every level (both forms)
static std::vector<int> parities(const mbg_ctx* ctx)
{
    std::vector<int> v;
    for (const Level& L : ctx->lv) {
        v.push_back(L.cur);
        v.push_back(L.lowp.cur);
    }
    return v;
}

// Capture two coarse steps (every level advances an even number of times, so
// the buffer parities come back to where they were) into a graph.  Nothing
// runs during the capture; the host bookkeeping it performs is undone by
// construction.  Returns false (and leaves no graph) if the capture fails.
static bool capture_steps(mbg_ctx* ctx)
{
    drop_graph(ctx);
    const std::vector<int> par0 = parities(ctx);
    const long long l0 = ctx->launches;
    if (cudaStreamBeginCapture(ctx->s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
    mbg_status st = MBG_OK;
    for (int i = 0; i < 2 && st == MBG_OK; ++i) st = time_step(ctx, 0);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->s, &g);
    const long long nl = ctx->launches - l0;
    ctx->launches = l0;
    if (st != MBG_OK || e != cudaSuccess || parities(ctx) != par0) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return false;
    }
    const cudaError_t ei = cudaGraphInstantiate(&ctx->graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        ctx->graph = nullptr;
        cudaGetLastError();
        return false;
    }
    ctx->graph_par = par0;
    ctx->graph_launches = nl;
    return true;
}

// Without per-kernel timing, pairs of coarse steps replay a CUDA graph of
// the whole subcycled hierarchy (captured on first use, re-captured when the
// buffer parities differ from the capture's, e.g. after manual
// advance/fillpatch calls); timing runs launch by launch.
mbg_status mbg_step(mbg_ctx* ctx, int nsteps)
{
    if (!ctx) return MBG_EINVAL;
    if (ctx->lv.empty()) return fail(ctx, MBG_ESTATE, "mbg_step: no level defined");
    int left = nsteps;
    if (left >= 2 && !ctx->timing) {
        // the first step runs eagerly (it uploads the constant blocks)
        if (!ctx->graph || parities(ctx) != ctx->graph_par) {
            mbg_status st = time_step(ctx, 0);
            if (st != MBG_OK) return st;
            --left;
            if (left >= 2) capture_steps(ctx);
        }
        while (left >= 2 && ctx->graph && parities(ctx) == ctx->graph_par) {
            MBG_CUDA(cudaGraphLaunch(ctx->graph, ctx->s));
            ctx->launches += ctx->graph_launches;
            left -= 2;
        }
    }
    for (; left > 0; --left) {
        mbg_status st = time_step(ctx, 0);
        if (st != MBG_OK) return st;
    }
    return MBG_OK;
}

mbg_status mbg_advance_level(mbg_ctx* ctx, int lev)
{
    if (!ctx) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)ctx->lv.size()) return fail(ctx, MBG_ESTATE, "mbg_advance_level: level not defined");
    return advance(ctx, lev);
}

mbg_status mbg_fillpatch(mbg_ctx* ctx, int lev)
{
    if (!ctx) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)ctx->lv.size()) return fail(ctx, MBG_ESTATE, "mbg_fillpatch: level not defined");
    if (lev == 0) return MBG_OK;  // level-0 ghosts are never stored: pulls read neighbours and BCs directly
    return explode(ctx, lev);
}

mbg_status mbg_autotune(mbg_ctx* ctx, int reps)
{
    if (!ctx) return MBG_EINVAL;
    drop_graph(ctx);
    if (reps < 1) return fail(ctx, MBG_EINVAL, "mbg_autotune: reps must be >= 1");
    if (ctx->p.precision == MBG_FP64) return MBG_OK;
    const int nl = (int)ctx->lv.size();
    for (int lev = 0; lev < nl; ++lev) {
        Level& L = ctx->lv[lev];
        const bool has_finer = lev + 1 < nl;
        mbg_status st = lowp_autotune(L.lowp, L.plan, ctx->bc, has_finer ? L.d_coal1 : nullptr,
                                      has_finer ? L.ncoal1 : 0, has_finer ? &ctx->lv[lev + 1].lowp : nullptr,
                                      has_finer ? &ctx->lv[lev + 1].plan : nullptr, reps, ctx->s, ctx->err);
        if (st != MBG_OK) return st;
    }
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    return MBG_OK;
}

mbg_status mbg_tuning(mbg_ctx* ctx, int lev, int* variant, double ms[4])
{
    if (!ctx || !variant || !ms) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)ctx->lv.size()) return fail(ctx, MBG_EINVAL, "mbg_tuning: no such level");
    if (ctx->p.precision == MBG_FP64) {
        *variant = 0;
        for (int v = 0; v < 4; ++v) ms[v] = 0.0;
        return MBG_OK;
    }
    lowp_variant(ctx->lv[lev].lowp, variant, ms);
    return MBG_OK;
}

mbg_status mbg_set_variant(mbg_ctx* ctx, int lev, int variant)
{
    if (!ctx) return MBG_EINVAL;
    drop_graph(ctx);
    if (lev < -1 || lev >= (int)ctx->lv.size()) return fail(ctx, MBG_EINVAL, "mbg_set_variant: no such level");
    const int nv = ctx->p.precision == MBG_FP64 ? 1 : lowp_variants();
    if (variant < 0 || variant >= nv) return fail(ctx, MBG_EINVAL, "mbg_set_variant: no such variant");
    if (ctx->p.precision == MBG_FP64) return MBG_OK;
    for (int l = 0; l < (int)ctx->lv.size(); ++l)
        if (lev < 0 || l == lev) lowp_set_variant(ctx->lv[l].lowp, variant);
    return MBG_OK;
}

mbg_status mbg_average_down(mbg_ctx* ctx, int crse_lev, int crse_ng)
{
    if (!ctx) return MBG_EINVAL;
    if (crse_lev < 0 || crse_lev + 1 >= (int)ctx->lv.size())
        return fail(ctx, MBG_ESTATE, "mbg_average_down: needs levels crse_lev and crse_lev+1");
    if (crse_ng != 0 && crse_ng != 1) return fail(ctx, MBG_EINVAL, "mbg_average_down: crse_ng must be 0 or 1");
    Level& C = ctx->lv[crse_lev];
    Level& F = ctx->lv[crse_lev + 1];
    const CoalesceCell* list = crse_ng ? C.d_coal1 : C.d_coal0;
    const long long n = crse_ng ? C.ncoal1 : C.ncoal0;
    if (ctx->p.precision != MBG_FP64) {
        lowp_average_down(C.lowp, C.plan, F.lowp, F.plan, list, n, ctx->s);
    } else {
        launch_coalesce(C.plan, F.plan, ctx->bc, phys64(ctx, C), list, n, F.f[F.cur], F.g[F.cur], F.fg[F.cur],
                        F.gg[F.cur], C.f[C.cur], C.g[C.cur], C.fg[C.cur], C.gg[C.cur], C.f[C.cur], C.g[C.cur], 1,
                        ctx->s);
    }
    ctx->launches++;
    MBG_CUDA(cudaGetLastError());
    return MBG_OK;
}

// FP64 views of a level's stored populations for the output kernels: the
// FP64 form's own buffers; the 16-bit forms' populations and ghost fabs
// decoded into FP64 scratch of the context (f, and g when want_g)
static mbg_status fp64_state(mbg_ctx* ctx, Level& L, bool want_g, const double** f, const double** g,
                             const double** fg, const double** gg)
{
    if (ctx->p.precision == MBG_FP64) {
        *f = L.f[L.cur];
        *g = L.g[L.cur];
        *fg = L.fg[L.cur];
        *gg = L.gg[L.cur];
        return MBG_OK;
    }
    const size_t need = (size_t)L.N * NQ, needg = (size_t)L.NG * NQ;
    for (int lat = 0; lat < (want_g ? 2 : 1); ++lat) {
        if (ctx->dec_n[lat] < need) {
            mbg_status st = dalloc(ctx, &ctx->d_dec[lat], need);
            if (st != MBG_OK) return st;
            ctx->dec_n[lat] = need;
        }
        if (ctx->decg_n[lat] < needg) {
            mbg_status st = dalloc(ctx, &ctx->d_decg[lat], needg);
            if (st != MBG_OK) return st;
            ctx->decg_n[lat] = needg;
        }
        lowp_decode(L.lowp, L.plan, lat, ctx->d_dec[lat], ctx->s);
        ctx->launches++;
        if (needg > 0) {
            lowp_decode_ghost(L.lowp, L.plan, lat, ctx->d_decg[lat], ctx->s);
            ctx->launches++;
        }
    }
    *f = ctx->d_dec[0];
    *g = want_g ? ctx->d_dec[1] : nullptr;
    *fg = needg > 0 ? ctx->d_decg[0] : nullptr;
    *gg = needg > 0 && want_g ? ctx->d_decg[1] : nullptr;
    return MBG_OK;
}

mbg_status mbg_eb_forces(mbg_ctx* ctx, double out[3])
{
    if (!ctx || !out) return MBG_EINVAL;
    if (ctx->lv.empty()) return fail(ctx, MBG_ESTATE, "mbg_eb_forces: no level defined");
    long long nt = 0;
    for (auto& L : ctx->lv) nt += L.ntiles;
    if (ctx->partial_n < (size_t)nt * 3) {
        mbg_status st = dalloc(ctx, &ctx->d_partial, (size_t)nt * 3);
        if (st != MBG_OK) return st;
        ctx->partial_n = (size_t)nt * 3;
    }
    long long off = 0;
    for (auto& L : ctx->lv) {
        const double *f, *g, *fg, *gg;
        mbg_status st = fp64_state(ctx, L, false, &f, &g, &fg, &gg);
        if (st != MBG_OK) return st;
        launch_eb_forces(L.plan, f, fg, ctx->d_partial + off * 3, ctx->s);
        ctx->launches++;
        off += L.ntiles;
    }
    launch_sum_partials(ctx->d_partial, nt, ctx->d_red, ctx->s);
    ctx->launches++;
    MBG_CUDA(cudaGetLastError());
    MBG_CUDA(cudaMemcpyAsync(out, ctx->d_red, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    return MBG_OK;
}

mbg_status mbg_check_state(mbg_ctx* ctx, long long counts[2], long long first[4])
{
    if (!ctx || !counts || !first) return MBG_EINVAL;
    if (ctx->lv.empty()) return fail(ctx, MBG_ESTATE, "mbg_check_state: no level defined");
    if (!ctx->d_check) {
        mbg_status st = dalloc(ctx, &ctx->d_check, 3);
        if (st != MBG_OK) return st;
    }
    const unsigned long long init[3] = {0ULL, 0ULL, ~0ULL};
    MBG_CUDA(cudaMemcpyAsync(ctx->d_check, init, sizeof(init), cudaMemcpyHostToDevice, ctx->s));
    for (int lev = 0; lev < (int)ctx->lv.size(); ++lev) {
        Level& L = ctx->lv[lev];
        const double *f, *g, *fg, *gg;
        mbg_status st = fp64_state(ctx, L, true, &f, &g, &fg, &gg);
        if (st != MBG_OK) return st;
        launch_check(L.plan, f, g, lev, ctx->d_check, ctx->s);
        ctx->launches++;
    }
    MBG_CUDA(cudaGetLastError());
    unsigned long long out[3];
    MBG_CUDA(cudaMemcpyAsync(out, ctx->d_check, sizeof(out), cudaMemcpyDeviceToHost, ctx->s));
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    counts[0] = (long long)out[0];
    counts[1] = (long long)out[1];
    if (out[2] == ~0ULL) {
        for (int i = 0; i < 4; ++i) first[i] = -1;
    } else {
        first[0] = (long long)(out[2] >> 58);
        first[1] = (long long)((out[2] >> 38) & 0xFFFFFULL);
        first[2] = (long long)((out[2] >> 7) & 0x7FFFFFFFULL);
        first[3] = (long long)(out[2] & 0x7FULL);
    }
    return MBG_OK;
}

// ---- tagging and regrid ------------------------------------------------------
mbg_status mbg_tag_cells(mbg_ctx* ctx, int lev, const mbg_tag* tags, int ntags, double time, uint8_t* out)
{
    if (!ctx || !out || ntags < 0 || (ntags > 0 && !tags)) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)ctx->lv.size()) return fail(ctx, MBG_ESTATE, "mbg_tag_cells: level not defined");
    if (ntags > MBG_MAX_TAGS) return fail(ctx, MBG_EINVAL, "mbg_tag_cells: too many criteria");
    TagSet ts;
    ts.n = ntags;
    for (int c = 0; c < ntags; ++c) {
        const mbg_tag& t = tags[c];
        if (t.field < 0 || t.field > 19 || t.kind < 0 || t.kind > 2)
            return fail(ctx, MBG_EINVAL, "mbg_tag_cells: field must be 0..19 and kind 0..2");
        ts.t[c] = t;
    }
    Level& L = ctx->lv[lev];
    const double *f, *g, *fg, *gg;
    mbg_status st = fp64_state(ctx, L, true, &f, &g, &fg, &gg);
    if (st != MBG_OK) return st;
    const size_t need = (size_t)L.N * 19;
    if (ctx->out19_n < need) {
        if ((st = dalloc(ctx, &ctx->d_out19, need)) != MBG_OK) return st;
        ctx->out19_n = need;
    }
    const bool md = ctx->p.precision == MBG_FP64 && L.md_valid;
    double plo[3];
    for (int d = 0; d < 3; ++d) plo[d] = ctx->p.prob_lo[d];
    launch_tags(L.plan, phys64(ctx, L), md ? L.md : nullptr, f, g, ts, time, lev, plo, L.dx,
                (uint8_t*)ctx->d_out19, ctx->s);
    ctx->launches++;
    MBG_CUDA(cudaGetLastError());
    MBG_CUDA(cudaMemcpyAsync(out, ctx->d_out19, (size_t)L.N, cudaMemcpyDeviceToHost, ctx->s));
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    return MBG_OK;
}

// frees the device memory of levels first.. and forgets them; the coarser
// level loses its coalescence lists and override flags
static mbg_status drop_levels(mbg_ctx* ctx, int first)
{
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    for (int l = (int)ctx->lv.size() - 1; l >= first; --l) {
        Level& L = ctx->lv[l];
        if (L.lowp.impl) lowp_release(L.lowp);
        for (size_t i = L.alloc_begin; i < L.alloc_end && i < ctx->allocs.size(); ++i) {
            cudaFree(ctx->allocs[i]);
            ctx->allocs[i] = nullptr;
        }
    }
    ctx->lv.resize(first);
    Level& C = ctx->lv[first - 1];
    C.d_coal1 = C.d_coal0 = nullptr;
    C.ncoal1 = C.ncoal0 = 0;
    for (auto& v : C.hflags) v = (uint8_t)(v & ~(FL_OVR | FL_COV));
    MBG_CUDA(cudaMemcpyAsync(C.d_flags, C.hflags.data(), C.hflags.size(), cudaMemcpyHostToDevice, ctx->s));
    if (ctx->p.precision != MBG_FP64) lowp_retile(C.lowp, C.hflags, ctx->s);
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    return MBG_OK;
}

mbg_status mbg_regrid(mbg_ctx* ctx, int first_lev, int nlev, const int* nbox, const int* lohi, const uint8_t* flags)
{
    if (!ctx || nlev < 0 || (nlev > 0 && (!nbox || !lohi || !flags))) return MBG_EINVAL;
    if (first_lev < 1 || first_lev > (int)ctx->lv.size())
        return fail(ctx, MBG_EINVAL, "mbg_regrid: first_lev must be 1 .. number of levels");
    drop_graph(ctx);
    // the old fine levels' state on the host, with their boxes
    struct Old { std::vector<HBox> boxes; std::vector<long long> off; std::vector<double> f, g; };
    std::vector<Old> old;
    for (int l = first_lev; l < (int)ctx->lv.size(); ++l) {
        Old o;
        o.boxes = ctx->lv[l].boxes;
        long long n = 0;
        for (const HBox& b : o.boxes) { o.off.push_back(n); n += b.vol(); }
        o.f.resize((size_t)n * NQ);
        o.g.resize((size_t)n * NQ);
        mbg_status st = mbg_get_state(ctx, l, o.f.data(), o.g.data());
        if (st != MBG_OK) return st;
        old.push_back(std::move(o));
    }
    mbg_status st = drop_levels(ctx, first_lev);
    if (st != MBG_OK) return st;
    long long boff = 0, foff = 0;
    for (int m = 0; m < nlev; ++m) {
        const int lev = first_lev + m;
        st = mbg_define_level(ctx, lev, nbox[m], lohi + 6 * boff, flags + foff);
        if (st != MBG_OK) return st;
        Level& F = ctx->lv[lev];
        Level& C = ctx->lv[lev - 1];
        // the interpolation stencil of every new cell must lie in the coarse level
        for (const HBox& b : F.boxes)
            for (int z = b.lo[2] / 2 - 1; z <= b.hi[2] / 2 + 1; ++z)
                for (int y = b.lo[1] / 2 - 1; y <= b.hi[1] / 2 + 1; ++y)
                    for (int x = b.lo[0] / 2 - 1; x <= b.hi[0] / 2 + 1; ++x) {
                        int c[3] = {x, y, z};
                        if (!wrap_host(C, ctx->p.is_periodic, c) || owner_host(C, c) < 0)
                            return fail(ctx, MBG_EINVAL, "mbg_regrid: level " + std::to_string(lev) +
                                                             " is not properly nested in level " +
                                                             std::to_string(lev - 1));
                    }
        // coarse-to-fine interpolation of every new cell on the GPU
        const double *cf, *cg, *cfg, *cgg;
        if ((st = fp64_state(ctx, C, true, &cf, &cg, &cfg, &cgg)) != MBG_OK) return st;
        double *d_if = nullptr, *d_ig = nullptr;
        cudaError_t e = cudaMalloc(&d_if, (size_t)F.N * NQ * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc(&d_ig, (size_t)F.N * NQ * sizeof(double));
        std::vector<double> nf((size_t)F.N * NQ), ng((size_t)F.N * NQ);
        if (e == cudaSuccess) {
            launch_interp_level(F.plan, C.plan, cf, d_if, ctx->s);
            launch_interp_level(F.plan, C.plan, cg, d_ig, ctx->s);
            ctx->launches += 2;
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(nf.data(), d_if, nf.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ng.data(), d_ig, ng.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->s);
        cudaFree(d_if);
        cudaFree(d_ig);
        if (e != cudaSuccess) return fail(ctx, MBG_ECUDA, std::string("mbg_regrid: ") + cudaGetErrorString(e));
        // cells an old box held keep their values; solid cells start at 0
        // (fill_f_inside_eb, Source/LBM.cpp:1278-1298)
        const Old* O = m < (int)old.size() ? &old[m] : nullptr;
        long long off = 0, goff = 0;
        for (size_t n = 0; n < F.boxes.size(); ++n) {
            const HBox& b = F.boxes[n];
            const long long v = b.vol();
            long long c = 0;
            for (int k = b.lo[2]; k <= b.hi[2]; ++k)
                for (int j = b.lo[1]; j <= b.hi[1]; ++j)
                    for (int i = b.lo[0]; i <= b.hi[0]; ++i, ++c) {
                        const uint8_t fl = flags[foff + goff + ((long long)(k - b.lo[2] + 3) * (b.n(1) + 6) +
                                                                (j - b.lo[1] + 3)) * (b.n(0) + 6) + (i - b.lo[0] + 3)];
                        if (!(fl & FL_FLUID)) {
                            for (int q = 0; q < NQ; ++q) nf[off * NQ + q * v + c] = ng[off * NQ + q * v + c] = 0.0;
                            continue;
                        }
                        if (!O) continue;
                        for (size_t ob = 0; ob < O->boxes.size(); ++ob) {
                            const HBox& B = O->boxes[ob];
                            if (i < B.lo[0] || i > B.hi[0] || j < B.lo[1] || j > B.hi[1] || k < B.lo[2] || k > B.hi[2])
                                continue;
                            const long long ov = B.vol();
                            const long long oc = ((long long)(k - B.lo[2]) * B.n(1) + (j - B.lo[1])) * B.n(0) + (i - B.lo[0]);
                            for (int q = 0; q < NQ; ++q) {
                                nf[off * NQ + q * v + c] = O->f[O->off[ob] * NQ + q * ov + oc];
                                ng[off * NQ + q * v + c] = O->g[O->off[ob] * NQ + q * ov + oc];
                            }
                            break;
                        }
                    }
            off += v;
            goff += b.gvol();
        }
        if ((st = mbg_set_state(ctx, lev, nf.data(), ng.data())) != MBG_OK) return st;
        boff += nbox[m];
        foff += goff;
    }
    return MBG_OK;
}

mbg_status mbg_get_derived(mbg_ctx* ctx, int lev, double* derived)
{
    if (!ctx || !derived) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)ctx->lv.size()) return fail(ctx, MBG_ESTATE, "mbg_get_derived: level not defined");
    Level& L = ctx->lv[lev];
    const size_t need = (size_t)L.N * 19;
    if (ctx->out19_n < need) {
        mbg_status st = dalloc(ctx, &ctx->d_out19, need);
        if (st != MBG_OK) return st;
        ctx->out19_n = need;
    }
    const double *f, *g, *fg, *gg;
    mbg_status st = fp64_state(ctx, L, true, &f, &g, &fg, &gg);
    if (st != MBG_OK) return st;
    launch_derived(L.plan, phys64(ctx, L), f, g, fg, gg, ctx->d_out19, ctx->s);
    ctx->launches++;
    MBG_CUDA(cudaGetLastError());
    MBG_CUDA(cudaMemcpyAsync(derived, ctx->d_out19, (size_t)L.N * 7 * sizeof(double), cudaMemcpyDeviceToHost,
                             ctx->s));
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    return MBG_OK;
}

mbg_status mbg_conserved(mbg_ctx* ctx, double out[5])
{
    if (!ctx || !out) return MBG_EINVAL;
    if (ctx->lv.empty()) return fail(ctx, MBG_ESTATE, "mbg_conserved: no level defined");
    MBG_CUDA(cudaMemsetAsync(ctx->d_red, 0, 5 * sizeof(double), ctx->s));
    for (auto& L : ctx->lv) {
        const double dV = L.dx[0] * L.dx[1] * L.dx[2];
        if (ctx->p.precision != MBG_FP64) lowp_conserved(L.lowp, L.plan, dV, ctx->d_red, ctx->s);
        else launch_conserved(L.plan, phys64(ctx, L), L.f[L.cur], L.g[L.cur], dV, ctx->d_red, ctx->s);
        ctx->launches++;
    }
    MBG_CUDA(cudaGetLastError());
    MBG_CUDA(cudaMemcpyAsync(out, ctx->d_red, 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->s));
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    return MBG_OK;
}

void* mbg_stream(const mbg_ctx* ctx) { return ctx ? (void*)ctx->s : nullptr; }

mbg_status mbg_set_timing(mbg_ctx* ctx, int enable)
{
    if (!ctx) return MBG_EINVAL;
    drain_events(ctx);
    ctx->timing = enable != 0;
    for (int k = 0; k < TK_N; ++k) { ctx->tk_count[k] = 0; ctx->tk_ms[k] = 0.0; }
    return MBG_OK;
}

int mbg_timing_count(void) { return TK_N; }

mbg_status mbg_timing(mbg_ctx* ctx, int k, const char** name, long long* launches, double* ms)
{
    if (!ctx || k < 0 || k >= TK_N) return MBG_EINVAL;
    drain_events(ctx);
    if (name) *name = TK_NAMES[k];
    if (launches) *launches = ctx->tk_count[k];
    if (ms) *ms = ctx->tk_ms[k];
    return MBG_OK;
}

mbg_status mbg_synchronize(mbg_ctx* ctx)
{
    if (!ctx) return MBG_EINVAL;
    MBG_CUDA(cudaStreamSynchronize(ctx->s));
    MBG_CUDA(cudaGetLastError());
    return MBG_OK;
}

}  // extern "C"
