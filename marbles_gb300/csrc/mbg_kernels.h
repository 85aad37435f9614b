// mbg_kernels.h -- plan structures shared by the host orchestration
// (mbg_capi.cu) and the kernel files, and the launcher declarations.
#pragma once

#include <cuda_runtime.h>

#include "../../include/marbles_gb300.h"
#include "mbg_level.cuh"

namespace mbg {

constexpr int TILE_CELLS = 128;   // cells (threads) per CTA in the per-cell passes

// scratch macro-field components of the FP64 form
enum {
    MD_RHO = 0, MD_U, MD_V, MD_W, MD_TRE, MD_PXX, MD_PYY, MD_PZZ, MD_PXY, MD_PXZ, MD_PYZ,
    MD_QX, MD_QY, MD_QZ, MD_T, MD_QCX, MD_QCY, MD_QCZ, MD_NCOMP
};

enum : uint8_t { FL_COV = 8 };   // covered by a finer level (EB force mask)

struct Tile {
    int box;
    int start;   // first cell (linear index inside the box)
};

struct GhostCell {
    int box;
    short x, y, z;   // box-local position in the grown fab (-3 .. n+2)
    short layer;     // Chebyshev distance to the box
};

// a coarse cell under a fine level's uncovered ghost shell (global coarse
// coordinates): the explosion computes its slopes and limiter once
struct XSlot {
    int x, y, z, pad;
};

struct CoalesceCell {
    int cbox;             // coarse box holding the cell
    int fbox;             // fine box whose average is kept (last writer)
    short cx, cy, cz;     // coarse box-local position
    short fx, fy, fz;     // first child, fine box-local position
};

struct Phys64 {
    double mesh_speed, Rg, cv, nu, alpha, dt;
    double idx[3];
    double small_num;
    Lattice<double> lat;
};

struct Phys32 {
    float mesh_speed, Rg, cv, nu, alpha, dt;
    float idx[3];
    float small_num;
    Lattice<float> lat;
    float frest[NQ], grest[NQ];   // rest-state equilibria (shift of the storage)
    float fscale, gscale;         // storage = (value - rest) / scale
    float inv_fscale, inv_gscale;
};

// One chunk of a box's neighbourhood.  Along each axis the box grown by one
// cell is cut into the layer below the box (chunk 0), runs of 2^lg cells of
// the box (chunks 1 .. nch) and the layer above (chunk nch + 1); a box's
// table holds one slot per chunk triple, index cx + tx (cy + ty cz) with
// t = nch + 2.  A slot gives the storage of its cells as an affine map of
// box-local positions, index = base + z sz + y sy + x, into the valid cells
// of the level (stride N) or into the box's own ghost fab (stride NG).  With
// 2^lg the largest power of two (at most 32) dividing every box corner and
// length of the level, each chunk lies in one box or in none, so AMR levels
// of uneven boxes on a blocking factor get tables too.
struct NbrSlot {
    long long base;
    int sy, sz;
    int ghost;   // 0: valid cells, 1: the box's ghost fab, 2: beyond a non-periodic side (step tables)
    int pad;
};
constexpr int SLOT_TABLE_MAX = 1024;   // slots of one box's table (24 KB of shared memory)

struct LevelPlan {
    LevelView<double> view64;
    const Tile* tiles = nullptr;
    int ntiles = 0;
    // FP64 form: the tiles of boxes whose neighbour chunks each map to one
    // box (or to the box's ghost fab), with no solid cell in the grown box and
    // no non-periodic domain side within one cell -- their pulls go through
    // the slot tables above -- and the tiles of the other boxes (general pull)
    const NbrSlot* slots = nullptr;      // the boxes' tables, one after another
    const int* slot_off = nullptr;       // [box]: first slot of the box's table (-1: none)
    int slot_lg[3] = {0, 0, 0};          // log2 of the chunk length along each axis
    int slot_max = 0;                    // largest table of a box on the slot lists
    const Tile* fast_tiles = nullptr;
    int nfast = 0;
    const Tile* fasteb_tiles = nullptr;   // the same for boxes holding solid cells
    int nfasteb = 0;
    // the same two for boxes within one cell of a non-periodic side, whose
    // tables mark the chunks beyond it (ghost = 2: the BC's values)
    const Tile* fastbc_tiles = nullptr;
    int nfastbc = 0;
    const Tile* fastebbc_tiles = nullptr;
    int nfastebbc = 0;
    const Tile* gen_tiles = nullptr;
    int ngen = 0;
    const GhostCell* ghost_list = nullptr;   // all uncovered ghost cells
    long long nghost_cells = 0;
    // FP64 ghost stream: ghost-shell slot tables (chunks 3 cells wide at the
    // box faces, the step tables' grain inside), the ghost cells that pull
    // through them and the others
    const NbrSlot* gslots = nullptr;
    const int* gslot_off = nullptr;
    const GhostCell* ghost_fast = nullptr;
    long long nghost_fast = 0;
    const GhostCell* ghost_gen = nullptr;
    long long nghost_gen = 0;
    const GhostCell* ghost_list1 = nullptr;  // first ghost layer only
    long long nghost1 = 0;
    // FP64 explosion: each ghost cell's slot, the slots' coarse cells, and per
    // slot the 7 coarse storage indices [7][nx], value and centred slopes
    // [lattice][4][NQ][nx], limiter [lattice][3][nx]
    const int* xslot = nullptr;
    const XSlot* xc = nullptr;
    long long nx = 0;
    int* xix = nullptr;
    double* xs = nullptr;
    double* xal = nullptr;
};

// FP64 form (mbg_fp64.cu)
void launch_moments(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                    const double* fAg, const double* gAg, const double* fB, const double* gB, double* md,
                    cudaStream_t s);
void launch_collide(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                    const double* fAg, const double* gAg, double* fB, double* gB, const double* md,
                    const double* gqc, cudaStream_t s);
// the step kernels of modes 3-4 (mbg_fp64_bc.cu, mbg_fp64_bcc.cu) and 0
// (mbg_fp64_gen.cu), called by launch_moments / launch_collide
void launch_moments_bc(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                       const double* fAg, const double* gAg, const double* fB, const double* gB, double* md,
                       cudaStream_t s);
void launch_collide_bc(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                       const double* fAg, const double* gAg, double* fB, double* gB, const double* md,
                       const double* gqc, cudaStream_t s);
void launch_moments_gen(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                        const double* fAg, const double* gAg, const double* fB, const double* gB, double* md,
                        cudaStream_t s);
void launch_collide_gen(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA, const double* gA,
                        const double* fAg, const double* gAg, double* fB, double* gB, const double* md,
                        const double* gqc, cudaStream_t s);
// the refinement criteria of one mbg_tag_cells call
struct TagSet {
    int n = 0;
    mbg_tag t[MBG_MAX_TAGS];
};
// ErrorEst tags of a level's valid cells into out ([box][cell], 0/1): field
// values from md (the FP64 macro scratch of the last collision) when given,
// else from the moments of the stored state f, g (FP64 layout)
void launch_tags(const LevelPlan& lp, const Phys64& ph, const double* md, const double* f, const double* g,
                 const TagSet& ts, double time, int lev, const double plo[3], const double dx[3], uint8_t* out,
                 cudaStream_t s);
// conservative linear interpolation (cell_cons_interp) of every valid cell
// of a fine level from the coarse level's stored values c (FP64 layout of
// the coarse plan), one lattice, into out in host layout [box][q][cell]
void launch_interp_level(const LevelPlan& fine, const LevelPlan& crse, const double* c, double* out,
                         cudaStream_t s);
// kernel launches of one launch_moments or launch_collide call
int fp64_step_launches(const LevelPlan& lp);
// kernel launches of one launch_ghost_stream call
int ghost_stream_launches(const LevelPlan& lp);
void launch_ghost_stream(const LevelPlan& lp, const BCParams& P, const Phys64& ph, const double* fA,
                         const double* gA, const double* fAg, const double* gAg, double* fBg, double* gBg,
                         cudaStream_t s);
// Q_corr of the first-layer ghost cells from the ghost fab that
// launch_ghost_stream has just written (fBg, gBg)
void launch_ghost_moments(const LevelPlan& lp, const Phys64& ph, const double* fBg, const double* gBg, double* gqc,
                          cudaStream_t s);
void launch_explode(const LevelPlan& fine, const LevelPlan& crse, const double* fc, const double* gc, double* fg,
                    double* gg, cudaStream_t s);
void launch_coalesce(const LevelPlan& crse, const LevelPlan& fine, const BCParams& P, const Phys64& ph,
                     const CoalesceCell* list, long long n, const double* ff, const double* gf, const double* ffg,
                     const double* gfg, const double* fcA, const double* gcA, const double* fcAg,
                     const double* gcAg, double* fcB, double* gcB, int into_state, cudaStream_t s);
// NaN and sentinel scan of a level's FP64 (or decoded) state into out[0..2]
// (counts at fluid and at solid cells, key of the first bad value)
void launch_check(const LevelPlan& lp, const double* f, const double* g, int lev, unsigned long long* out,
                  cudaStream_t s);
// host layout [box][q][cell] (stage) <-> FP64 state v [q][N], to_state: into v
void launch_stage(const LevelPlan& lp, double* stage, double* v, int to_state, cudaStream_t s);
void launch_macro_local(const LevelPlan& lp, const Phys64& ph, const double* f, const double* g, double* out19,
                        cudaStream_t s);
// per-block partial force sums (3 per tile) of one level; launch_sum_partials
// adds n partials in a fixed order into out3
void launch_eb_forces(const LevelPlan& lp, const double* f, const double* fg, double* partial3, cudaStream_t s);
void launch_sum_partials(const double* partial3, long long n, double* out3, cudaStream_t s);
// vorticity and q-correction gradients of the stored state, [box][7][cell]
void launch_derived(const LevelPlan& lp, const Phys64& ph, const double* f, const double* g, const double* fg,
                    const double* gg, double* out7, cudaStream_t s);
void launch_conserved(const LevelPlan& lp, const Phys64& ph, const double* f, const double* g, double dV, double* out5,
                      cudaStream_t s);

}  // namespace mbg
