// mbg_lowp_types.cuh -- types shared by the host code of the 16-bit form
// (mbg_lowp.cu) and its kernels (mbg_lowp_kern.cuh, compiled once per storage
// format in mbg_lowp_f16.cu and mbg_lowp_bf16.cu).
#pragma once

#include "mbg_lowp.h"

namespace mbg {

using u16 = uint16_t;
using LV16 = LevelView<u16>;

constexpr u16 SENT16 = 0xFFFFu;
// override code of a (coarse cell, direction) whose eight fine children were
// all masked: the step takes the cell's own streamed value (a NaN pattern the
// encoder never produces)
constexpr u16 NOOVR16 = 0xFFFDu;
constexpr int FT_THREADS = 256;   // threads of a fused-step CTA
constexpr int FT_QX = 320;        // shared Q_corr rows: max over tw of th * (tw + 2)
constexpr int FT_QY = 320;        // max over tw of (th + 2) * tw

struct CodecTab {
    float frest[NQ], grest[NQ], fsc[NQ], gsc[NQ], fisc[NQ], gisc[NQ];
};

struct Bufs16 {
    const u16 *f, *g, *fg, *gg;   // source state (valid, ghost)
    const u16 *fo, *go;           // coalescence override (coarse levels), or null
};

// everything the kernels of one level read, for one buffer parity
struct LowpK {
    LV16 L;
    BCParams P;
    Phys32 ph;
    CodecTab ct;
    Lattice<double> lat64;
    Bufs16 s;                      // source: the current state
    u16 *fA, *gA;                  // the source again, writable (its pad is filled in place)
    u16 *fB, *gB, *fBg, *gBg;      // destination: the other buffer
    const Phys32* phys;            // per-box parameters (batched domains), or null: ph for all boxes
    // per valid cell of boxes holding solid cells, at the cell's storage
    // index: bit q (0 .. 26) set where the fluid cell's source x - e_q is
    // solid, bit NMASK_FLUID where the cell is fluid (null: no such boxes)
    const unsigned* nmask;
};
constexpr int NMASK_FLUID = 27;

// one cell of a box's pad: box-local coordinates, each -1 .. n
struct HaloCell {
    int box;
    short x, y, z, pad;
};

// pad fill of one pad cell: for each direction q in qmask, component q of
// storage index dst takes component q of src (a valid cell, or the ghost fab
// index -src - 1)
struct HaloCopy {
    long long dst;
    long long src;
    unsigned qmask;
    unsigned pad;
};

// explosion plan of a fine level: the distinct coarse cells under its
// uncovered ghost cells (XSlot), each ghost cell's slot among them, and
// per-slot scratch: the 7 coarse neighbours' storage indices [7][nx], value
// and centred slopes [lattice][4][NQ][nx], limiter [lattice][3][nx]
struct ExplodePlan {
    const GhostCell* gl;
    const int* slot;
    long long n;
    const XSlot* xc;
    int* ix;
    float* xs;
    float* al;
    long long nx;
};

// Q_corr of the pad face cells that gradients read (inside the domain box,
// fluid): copies from the valid cell of the owning box (qs indices d N + i),
// and the pad cells on the coarse-fine shell, whose Q_corr is the moments of
// the box's ghost fab (k_qhalo16)
struct QPad {
    const long long* dst = nullptr;
    const long long* src = nullptr;
    long long ncopy = 0;
    const HaloCell* ghost = nullptr;
    long long nghost = 0;
};

// the device pair tile lists of a step (StepTiles)
struct PairLists {
    const Tile* pair = nullptr;
    int npair = 0;
    const Tile* pair_ovr = nullptr;
    int npair_ovr = 0;
    const Tile* pair_eb = nullptr;
    int npair_eb = 0;
};

struct FusedTile {
    int box;
    short x0, y0, z0, z1;
    short lgw;   // log2 of the tile width in x (3, 4 or 5)
    short pad;
};

// host helpers of the layout (mbg_lowp.cu), shared with the batched domains
// (mbg_batch.cu)
// step variants: 0 two-pass (cell pairs where the box allows), 1 and 2
// fused with runs of FUSED_ZC[v - 1] planes, 3 two-pass one cell per thread
// with the collision pass capped at 80 registers
constexpr int FUSED_ZC[2] = {4, 8};
CodecTab make_codec(const mbg_params& p);
Phys32 phys32(const mbg_params& p, double dt, const double idx[3]);
long long pad_boxes(std::vector<DevBox>& box);
std::vector<HaloCell> halo_cells(const std::vector<DevBox>& box);
std::vector<FusedTile> fused_tiles(const std::vector<DevBox>& box, int zc);
// the step's tile lists: pair tiles (PAIR_CELLS cells, two per thread) of
// boxes with an even x extent whose cells one layer out are all fluid --
// those without and those with a cell overwritten by coalescence (FL_OVR in
// flags, the grown flag fabs of the boxes) -- and per-cell tiles
// (TILE_CELLS) of the other boxes
constexpr int PAIR_CELLS = 2 * TILE_CELLS;
struct StepTiles {
    std::vector<Tile> pair;       // pair tiles of boxes fluid one cell out
    std::vector<Tile> pair_ovr;   // the same holding cells overwritten by coalescence
    std::vector<Tile> pair_eb;    // pair tiles of boxes holding solid cells (no overwritten cell)
    std::vector<Tile> cell;       // per-cell tiles of the rest
};
StepTiles step_tiles(const std::vector<DevBox>& box, const std::vector<uint8_t>* flags);

// per-direction base pointers of the source and destination arrays of one
// step (kernel parameters, so each population access is one 32-bit offset
// from a constant-bank operand)
struct QPtrs {
    const u16* f[NQ];
    const u16* g[NQ];
    u16* fo[NQ];
    u16* go[NQ];
};

inline QPtrs make_qptrs(const void* f, const void* g, void* fo, void* go, long long N)
{
    QPtrs p;
    for (int q = 0; q < NQ; ++q) {
        p.f[q] = (const u16*)f + q * N;
        p.g[q] = (const u16*)g + q * N;
        p.fo[q] = (u16*)fo + q * N;
        p.go[q] = (u16*)go + q * N;
    }
    return p;
}

// kernel launchers, instantiated for FP16 (BF = false) and BF16 (BF = true)
template <bool BF>
struct Lowp16 {
    static void halo(const LowpK* k, const HaloCell* h, long long n, cudaStream_t s);
    static void halo_copy(const LowpK* k, const HaloCopy* hc, long long n, cudaStream_t s);
    static void halo_periodic(const LowpK* k, const HaloCell* h, long long n, cudaStream_t s);
    static void fused(const LowpK* k, const CodecTab& ct, const Lattice<float>& lat, const FusedTile* t, int ntiles,
                      int grid, cudaStream_t s);
    static int fused_blocks_per_sm();   // resident CTAs of the fused step per SM
    // the two-pass step: Q_corr pass, pad of Q_corr, collision pass, over the
    // pair tiles (two cells per thread, 256 cells per tile; see StepTiles)
    // and the per-cell tiles; returns the launches made
    static int two_pass(const LowpK* k, const CodecTab& ct, const Lattice<float>& lat, const Tile* tiles,
                        int ntiles, const PairLists& pl, const QPad& qpad, float* qs, const QPtrs& qp, int tight,
                        cudaStream_t s);
    static void ghost_stream(const LowpK* k, const GhostCell* gl, long long n, cudaStream_t s);
    // the ghost stream through its plan: gather, then the general entries
    static void ghost_gather(const LowpK* k, const long long* dst, const long long* src, long long n,
                             const GhostCell* gl, const int* gcell, const int* gq, long long ngen, cudaStream_t s);
    // the ghost stream of the ghost cells of all-fluid boxes with a
    // ghost-shell slot table: a copy of the code each pull reads; at the pad
    // face cells inside the domain box also the Q_corr component normal to
    // the face, into qs (the step's Q_corr array)
    static void ghost_slots(const LowpK* k, const NbrSlot* T, const int* off, const int lg[3], const GhostCell* gl,
                            long long n, float* qs, cudaStream_t s);
    // explosion: coarse neighbours, slopes and limiter per coarse cell, then
    // the fine ghost cells (3 launches)
    static void explode(const LowpK* kf, const LowpK* kc, const ExplodePlan& xp, u16* fg, u16* gg, cudaStream_t s);
    static void coalesce(const LowpK* kc, const LowpK* kf, const CoalesceCell* cl, long long n, u16* fo, u16* go,
                         int into_state, cudaStream_t s);
    static void encode(const LowpK* k, const Tile* tiles, int ntiles, const double* src, long long NV, u16* dst,
                       int isg, cudaStream_t s);
    static void decode(const LowpK* k, const Tile* tiles, int ntiles, const u16* src, long long NV, double* dst,
                       int isg, cudaStream_t s);
    static void macro(const LowpK* k, const CodecTab& ct, const Tile* tiles, int ntiles, double* out19,
                      cudaStream_t s);
    static void conserved(const LowpK* k, const Tile* tiles, int ntiles, double dV, double* out5, cudaStream_t s);
    // every value of a [q][n] array (the ghost fabs) decoded to FP64
    static void decode_flat(const LowpK* k, const u16* src, long long n, double* dst, int isg, cudaStream_t s);
};
extern template struct Lowp16<false>;
extern template struct Lowp16<true>;

}  // namespace mbg
