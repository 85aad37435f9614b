// mbg_lowp.h -- FP32-arithmetic / 16-bit shifted-storage form of the level
// step (mbg_lowp.cu).
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "../../include/marbles_gb300.h"
#include "mbg_kernels.h"

namespace mbg {

struct LowpLevel {
    int precision = 0;           // MBG_FP32C_F16S or MBG_FP32C_BF16S
    long long N = 0, NG = 0;            // storage cells (valid + one-cell pad per box), ghost-fab cells
    long long NV = 0;                   // valid cells
    void* f[2] = {nullptr, nullptr};    // 16-bit populations, [q][N]
    void* g[2] = {nullptr, nullptr};
    void* fg[2] = {nullptr, nullptr};   // ghost fabs, [q][NG]
    void* gg[2] = {nullptr, nullptr};
    double* tmp = nullptr;              // FP64 staging for state transfer, [q][NV]
    int cur = 0;
    Phys32 ph;
    void* impl = nullptr;               // codecs, tiles, override buffers (mbg_lowp.cu)
    std::vector<void*> allocs;
};

// host copy of a level's geometry, for the plans built at definition time
struct LevelHost {
    const std::vector<uint8_t>* flags;   // one byte per cell of each box grown by 3
    const std::vector<int>* omap;        // owner of each G^3 bin, or -1
    const std::vector<GhostCell>* ghosts;   // uncovered ghost cells (fine levels)
    int dlo[3], dhi[3], G[3], nb[3], per[3];
};

// the explosion's slots: the distinct coarse cells under a fine level's
// uncovered ghost cells, numbered in order of first use, and each ghost cell's
// slot (shared by both forms)
void explode_plan(const std::vector<DevBox>& box, const std::vector<GhostCell>& ghosts, const LevelHost& h,
                  std::vector<XSlot>& xc, std::vector<int>& slot);
mbg_status lowp_define(const mbg_params& p, const LevelPlan& plan, const std::vector<DevBox>& hbox, long long N,
                       long long NG, double dt, const double idx[3], const LevelHost& host, LowpLevel& L,
                       std::string& err);
void lowp_release(LowpLevel& L);
// rebuild the step's tile lists after the level's FL_OVR flags changed
void lowp_retile(LowpLevel& L, const std::vector<uint8_t>& flags, cudaStream_t s);
mbg_status lowp_set_state(LowpLevel& L, const LevelPlan& plan, const std::vector<DevBox>& hbox, const double* f,
                          const double* g, cudaStream_t s, std::string& err);
mbg_status lowp_get_state(LowpLevel& L, const LevelPlan& plan, const std::vector<DevBox>& hbox, double* f,
                          double* g, cudaStream_t s, std::string& err);
// the stored populations of lattice lat (0: f, 1: g) decoded to FP64 into
// dst, [q][NV] in the FP64 form's valid-cell layout (the plan's view64)
void lowp_decode(LowpLevel& L, const LevelPlan& plan, int lat, double* dst, cudaStream_t s);
// the ghost fabs of lattice lat decoded to FP64 into dst, [q][NG] (fine levels)
void lowp_decode_ghost(LowpLevel& L, const LevelPlan& plan, int lat, double* dst, cudaStream_t s);
mbg_status lowp_macro(LowpLevel& L, const LevelPlan& plan, double* out19, cudaStream_t s, std::string& err);
// adds the level's conserved totals (FP64) to out5 on the device
void lowp_conserved(LowpLevel& L, const LevelPlan& plan, double dV, double* out5, cudaStream_t s);
// Stages of one 16-bit level advance, each one kernel launch; the caller's
// runner wraps every launch (the library times them with CUDA events).
enum { LOWP_STAGE_COALESCE = 0, LOWP_STAGE_GHOST_STREAM, LOWP_STAGE_FUSED, LOWP_STAGE_HALO };
using LowpRunner = std::function<void(int stage, const std::function<void()>& launch)>;
// returns the number of kernels launched
int lowp_advance(const mbg_params& p, const BCParams& bc, LowpLevel& L, const LevelPlan& plan, double dt,
                 const double idx[3], const CoalesceCell* coal, long long ncoal, const LowpLevel* fine,
                 const LevelPlan* fplan, cudaStream_t s, const LowpRunner& run);
// step variants (0: two-pass, 1..2: fused with 4- or 8-plane runs, 3:
// two-pass with a tighter register cap) and the tuner that times them on the
// level's data and keeps the fastest
int lowp_variants();
mbg_status lowp_autotune(LowpLevel& L, const LevelPlan& plan, const BCParams& bc, const CoalesceCell* coal,
                         long long ncoal, const LowpLevel* fine, const LevelPlan* fplan, int reps, cudaStream_t s,
                         std::string& err);
void lowp_variant(LowpLevel& L, int* variant, double ms[4]);
void lowp_set_variant(LowpLevel& L, int variant);
// returns the number of kernels launched
int lowp_explode(LowpLevel& F, const LevelPlan& fplan, const LowpLevel& C, const LevelPlan& cplan, cudaStream_t s);
void lowp_average_down(LowpLevel& C, const LevelPlan& cplan, const LowpLevel& F, const LevelPlan& fplan,
                       const CoalesceCell* list, long long n, cudaStream_t s);

}  // namespace mbg
