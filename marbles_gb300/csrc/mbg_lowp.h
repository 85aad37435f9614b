// mbg_lowp.h -- FP32-arithmetic / 16-bit shifted-storage form of the level
// step (mbg_lowp.cu).
#pragma once

#include <string>
#include <vector>

#include "../../include/marbles_gb300.h"
#include "mbg_kernels.h"

namespace mbg {

struct LowpLevel {
    int precision = 0;           // MBG_FP32C_F16S or MBG_FP32C_BF16S
    long long N = 0, NG = 0;
    void* f[2] = {nullptr, nullptr};    // 16-bit populations, [q][N]
    void* g[2] = {nullptr, nullptr};
    void* fg[2] = {nullptr, nullptr};   // ghost fabs, [q][NG]
    void* gg[2] = {nullptr, nullptr};
    float* qc = nullptr;                // Q_corr scratch of the two-pass kernels
    float* gqc = nullptr;
    double* tmp = nullptr;              // FP64 staging for state transfer
    int cur = 0;
    Phys32 ph;
    std::vector<void*> allocs;
};

mbg_status lowp_define(const mbg_params& p, const LevelPlan& plan, const std::vector<DevBox>& hbox, long long N,
                       long long NG, LowpLevel& L, std::string& err);
mbg_status lowp_set_state(LowpLevel& L, const LevelPlan& plan, const std::vector<DevBox>& hbox, const double* f,
                          const double* g, cudaStream_t s, std::string& err);
mbg_status lowp_get_state(LowpLevel& L, const LevelPlan& plan, const std::vector<DevBox>& hbox, double* f,
                          double* g, cudaStream_t s, std::string& err);
mbg_status lowp_macro(LowpLevel& L, const LevelPlan& plan, double* out19, cudaStream_t s, std::string& err);
// returns the number of kernels launched
int lowp_advance(const mbg_params& p, const BCParams& bc, LowpLevel& L, const LevelPlan& plan, double dt,
                 const double idx[3], const CoalesceCell* coal, long long ncoal, const LowpLevel* fine,
                 const LevelPlan* fplan, cudaStream_t s);
void lowp_explode(LowpLevel& F, const LevelPlan& fplan, const LowpLevel& C, const LevelPlan& cplan, cudaStream_t s);
void lowp_average_down(LowpLevel& C, const LevelPlan& cplan, const LowpLevel& F, const LevelPlan& fplan,
                       const CoalesceCell* list, long long n, cudaStream_t s);

}  // namespace mbg
