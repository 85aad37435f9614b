// mbg_lowp.cu -- placeholder
#include "mbg_lowp.h"
namespace mbg {
mbg_status lowp_define(const mbg_params&, const LevelPlan&, const std::vector<DevBox>&, long long, long long,
                       LowpLevel&, std::string& err) { err = "16-bit form not built"; return MBG_EINVAL; }
mbg_status lowp_set_state(LowpLevel&, const LevelPlan&, const std::vector<DevBox>&, const double*, const double*,
                          cudaStream_t, std::string& err) { err = "16-bit form not built"; return MBG_EINVAL; }
mbg_status lowp_get_state(LowpLevel&, const LevelPlan&, const std::vector<DevBox>&, double*, double*,
                          cudaStream_t, std::string& err) { err = "16-bit form not built"; return MBG_EINVAL; }
mbg_status lowp_macro(LowpLevel&, const LevelPlan&, double*, cudaStream_t, std::string& err) { err = "x"; return MBG_EINVAL; }
int lowp_advance(const mbg_params&, const BCParams&, LowpLevel&, const LevelPlan&, double, const double*,
                 const CoalesceCell*, long long, const LowpLevel*, const LevelPlan*, cudaStream_t) { return 0; }
void lowp_explode(LowpLevel&, const LevelPlan&, const LowpLevel&, const LevelPlan&, cudaStream_t) {}
void lowp_average_down(LowpLevel&, const LevelPlan&, const LowpLevel&, const LevelPlan&, const CoalesceCell*,
                       long long, cudaStream_t) {}
}
