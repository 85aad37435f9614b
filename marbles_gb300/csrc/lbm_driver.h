// lbm_driver.h -- host-side drop-in for the reference's LBM/AmrCore driver
// (Source/LBM.H, Source/LBM.cpp) on top of the C ABI: inputs parsing with
// the reference's keys, the IC and velocity-BC factories, embedded-boundary
// flags, static AMR box generation, init_data / evolve and plotfile output.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "../../include/marbles_gb300.h"
#include "mbg_geometry.cuh"

namespace mbgdrv {

// ParmParse-compatible inputs: "key = v1 v2 ..." lines, '#' comments,
// quoted strings; a later definition of a key overrides an earlier one and
// command-line "key=value" arguments override the file.
class Inputs {
public:
    bool parse_text(const std::string& text, std::string& err);
    bool parse_override(const std::string& kv, std::string& err);
    bool contains(const std::string& key) const { return kv_.count(key) != 0; }
    const std::vector<std::string>* values(const std::string& key) const;
    bool query(const std::string& key, int& v) const;
    bool query(const std::string& key, double& v) const;
    bool query(const std::string& key, std::string& v) const;
    bool query(const std::string& key, bool& v) const;
    bool queryarr(const std::string& key, std::vector<int>& v) const;
    bool queryarr(const std::string& key, std::vector<double>& v) const;
    bool queryarr(const std::string& key, std::vector<std::string>& v) const;

private:
    std::map<std::string, std::vector<std::string>> kv_;
    static bool tokenize(const std::string& line, std::vector<std::string>& out);
};

struct Box {
    int lo[3], hi[3];
    int n(int d) const { return hi[d] - lo[d] + 1; }
    long long vol() const { return (long long)n(0) * n(1) * n(2); }
};

// chop a box into pieces no longer than mgs, AMReX BoxList::maxSize style
std::vector<Box> chop_max_size(const Box& b, int mgs);

struct Config {
    // top level
    int max_step = 2147483647;
    double stop_time = 1.7976931348623157e308;
    // amr.*
    int n_cell[3] = {0, 0, 0};
    int max_level = 0;
    int max_grid_size = 32;
    int blocking_factor = 8;
    int n_error_buf = 1;
    int regrid_int = 2;
    int plot_int = -1, chk_int = -1;
    std::string plot_file = "plt", chk_file = "chk";
    std::string restart;   // amr.restart: checkpoint directory to resume from
    int file_name_digits = 5;
    // geometry.*
    double prob_lo[3] = {0, 0, 0}, prob_hi[3] = {1, 1, 1};
    int is_periodic[3] = {0, 0, 0};
    // lbm.*
    int bc_lo[3] = {0, 0, 0}, bc_hi[3] = {0, 0, 0};
    std::string velocity_bc_type = "noop";
    std::string ic_type;
    double dx_outer = 1.0, dt_outer = 1.0, nu = 1.0, alpha = 1.0;
    bool save_streaming = true, save_derived = true, compute_forces = false;
    std::string forces_file = "forces.txt";
    double initial_temperature = 1.0 / 3.0, adiabatic_exponent = 5.0 / 3.0, m_bar = 28.96;
    // eb2.* (and extruded_triangles.*)
    std::string geom_type = "all_regular";
    mbg_geometry geom{};
    // tagging.*
    struct Tag {
        std::string name;
        bool has_box = false;
        double box_lo[3], box_hi[3];
        std::string field;
        int field_index = 19;  // macro component 0..18 (mbg_get_macro order) or 19 = is_fluid
        int kind = 0;  // 0 box only, 1 value_greater, 2 value_less
        double value = 0.0;
        int max_level = 1000;
        double start_time = -1.0e300, end_time = 1.0e300;
    };
    std::vector<Tag> tags;
    // the form of the populations
    int precision = MBG_FP64;
};

// initial-condition functor parameters (Source/IC.H, Source/IC.cpp)
struct ICParams {
    int type = 0;  // 0 constant, 1 taylorgreen, 2 viscosity_test, 3 thermaldiffusivity_test, 4 sod,
                   // 5 gaussian_pulse, 6 temperature_field
    double density = 1.0, velocity[3] = {0, 0, 0}, mach[3] = {0, 0, 0};
    double initial_temperature = 1.0 / 3.0, adiabatic_exponent = 5.0 / 3.0, m_bar = 28.96;
    double wave_length = 1.0;
    double rho0 = 1.0, v0 = 1.0, omega[3] = {1, 1, 1};
    double density_ratio = 1.0, temperature_ratio = 1.0, x_discontinuity = 10.0;
    double amplitude = 0.01, width = 8.0, center[3] = {0, 0, 0};
    std::vector<double> tfield;  // temperature_field: level-0 cell values
    double sos = 0.0;            // speed_of_sound_ref
};

// velocity-BC functor parameters (Source/VelocityBC.H, VelocityBC.cpp)
struct VelBC {
    int type = 0;
    int dir = 1, normal_dir = 0, tangential_dir = 1;
    double mach_ref = 0.005, initial_density = 1.0, initial_temperature = 1.0 / 3.0;
    double adiabatic_exponent = 5.0 / 3.0, m_bar = 28.96;
    double u_ref = 0.0;
};

class LBM {
public:
    ~LBM();
    bool configure(const Inputs& in, std::string& err);
    mbg_status prepare();               // grids and flags, host only
    mbg_status init_data();
    mbg_status evolve(int nsteps);      // nsteps <= 0: run to max_step / stop_time
    mbg_status write_plot_file(const std::string& name);
    mbg_status write_checkpoint(const std::string& name);
    // ErrorEst on the GPU, new grids from the tags, RemakeLevel of levels >= 1
    // (Source/LBM.cpp:452-521 regrid branch); no-op when the grids do not change
    mbg_status regrid();
    mbg_ctx* context() { return ctx_; }
    const Config& config() const { return cfg_; }
    const std::vector<std::vector<Box>>& grids() const { return grids_; }
    const std::vector<std::vector<uint8_t>>& flags() const { return flags_; }
    int step() const { return step_; }
    double time() const { return time_; }
    std::string err;
    std::vector<double> last_forces{0.0, 0.0, 0.0};

    // host IC of one level (valid cells, [box][q][k][j][i])
    void initial_state(int lev, std::vector<double>& f, std::vector<double>& g) const;

private:
    Config cfg_;
    mbg::GeomDesc geom_;   // implicit function of cfg_.geom (host evaluation)
    ICParams ic_;
    VelBC vbc_;
    mbg_ctx* ctx_ = nullptr;
    std::vector<std::vector<Box>> grids_;
    std::vector<std::vector<uint8_t>> flags_;
    int step_ = 0;
    double time_ = 0.0;
    int last_plot_step_ = -1;
    int last_regrid_step_ = 0;
    bool prepared_ = false;
    mbg_params params_{};

    mbg_status build_context();
    bool has_field_tags() const;
    // per level below max_level that exists: the tags of every cell of the
    // level's index space (x fastest), 0 outside the level's boxes
    mbg_status gpu_tags(std::vector<std::vector<uint8_t>>& dense);
    mbg_status level_flags_gpu(int lev, std::vector<uint8_t>& out);

    mbg_status read_checkpoint();
    std::string numbered(const std::string& root) const;

    void level_geometry(int lev, double dx[3]) const;
    bool covered_cell(int lev, int i, int j, int k) const;
    void make_flags(int lev);
    bool make_grids(std::string& e, const std::vector<std::vector<uint8_t>>* dense = nullptr);
    void ic_state(int lev, int i, int j, int k, double& rho, double vel[3], double& t, double& Rg,
                  double& gamma) const;
    void write_forces(bool init);
};

}  // namespace mbgdrv
