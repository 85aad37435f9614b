// lbm_driver.cu -- host drop-in for the reference's LBM driver (host code
// only; compiled by nvcc so that it shares mbg_physics.cuh with the
// kernels).  See lbm_driver.h.
#include <algorithm>
#include <cerrno>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <set>
#include <sstream>
#include <sys/stat.h>

#include "lbm_driver.h"
#include "mbg_geometry.cuh"
#include "mbg_physics.cuh"

namespace mbgdrv {

static const double R_U = 28.96;  // Source/Constants.H:66 (AIR_MOLAR_MASS)

// ---------------------------------------------------------------------------
// Inputs (ParmParse semantics, Docs/sphinx/InputFiles.rst)
// ---------------------------------------------------------------------------
bool Inputs::tokenize(const std::string& line, std::vector<std::string>& out)
{
    out.clear();
    size_t i = 0;
    while (i < line.size()) {
        const char c = line[i];
        if (c == '#') break;
        if (std::isspace((unsigned char)c)) { ++i; continue; }
        if (c == '"') {
            const size_t j = line.find('"', i + 1);
            if (j == std::string::npos) return false;
            out.push_back(line.substr(i + 1, j - i - 1));
            i = j + 1;
            continue;
        }
        size_t j = i;
        while (j < line.size() && !std::isspace((unsigned char)line[j]) && line[j] != '#' && line[j] != '"' &&
               line[j] != '=')
            ++j;
        if (j == i) {  // a lone '='
            out.push_back("=");
            i = j + 1;
            continue;
        }
        out.push_back(line.substr(i, j - i));
        i = j;
    }
    return true;
}

bool Inputs::parse_text(const std::string& text, std::string& err)
{
    std::istringstream is(text);
    std::string line;
    int ln = 0;
    while (std::getline(is, line)) {
        ++ln;
        std::vector<std::string> t;
        if (!tokenize(line, t)) {
            err = "inputs line " + std::to_string(ln) + ": unterminated quote";
            return false;
        }
        if (t.empty()) continue;
        if (t.size() < 2 || t[1] != "=") {
            err = "inputs line " + std::to_string(ln) + ": expected 'key = value'";
            return false;
        }
        kv_[t[0]] = std::vector<std::string>(t.begin() + 2, t.end());
    }
    return true;
}

bool Inputs::parse_override(const std::string& s, std::string& err)
{
    const size_t e = s.find('=');
    if (e == std::string::npos) {
        err = "override '" + s + "' is not key=value";
        return false;
    }
    std::string key = s.substr(0, e);
    key.erase(key.find_last_not_of(" \t") + 1);
    std::vector<std::string> t;
    if (!tokenize(s.substr(e + 1), t)) {
        err = "override '" + s + "': unterminated quote";
        return false;
    }
    kv_[key] = t;
    return true;
}

const std::vector<std::string>* Inputs::values(const std::string& key) const
{
    auto it = kv_.find(key);
    return it == kv_.end() ? nullptr : &it->second;
}

bool Inputs::query(const std::string& key, int& v) const
{
    auto* x = values(key);
    if (!x || x->empty()) return false;
    v = (int)std::stol((*x)[0]);
    return true;
}
bool Inputs::query(const std::string& key, double& v) const
{
    auto* x = values(key);
    if (!x || x->empty()) return false;
    v = std::stod((*x)[0]);
    return true;
}
bool Inputs::query(const std::string& key, std::string& v) const
{
    auto* x = values(key);
    if (!x || x->empty()) return false;
    v = (*x)[0];
    return true;
}
bool Inputs::query(const std::string& key, bool& v) const
{
    auto* x = values(key);
    if (!x || x->empty()) return false;
    const std::string& s = (*x)[0];
    v = !(s == "0" || s == "false" || s == "False" || s == "FALSE");
    return true;
}
bool Inputs::queryarr(const std::string& key, std::vector<int>& v) const
{
    auto* x = values(key);
    if (!x) return false;
    v.clear();
    for (auto& s : *x) v.push_back((int)std::stol(s));
    return true;
}
bool Inputs::queryarr(const std::string& key, std::vector<double>& v) const
{
    auto* x = values(key);
    if (!x) return false;
    v.clear();
    for (auto& s : *x) v.push_back(std::stod(s));
    return true;
}
bool Inputs::queryarr(const std::string& key, std::vector<std::string>& v) const
{
    auto* x = values(key);
    if (!x) return false;
    v = *x;
    return true;
}

// ---------------------------------------------------------------------------
// boxes
// ---------------------------------------------------------------------------
std::vector<Box> chop_max_size(const Box& dom, int mgs)
{
    std::vector<int> cuts[3];
    for (int d = 0; d < 3; ++d) {
        const int len = dom.n(d);
        std::vector<int> sizes;
        if (len > mgs) {
            int ratio = 1, bs = mgs, nlen = len;
            while ((bs % 2 == 0) && (nlen % 2 == 0)) { ratio *= 2; bs /= 2; nlen /= 2; }
            const int numblk = (nlen + bs - 1) / bs;
            const int sz = nlen / numblk;
            const int extra = nlen - sz * numblk;
            for (int b = 0; b < numblk; ++b) sizes.push_back((sz + (b < extra ? 1 : 0)) * ratio);
        } else {
            sizes.push_back(len);
        }
        int lo = dom.lo[d];
        for (int s : sizes) { cuts[d].push_back(lo); lo += s; }
        cuts[d].push_back(lo);
    }
    std::vector<Box> out;
    for (size_t k = 0; k + 1 < cuts[2].size(); ++k)
        for (size_t j = 0; j + 1 < cuts[1].size(); ++j)
            for (size_t i = 0; i + 1 < cuts[0].size(); ++i) {
                Box b;
                b.lo[0] = cuts[0][i]; b.hi[0] = cuts[0][i + 1] - 1;
                b.lo[1] = cuts[1][j]; b.hi[1] = cuts[1][j + 1] - 1;
                b.lo[2] = cuts[2][k]; b.hi[2] = cuts[2][k + 1] - 1;
                out.push_back(b);
            }
    return out;
}

// ---------------------------------------------------------------------------
// configuration (Source/LBM.cpp:196-396, IC.cpp, VelocityBC.cpp, EB.cpp)
// ---------------------------------------------------------------------------
static bool need3(const Inputs& in, const std::string& k, std::vector<double>& v, std::string& err)
{
    if (!in.queryarr(k, v) || v.size() < 3) {
        err = "missing or short key " + k;
        return false;
    }
    return true;
}

bool LBM::configure(const Inputs& in, std::string& e)
{
    Config& c = cfg_;
    in.query("max_step", c.max_step);
    in.query("stop_time", c.stop_time);
    std::vector<int> iv;
    if (!in.queryarr("amr.n_cell", iv) || iv.size() < 3) { e = "amr.n_cell must have 3 entries"; return false; }
    for (int d = 0; d < 3; ++d) c.n_cell[d] = iv[d];
    in.query("amr.max_level", c.max_level);
    if (in.queryarr("amr.max_grid_size", iv) && !iv.empty()) c.max_grid_size = iv[0];
    if (in.queryarr("amr.blocking_factor", iv) && !iv.empty()) c.blocking_factor = iv[0];
    if (in.queryarr("amr.n_error_buf", iv) && !iv.empty()) c.n_error_buf = iv[0];
    if (in.queryarr("amr.ref_ratio", iv))
        for (int r : iv)
            if (r != 2) { e = "amr.ref_ratio: only 2 is supported"; return false; }
    in.query("amr.regrid_int", c.regrid_int);
    in.query("amr.plot_int", c.plot_int);
    in.query("amr.plot_file", c.plot_file);
    in.query("amr.chk_int", c.chk_int);
    in.query("amr.chk_file", c.chk_file);
    in.query("amr.file_name_digits", c.file_name_digits);
    in.query("amr.restart", c.restart);
    std::vector<double> dv;
    if (!need3(in, "geometry.prob_lo", dv, e)) return false;
    for (int d = 0; d < 3; ++d) c.prob_lo[d] = dv[d];
    if (!need3(in, "geometry.prob_hi", dv, e)) return false;
    for (int d = 0; d < 3; ++d) c.prob_hi[d] = dv[d];
    if (in.queryarr("geometry.is_periodic", iv))
        for (int d = 0; d < 3 && d < (int)iv.size(); ++d) c.is_periodic[d] = iv[d];
    if (in.queryarr("lbm.bc_lo", iv))
        for (int d = 0; d < 3 && d < (int)iv.size(); ++d) c.bc_lo[d] = iv[d];
    if (in.queryarr("lbm.bc_hi", iv))
        for (int d = 0; d < 3 && d < (int)iv.size(); ++d) c.bc_hi[d] = iv[d];
    // LBM.cpp:224-256 consistency of periodicity and BC codes
    for (int d = 0; d < 3; ++d) {
        if (c.is_periodic[d] && (c.bc_lo[d] != 0 || c.bc_hi[d] != 0)) {
            e = "BC is periodic in direction " + std::to_string(d) + " but low/high BC is not 0";
            return false;
        }
        if (!c.is_periodic[d] && (c.bc_lo[d] == 0 || c.bc_hi[d] == 0)) {
            e = "BC is interior in direction " + std::to_string(d) + " but not periodic";
            return false;
        }
    }
    bool has_vel = false;
    for (int d = 0; d < 3; ++d) has_vel |= (c.bc_lo[d] == 2 || c.bc_hi[d] == 2);
    if (has_vel && !in.contains("lbm.velocity_bc_type")) {
        e = "LBM::read_paramaters: velocity BC is used without specifying the type to be used";
        return false;
    }
    in.query("lbm.velocity_bc_type", c.velocity_bc_type);
    if (!in.query("lbm.ic_type", c.ic_type)) { e = "lbm.ic_type is required"; return false; }
    in.query("lbm.dx_outer", c.dx_outer);
    in.query("lbm.dt_outer", c.dt_outer);
    in.query("lbm.nu", c.nu);
    c.alpha = c.nu;
    in.query("lbm.alpha", c.alpha);
    in.query("lbm.save_streaming", c.save_streaming);
    in.query("lbm.save_derived", c.save_derived);
    in.query("lbm.compute_forces", c.compute_forces);
    in.query("lbm.forces_file", c.forces_file);
    in.query("lbm.initial_temperature", c.initial_temperature);
    in.query("lbm.adiabatic_exponent", c.adiabatic_exponent);
    in.query("lbm.mean_molecular_mass", c.m_bar);
    std::string prec = "fp64";
    in.query("lbm.precision", prec);
    if (prec == "fp64") c.precision = MBG_FP64;
    else if (prec == "fp16") c.precision = MBG_FP32C_F16S;
    else if (prec == "bf16") c.precision = MBG_FP32C_BF16S;
    else { e = "lbm.precision must be fp64, fp16 or bf16"; return false; }
    // eb2.*
    in.query("eb2.geom_type", c.geom_type);
    {
        // Source/EB.cpp:5-38 (AMReX built-ins) and Source/Geometry.cpp:5-200
        mbg_geometry& g = c.geom;
        std::memset(&g, 0, sizeof g);
        g.height = -1.0;
        g.normal[0] = 1.0;
        const std::string& t = c.geom_type;
        auto get3 = [&](const std::string& key, double* out, bool required) -> bool {
            std::vector<double> v;
            if (!in.queryarr(key, v) || v.size() < 3) {
                if (required) e = key + " must have 3 entries";
                return !required;
            }
            for (int d = 0; d < 3; ++d) out[d] = v[d];
            return true;
        };
        bool inside = false;
        if (t == "all_regular") {
            g.type = MBG_GEOM_ALL_REGULAR;
        } else if (t == "sphere") {
            g.type = MBG_GEOM_SPHERE;
            in.query("eb2.sphere_radius", g.radius);
            if (!get3("eb2.sphere_center", g.center, true)) return false;
            in.query("eb2.sphere_has_fluid_inside", inside);
        } else if (t == "box" || t == "rotated_box") {
            g.type = t == "box" ? MBG_GEOM_BOX : MBG_GEOM_ROTATED_BOX;
            if (!get3("eb2.box_lo", g.lo, true) || !get3("eb2.box_hi", g.hi, true)) return false;
            in.query("eb2.box_has_fluid_inside", inside);
            in.query("eb2.box_rotation", g.rotation_deg);
            in.query("eb2.box_rotation_axe", g.rotation_axis);
            get3("eb2.box_rotation_center", g.rotation_center, false);
        } else if (t == "cylinder" || t == "rotated_cylinder") {
            g.type = t == "cylinder" ? MBG_GEOM_CYLINDER : MBG_GEOM_ROTATED_CYLINDER;
            if (t == "rotated_cylinder") {   // RotatedCylinder's defaults (Geometry.cpp:131-136)
                g.radius = 0.0002;
                inside = true;
            }
            in.query("eb2.cylinder_radius", g.radius);
            in.query("eb2.cylinder_direction", g.direction);
            if (t == "cylinder") in.query("eb2.cylinder_height", g.height);
            if (!get3("eb2.cylinder_center", g.center, true)) return false;
            in.query("eb2.cylinder_has_fluid_inside", inside);
            in.query("eb2.cylinder_rotation", g.rotation_deg);
            in.query("eb2.cylinder_rotation_axe", g.rotation_axis);
        } else if (t == "plane") {
            g.type = MBG_GEOM_PLANE;
            if (!get3("eb2.plane_point", g.point, true) || !get3("eb2.plane_normal", g.normal, true)) return false;
        } else if (t == "extruded_triangles") {
            g.type = MBG_GEOM_EXTRUDED_TRIANGLES;
            if (!in.query("extruded_triangles.num_tri", g.ntri) || g.ntri < 0 || g.ntri > 5) {
                e = "extruded_triangles.num_tri must be 0 .. 5";
                return false;
            }
            for (int tri = 0; tri < g.ntri; ++tri)
                for (int pt = 0; pt < 3; ++pt) {
                    double v[3];
                    const std::string key =
                        "extruded_triangles.tri_" + std::to_string(tri) + "_point_" + std::to_string(pt);
                    if (!get3(key, v, true)) return false;
                    g.tri[tri][pt][0] = v[0];
                    g.tri[tri][pt][1] = v[1];
                }
        } else {
            e = "eb2.geom_type '" + t + "' is not supported (all_regular, sphere, box, cylinder, plane, "
                "rotated_box, rotated_cylinder, extruded_triangles)";
            return false;
        }
        g.has_fluid_inside = inside ? 1 : 0;
        if (g.direction < 0 || g.direction > 2 || g.rotation_axis < 0 || g.rotation_axis > 2) {
            e = "eb2: cylinder_direction and the rotation axis must be 0, 1 or 2";
            return false;
        }
        geom_ = mbg::geom_from(g);
    }
    // tagging.* (LBM.cpp:302-396)
    std::vector<std::string> inds;
    in.queryarr("tagging.refinement_indicators", inds);
    for (auto& name : inds) {
        Config::Tag t;
        t.name = name;
        const std::string pre = "tagging." + name + ".";
        std::vector<double> blo, bhi;
        if (in.queryarr(pre + "in_box_lo", blo) && in.queryarr(pre + "in_box_hi", bhi) && blo.size() >= 3 &&
            bhi.size() >= 3) {
            t.has_box = true;
            for (int d = 0; d < 3; ++d) { t.box_lo[d] = blo[d]; t.box_hi[d] = bhi[d]; }
        }
        in.query(pre + "max_level", t.max_level);
        in.query(pre + "start_time", t.start_time);
        in.query(pre + "end_time", t.end_time);
        double v;
        if (in.query(pre + "value_greater", v)) { t.kind = 1; t.value = v; }
        else if (in.query(pre + "value_less", v)) { t.kind = 2; t.value = v; }
        else if (in.contains(pre + "adjacent_difference_greater")) {
            e = "tagging: adjacent_difference_greater is not supported with static grids";
            return false;
        } else if (!t.has_box) {
            e = "LBM::read_tagging_parameters(): unrecognized refinement indicator for " + name;
            return false;
        }
        if (t.kind) {
            in.query(pre + "field_name", t.field);
            // the macro fields and the id fields (get_field copies is_fluid
            // component 0 for either id name, Source/LBM.cpp:1536-1546)
            static const char* names[19] = {"rho", "vel_x", "vel_y", "vel_z", "vel_mag", "two_rho_e", "QCorrX",
                                            "QCorrY", "QCorrZ", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz",
                                            "qx", "qy", "qz", "temperature"};
            t.field_index = -1;
            for (int k = 0; k < 19; ++k)
                if (t.field == names[k]) t.field_index = k;
            if (t.field == "is_fluid" || t.field == "eb_boundary") t.field_index = 19;
            if (t.field_index < 0) {
                e = "LBM::read_tagging_parameters(): unknown variable field for tagging criteria " + name +
                    " (the macro fields, is_fluid, eb_boundary)";
                return false;
            }
        }
        c.tags.push_back(t);
    }
    // IC factory (Source/LBM.cpp:1453-1476, IC.cpp)
    ICParams& ic = ic_;
    const std::map<std::string, int> ics = {{"constant", 0}, {"taylorgreen", 1}, {"viscosity_test", 2},
                                            {"thermaldiffusivity_test", 3}, {"sod", 4},
                                            {"gaussian_pulse", 5}, {"temperature_field", 6}};
    auto it = ics.find(c.ic_type);
    if (it == ics.end()) { e = "LBM::set_ics(): User must specify a valid initial condition"; return false; }
    ic.type = it->second;
    const std::string ipre = (ic.type == 1) ? "ic_taylorgreen." : (ic.type == 0) ? "ic_constant."
                           : (ic.type == 2) ? "ic_viscosity_test." : (ic.type == 3) ? "ic_thermaldiffusivity_test."
                           : (ic.type == 4) ? "ic_sod." : (ic.type == 5) ? "ic_gaussian_pulse." : "ic_temperature_field.";
    if (ic.type == 1) {
        in.query(ipre + "rho0", ic.rho0);
        in.query(ipre + "v0", ic.v0);
        if (in.queryarr(ipre + "omega", dv))
            for (int d = 0; d < 3 && d < (int)dv.size(); ++d) ic.omega[d] = dv[d];
    } else {
        in.query(ipre + "density", ic.density);
        if (in.queryarr(ipre + "velocity", dv))
            for (int d = 0; d < 3 && d < (int)dv.size(); ++d) ic.velocity[d] = dv[d];
        if (in.queryarr(ipre + "mach_components", dv))
            for (int d = 0; d < 3 && d < (int)dv.size(); ++d) ic.mach[d] = dv[d];
        in.query(ipre + "wave_length", ic.wave_length);
        in.query(ipre + "density_ratio", ic.density_ratio);
        in.query(ipre + "temperature_ratio", ic.temperature_ratio);
        in.query(ipre + "x_discontinuity", ic.x_discontinuity);
        in.query(ipre + "initial_temperature", ic.initial_temperature);
        in.query(ipre + "adiabatic_exponent", ic.adiabatic_exponent);
        in.query(ipre + "mean_molecular_mass", ic.m_bar);
        in.query(ipre + "amplitude", ic.amplitude);
        in.query(ipre + "width", ic.width);
        for (int d = 0; d < 3; ++d) ic.center[d] = 0.5 * (c.prob_lo[d] + c.prob_hi[d]);
        if (in.queryarr(ipre + "center", dv))
            for (int d = 0; d < 3 && d < (int)dv.size(); ++d) ic.center[d] = dv[d];
        if (ic.type == 6) {
            std::string file;
            if (!in.query(ipre + "file", file)) { e = "ic_temperature_field.file is required"; return false; }
            std::ifstream f(file, std::ios::binary);
            const size_t n = (size_t)c.n_cell[0] * c.n_cell[1] * c.n_cell[2];
            ic.tfield.resize(n);
            if (!f.read((char*)ic.tfield.data(), n * sizeof(double))) {
                e = "ic_temperature_field.file: cannot read " + std::to_string(n) + " doubles from " + file;
                return false;
            }
        }
    }
    ic.sos = std::sqrt(ic.adiabatic_exponent * (R_U / ic.m_bar) * ic.initial_temperature);
    // velocity-BC factory (LBM.cpp:1382-1451, VelocityBC.cpp)
    const std::map<std::string, int> vbcs = {{"noop", 0}, {"constant", 1}, {"channel", 2}, {"parabolic", 3}};
    auto vt = vbcs.find(c.velocity_bc_type);
    if (vt == vbcs.end()) { e = "LBM::set_bcs(): Unknown velocity BC"; return false; }
    vbc_.type = vt->second;
    const std::string vpre = "velocity_bc_" + c.velocity_bc_type + ".";
    vbc_.mach_ref = (vbc_.type == 3) ? 0.05 : 0.005;
    in.query(vpre + "dir", vbc_.dir);
    in.query(vpre + "normal_dir", vbc_.normal_dir);
    in.query(vpre + "tangential_dir", vbc_.tangential_dir);
    in.query(vpre + "Mach_ref", vbc_.mach_ref);
    in.query(vpre + "initial_density", vbc_.initial_density);
    in.query(vpre + "initial_temperature", vbc_.initial_temperature);
    in.query(vpre + "adiabatic_exponent", vbc_.adiabatic_exponent);
    in.query(vpre + "mean_molecular_mass", vbc_.m_bar);
    const double sos = std::sqrt(vbc_.adiabatic_exponent * (R_U / vbc_.m_bar) * vbc_.initial_temperature);
    vbc_.u_ref = vbc_.mach_ref * sos;
    return true;
}

// ---------------------------------------------------------------------------
// geometry and flags (Source/LBM.cpp:1213-1262, EB2 sphere)
// ---------------------------------------------------------------------------
void LBM::level_geometry(int lev, double dx[3]) const
{
    for (int d = 0; d < 3; ++d) dx[d] = (cfg_.prob_hi[d] - cfg_.prob_lo[d]) / (cfg_.n_cell[d] << lev);
}

bool LBM::covered_cell(int lev, int i, int j, int k) const
{
    double dx[3];
    level_geometry(lev, dx);
    return mbg::geom_covered(geom_, cfg_.prob_lo, dx, i, j, k);
}

namespace {
struct LevelIndex {
    int dhi[3];
    const int* per;
    const std::vector<Box>* boxes;
    bool wrap(int p[3]) const
    {
        for (int d = 0; d < 3; ++d) {
            if (p[d] < 0 || p[d] > dhi[d]) {
                if (!per[d]) return false;
                const int L = dhi[d] + 1;
                p[d] = ((p[d] % L) + L) % L;
            }
        }
        return true;
    }
    int owner(const int p[3]) const
    {
        for (size_t n = 0; n < boxes->size(); ++n) {
            const Box& b = (*boxes)[n];
            if (p[0] >= b.lo[0] && p[0] <= b.hi[0] && p[1] >= b.lo[1] && p[1] <= b.hi[1] && p[2] >= b.lo[2] &&
                p[2] <= b.hi[2])
                return (int)n;
        }
        return -1;
    }
};
}  // namespace

// is_fluid of every box grown by 3, with the values that the reference's
// FillBoundary leaves in ghost cells covered by valid cells
void LBM::make_flags(int lev)
{
    const std::vector<Box>& ba = grids_[lev];
    LevelIndex li;
    for (int d = 0; d < 3; ++d) li.dhi[d] = (cfg_.n_cell[d] << lev) - 1;
    li.per = cfg_.is_periodic;
    li.boxes = &ba;
    auto comp0 = [&](int i, int j, int k) -> int {
        int p[3] = {i, j, k};
        if (li.wrap(p) && li.owner(p) >= 0) return covered_cell(lev, p[0], p[1], p[2]) ? 0 : 1;
        return covered_cell(lev, i, j, k) ? 0 : 1;
    };
    auto comp1 = [&](int i, int j, int k) -> int {
        bool all_covered = true;
        all_covered &= (comp0(i - 1, j, k) == 0) && (comp0(i + 1, j, k) == 0);
        all_covered &= (comp0(i, j - 1, k) == 0) && (comp0(i, j + 1, k) == 0);
        all_covered &= (comp0(i, j, k - 1) == 0) && (comp0(i, j, k + 1) == 0);
        return (all_covered || comp0(i, j, k) == 1) ? 0 : 1;
    };
    std::vector<uint8_t>& out = flags_[lev];
    out.clear();
    const bool regular = geom_.type == mbg::GEOM_ALL_REGULAR;
    for (const Box& b : ba) {
        for (int k = b.lo[2] - 3; k <= b.hi[2] + 3; ++k)
            for (int j = b.lo[1] - 3; j <= b.hi[1] + 3; ++j)
                for (int i = b.lo[0] - 3; i <= b.hi[0] + 3; ++i) {
                    if (regular) { out.push_back(1); continue; }
                    const int c0 = comp0(i, j, k);
                    int c1 = 0;
                    int p[3] = {i, j, k};
                    const bool covered = li.wrap(p) && li.owner(p) >= 0;
                    const bool layer3 = i == b.lo[0] - 3 || i == b.hi[0] + 3 || j == b.lo[1] - 3 ||
                                        j == b.hi[1] + 3 || k == b.lo[2] - 3 || k == b.hi[2] + 3;
                    if (covered) c1 = comp1(p[0], p[1], p[2]);
                    else if (!layer3) c1 = comp1(i, j, k);
                    out.push_back((uint8_t)(c0 | (c1 << 1)));
                }
    }
}

// ---------------------------------------------------------------------------
// static grids: level 0 chopped by max_grid_size; finer levels from the
// tagging criteria, buffered, clustered on blocking-factor blocks, chopped
// ---------------------------------------------------------------------------
bool LBM::make_grids(std::string& e, const std::vector<std::vector<uint8_t>>* dense)
{
    Box dom;
    for (int d = 0; d < 3; ++d) { dom.lo[d] = 0; dom.hi[d] = cfg_.n_cell[d] - 1; }
    grids_.clear();
    grids_.push_back(chop_max_size(dom, cfg_.max_grid_size));
    const int L = cfg_.max_level;
    if (L <= 0) return true;
    const int bfc = std::max(1, cfg_.blocking_factor / 2);  // block edge in cells of the coarser level
    const int margin = 4;                                    // explosion stencil + coalescence ring
    // 1. blocks of level l to refine, from the tagging criteria
    std::vector<std::vector<uint8_t>> blk(L);
    std::vector<std::array<int, 3>> nbk(L), ncell(L);
    for (int lev = 0; lev < L; ++lev) {
        int n[3];
        for (int d = 0; d < 3; ++d) { n[d] = cfg_.n_cell[d] << lev; ncell[lev][d] = n[d]; nbk[lev][d] = (n[d] + bfc - 1) / bfc; }
        double dx[3];
        level_geometry(lev, dx);
        blk[lev].assign((size_t)nbk[lev][0] * nbk[lev][1] * nbk[lev][2], 0);
        const int eb = cfg_.n_error_buf;
        for (int k = 0; k < n[2]; ++k)
            for (int j = 0; j < n[1]; ++j)
                for (int i = 0; i < n[0]; ++i) {
                    bool t = false;
                    if (dense) {
                        // tags evaluated on the GPU (mbg_tag_cells) where the level exists
                        const auto& dl = (*dense)[lev];
                        t = !dl.empty() && dl[((size_t)k * n[1] + j) * n[0] + i];
                    }
                    for (const auto& tg : cfg_.tags) {
                        if (dense) break;
                        if (lev >= tg.max_level || !(0.0 >= tg.start_time && 0.0 <= tg.end_time)) continue;
                        if (tg.kind != 0 && tg.field_index != 19) continue;   // state fields: tagged on the GPU
                        bool inbox = true;
                        if (tg.has_box) {
                            const double c[3] = {cfg_.prob_lo[0] + (i + 0.5) * dx[0], cfg_.prob_lo[1] + (j + 0.5) * dx[1],
                                                 cfg_.prob_lo[2] + (k + 0.5) * dx[2]};
                            for (int d = 0; d < 3; ++d) inbox &= c[d] >= tg.box_lo[d] && c[d] <= tg.box_hi[d];
                        }
                        if (!inbox) continue;
                        if (tg.kind == 0) t = true;
                        else {
                            const double v = covered_cell(lev, i, j, k) ? 0.0 : 1.0;
                            if ((tg.kind == 1 && v > tg.value) || (tg.kind == 2 && v < tg.value)) t = true;
                        }
                    }
                    if (!t) continue;
                    for (int kk = k - eb; kk <= k + eb; ++kk)
                        for (int jj = j - eb; jj <= j + eb; ++jj)
                            for (int ii = i - eb; ii <= i + eb; ++ii) {
                                int p[3] = {ii, jj, kk};
                                bool ok = true;
                                for (int d = 0; d < 3; ++d) {
                                    if (p[d] < 0 || p[d] >= n[d]) {
                                        if (!cfg_.is_periodic[d]) ok = false;
                                        else p[d] = ((p[d] % n[d]) + n[d]) % n[d];
                                    }
                                }
                                if (ok)
                                    blk[lev][((size_t)(p[2] / bfc) * nbk[lev][1] + p[1] / bfc) * nbk[lev][0] + p[0] / bfc] = 1;
                            }
                }
    }
    // 2. drop blocks too close to a non-periodic side; make each coarser
    //    level's blocks cover the next finer level's blocks grown by the margin
    auto near_wall = [&](int lev, int bi, int bj, int bk) {
        const int b[3] = {bi, bj, bk};
        for (int d = 0; d < 3; ++d) {
            if (cfg_.is_periodic[d]) continue;
            if (b[d] * bfc - margin < 0 || (b[d] + 1) * bfc + margin > ncell[lev][d]) return true;
        }
        return false;
    };
    for (int lev = L - 1; lev >= 0; --lev) {
        for (int bk = 0; bk < nbk[lev][2]; ++bk)
            for (int bj = 0; bj < nbk[lev][1]; ++bj)
                for (int bi = 0; bi < nbk[lev][0]; ++bi) {
                    uint8_t& v = blk[lev][((size_t)bk * nbk[lev][1] + bj) * nbk[lev][0] + bi];
                    if (v && near_wall(lev, bi, bj, bk)) v = 0;
                }
        if (lev == 0) break;
        // level-lev cells needed = blocks grown by margin; as cells of lev-1
        const int* n = ncell[lev].data();
        for (int bk = 0; bk < nbk[lev][2]; ++bk)
            for (int bj = 0; bj < nbk[lev][1]; ++bj)
                for (int bi = 0; bi < nbk[lev][0]; ++bi) {
                    if (!blk[lev][((size_t)bk * nbk[lev][1] + bj) * nbk[lev][0] + bi]) continue;
                    for (int k = bk * bfc - margin; k < (bk + 1) * bfc + margin; ++k)
                        for (int j = bj * bfc - margin; j < (bj + 1) * bfc + margin; ++j)
                            for (int i = bi * bfc - margin; i < (bi + 1) * bfc + margin; ++i) {
                                int p[3] = {i, j, k};
                                bool ok = true;
                                for (int d = 0; d < 3; ++d) {
                                    if (p[d] < 0 || p[d] >= n[d]) {
                                        if (!cfg_.is_periodic[d]) ok = false;
                                        else p[d] = ((p[d] % n[d]) + n[d]) % n[d];
                                    }
                                }
                                if (!ok) continue;
                                const int c[3] = {p[0] / 2, p[1] / 2, p[2] / 2};
                                blk[lev - 1][((size_t)(c[2] / bfc) * nbk[lev - 1][1] + c[1] / bfc) * nbk[lev - 1][0] +
                                             c[0] / bfc] = 1;
                            }
                }
    }
    // 3. cluster blocks into boxes (greedy x runs, then y, then z), refine, chop
    for (int lev = 0; lev < L; ++lev) {
        const auto& nb = nbk[lev];
        const int* n = ncell[lev].data();
        std::vector<uint8_t> used(blk[lev].size(), 0);
        auto B = [&](int i, int j, int k) { return ((size_t)k * nb[1] + j) * nb[0] + i; };
        auto free_tag = [&](int i, int j, int k) { return blk[lev][B(i, j, k)] && !used[B(i, j, k)]; };
        std::vector<Box> fine;
        for (int bk = 0; bk < nb[2]; ++bk)
            for (int bj = 0; bj < nb[1]; ++bj)
                for (int bi = 0; bi < nb[0]; ++bi) {
                    if (!free_tag(bi, bj, bk)) continue;
                    int ie = bi;
                    while (ie + 1 < nb[0] && free_tag(ie + 1, bj, bk)) ++ie;
                    int je = bj;
                    for (bool grow = true; grow && je + 1 < nb[1];) {
                        for (int i = bi; i <= ie; ++i) grow &= free_tag(i, je + 1, bk);
                        if (grow) ++je;
                    }
                    int ke = bk;
                    for (bool grow = true; grow && ke + 1 < nb[2];) {
                        for (int j = bj; j <= je; ++j)
                            for (int i = bi; i <= ie; ++i) grow &= free_tag(i, j, ke + 1);
                        if (grow) ++ke;
                    }
                    for (int k = bk; k <= ke; ++k)
                        for (int j = bj; j <= je; ++j)
                            for (int i = bi; i <= ie; ++i) used[B(i, j, k)] = 1;
                    Box fb;
                    const int lo3[3] = {bi, bj, bk}, hi3[3] = {ie, je, ke};
                    for (int d = 0; d < 3; ++d) {
                        fb.lo[d] = 2 * lo3[d] * bfc;
                        fb.hi[d] = 2 * std::min(n[d], (hi3[d] + 1) * bfc) - 1;
                    }
                    for (const Box& x : chop_max_size(fb, cfg_.max_grid_size)) fine.push_back(x);
                }
        if (fine.empty()) break;
        grids_.push_back(fine);
    }
    (void)e;
    return true;
}

// ---------------------------------------------------------------------------
// initial conditions (Source/IC.H:13-425) and Initializer (IC.H:460-525)
// ---------------------------------------------------------------------------
void LBM::ic_state(int lev, int i, int j, int k, double& rho, double vel[3], double& temp, double& Rg,
                   double& gamma) const
{
    const ICParams& p = ic_;
    double dx[3];
    level_geometry(lev, dx);
    const double* plo = cfg_.prob_lo;
    switch (p.type) {
    case 0:
        rho = p.density;
        for (int d = 0; d < 3; ++d) vel[d] = p.mach[d] * p.sos;
        temp = p.initial_temperature; Rg = R_U / p.m_bar; gamma = p.adiabatic_exponent;
        break;
    case 1: {
        const double L_ = 1.0 / M_PI;
        const double x = plo[0] + (i + 0.5) * dx[0];
        const double y = plo[1] + (j + 0.5) * dx[1];
        const double z = plo[2] + (k + 0.5) * dx[2];
        const double o0 = p.omega[0], o1 = p.omega[1], o2 = p.omega[2];
        rho = p.rho0 + p.rho0 * p.v0 * p.v0 / 16.0 *
                           (std::cos(2.0 * o0 * x / L_) + std::cos(2.0 * o1 * y / L_)) *
                           (std::cos(2.0 * o2 * z / L_) + 2.0);
        vel[0] = p.v0 * std::sin(o0 * x / L_) * std::cos(o1 * y / L_) * std::cos(o2 * z / L_);
        vel[1] = -p.v0 * std::cos(o0 * x / L_) * std::sin(o1 * y / L_) * std::cos(o2 * z / L_);
        vel[2] = 0.0;
        temp = 1.0 / 3.0; Rg = R_U / R_U; gamma = 5.0 / 3.0;
    } break;
    case 2: {
        const double y = plo[1] + (j + 0.5 * 0.0) * dx[1];
        rho = p.density;
        const double a0 = 0.010 * p.sos;
        vel[0] = p.mach[0] * p.sos + a0 * std::sin(2.0 * M_PI * y / p.wave_length);
        vel[1] = p.mach[1] * p.sos;
        vel[2] = p.mach[2] * p.sos;
        temp = p.initial_temperature; Rg = R_U / p.m_bar; gamma = p.adiabatic_exponent;
    } break;
    case 3: {
        const double y = plo[1] + (j + 0.5 * 0.0) * dx[1];
        const double a0 = 0.0010 * p.initial_temperature;
        Rg = R_U / p.m_bar;
        const double pressure = p.density * Rg * p.initial_temperature;
        rho = p.density + a0 * std::sin(2.0 * M_PI * y / p.wave_length);
        for (int d = 0; d < 3; ++d) vel[d] = p.mach[d] * p.sos;
        gamma = p.adiabatic_exponent;
        temp = pressure / (rho * Rg);
    } break;
    case 4: {
        const double x = plo[0] + (i + 0.5 * 0.0) * dx[0];
        Rg = R_U / p.m_bar;
        for (int d = 0; d < 3; ++d) vel[d] = p.mach[d] * p.sos;
        gamma = p.adiabatic_exponent;
        rho = p.density + 0.5 * (1.0 + std::tanh((x - p.x_discontinuity) * 3.0)) *
                              (p.density_ratio * p.density - p.density);
        temp = p.initial_temperature + 0.5 * (1.0 + std::tanh((x - p.x_discontinuity) * 3.0)) *
                                           (p.temperature_ratio * p.initial_temperature - p.initial_temperature);
    } break;
    case 5: {
        const double x = plo[0] + (i + 0.5) * dx[0] - p.center[0];
        const double y = plo[1] + (j + 0.5) * dx[1] - p.center[1];
        const double z = plo[2] + (k + 0.5) * dx[2] - p.center[2];
        const double r2 = x * x + y * y + z * z;
        rho = p.density + p.amplitude * std::exp(-r2 / (2.0 * p.width * p.width));
        vel[0] = vel[1] = vel[2] = 0.0;
        temp = p.initial_temperature; Rg = R_U / p.m_bar; gamma = p.adiabatic_exponent;
    } break;
    case 6: {
        const int n0 = cfg_.n_cell[0] << lev, n1 = cfg_.n_cell[1] << lev, n2 = cfg_.n_cell[2] << lev;
        int ii = ((i % n0) + n0) % n0, jj = ((j % n1) + n1) % n1, kk = ((k % n2) + n2) % n2;
        ii >>= lev; jj >>= lev; kk >>= lev;
        rho = p.density;
        vel[0] = vel[1] = vel[2] = 0.0;
        temp = p.tfield[((size_t)kk * cfg_.n_cell[1] + jj) * cfg_.n_cell[0] + ii];
        Rg = R_U / p.m_bar; gamma = p.adiabatic_exponent;
    } break;
    }
}

void LBM::initial_state(int lev, std::vector<double>& f, std::vector<double>& g) const
{
    const std::vector<Box>& ba = grids_[lev];
    long long tot = 0;
    std::vector<long long> off;
    for (const Box& b : ba) { off.push_back(tot); tot += b.vol(); }
    f.assign((size_t)tot * mbg::NQ, 0.0);
    g.assign((size_t)tot * mbg::NQ, 0.0);
    const mbg::Lattice<double> lat = mbg::make_lattice<double>();
    const std::vector<uint8_t>& fl = flags_[lev];
    std::vector<long long> foff;
    long long fo = 0;
    for (const Box& b : ba) { foff.push_back(fo); fo += (long long)(b.n(0) + 6) * (b.n(1) + 6) * (b.n(2) + 6); }
#pragma omp parallel for schedule(dynamic)
    for (int n = 0; n < (int)ba.size(); ++n) {
        const Box& b = ba[n];
        const long long vol = b.vol();
        double* F = f.data() + off[n] * mbg::NQ;
        double* G = g.data() + off[n] * mbg::NQ;
        long long c = 0;
        for (int k = b.lo[2]; k <= b.hi[2]; ++k)
            for (int j = b.lo[1]; j <= b.hi[1]; ++j)
                for (int i = b.lo[0]; i <= b.hi[0]; ++i, ++c) {
                    const long long fi = foff[n] + ((long long)(k - b.lo[2] + 3) * (b.n(1) + 6) + (j - b.lo[1] + 3)) *
                                                       (b.n(0) + 6) + (i - b.lo[0] + 3);
                    if (!(fl[fi] & 1)) {  // fill_f_inside_eb (LBM.cpp:1278-1298)
                        for (int q = 0; q < mbg::NQ; ++q) { F[q * vol + c] = 0.0; G[q * vol + c] = 0.0; }
                        continue;
                    }
                    double rho = 1.0, vel[3] = {0, 0, 0}, t = 1.0 / 3.0, Rg = 1.0, gamma = 1.667;
                    ic_state(lev, i, j, k, rho, vel, t, Rg, gamma);
                    for (int q = 0; q < mbg::NQ; ++q) {
                        F[q * vol + c] = mbg::eq_f_plain<double>(q, rho, vel, Rg * t);
                        G[q * vol + c] = mbg::eq_g_plain<double>(q, rho, vel, Rg, t, gamma, lat);
                    }
                }
    }
}

// ---------------------------------------------------------------------------
// init_data / evolve (Source/LBM.cpp:155-194, 398-448)
// ---------------------------------------------------------------------------
LBM::~LBM()
{
    if (ctx_) mbg_destroy(ctx_);
}

mbg_status LBM::prepare()
{
    if (prepared_) return MBG_OK;
    if (!make_grids(err)) return MBG_EINVAL;
    flags_.assign(grids_.size(), {});
    for (size_t lev = 0; lev < grids_.size(); ++lev) make_flags((int)lev);
    prepared_ = true;
    return MBG_OK;
}

bool LBM::has_field_tags() const
{
    for (const auto& t : cfg_.tags)
        if (t.kind != 0 && t.field_index != 19) return true;
    return false;
}

// the context, the levels with their GPU flags and (no restart) the IC
mbg_status LBM::build_context()
{
    mbg_params& p = params_;
    std::memset(&p, 0, sizeof(p));
    for (int d = 0; d < 3; ++d) {
        p.n_cell[d] = cfg_.n_cell[d];
        p.prob_lo[d] = cfg_.prob_lo[d];
        p.prob_hi[d] = cfg_.prob_hi[d];
        p.is_periodic[d] = cfg_.is_periodic[d];
        p.bc_lo[d] = cfg_.bc_lo[d];
        p.bc_hi[d] = cfg_.bc_hi[d];
    }
    p.nu = cfg_.nu; p.alpha = cfg_.alpha; p.dx_outer = cfg_.dx_outer; p.dt_outer = cfg_.dt_outer;
    p.adiabatic_exponent = cfg_.adiabatic_exponent; p.m_bar = cfg_.m_bar;
    p.precision = cfg_.precision;
    p.rho_ref = ic_.type == 1 ? ic_.rho0 : ic_.density;
    p.t_ref = ic_.type == 1 ? 1.0 / 3.0 : ic_.initial_temperature;
    if (ic_.type == 0)   // uniform initial flow: the storage shift follows it
        for (int d = 0; d < 3; ++d) p.u_ref[d] = ic_.mach[d] * ic_.sos;
    p.velbc_type = vbc_.type;
    p.vbc_dir = vbc_.dir; p.vbc_normal_dir = vbc_.normal_dir; p.vbc_tangential_dir = vbc_.tangential_dir;
    p.vbc_u_ref = vbc_.u_ref; p.vbc_initial_density = vbc_.initial_density;
    p.vbc_initial_temperature = vbc_.initial_temperature; p.vbc_adiabatic_exponent = vbc_.adiabatic_exponent;
    p.vbc_m_bar = vbc_.m_bar;
    if (ctx_) { mbg_destroy(ctx_); ctx_ = nullptr; }
    mbg_status st = mbg_create(&p, nullptr, &ctx_);
    if (st != MBG_OK) { err = mbg_last_error(nullptr); return st; }
    for (size_t lev = 0; lev < grids_.size(); ++lev) {
        std::vector<int> lohi;
        for (const Box& b : grids_[lev])
            for (int x : {b.lo[0], b.lo[1], b.lo[2], b.hi[0], b.hi[1], b.hi[2]}) lohi.push_back(x);
        // the level's is_fluid flags from the geometry, on the GPU (the grids
        // were tagged from the same implicit functions on the host)
        if ((st = level_flags_gpu((int)lev, flags_[lev])) != MBG_OK) return st;
        st = mbg_define_level(ctx_, (int)lev, (int)grids_[lev].size(), lohi.data(), flags_[lev].data());
        if (st != MBG_OK) { err = mbg_last_error(ctx_); return st; }
        if (!cfg_.restart.empty()) continue;
        std::vector<double> f, g;
        initial_state((int)lev, f, g);
        st = mbg_set_state(ctx_, (int)lev, f.data(), g.data());
        if (st != MBG_OK) { err = mbg_last_error(ctx_); return st; }
    }
    return MBG_OK;
}

mbg_status LBM::level_flags_gpu(int lev, std::vector<uint8_t>& out)
{
    std::vector<int> lohi;
    long long n = 0;
    for (const Box& b : grids_[lev]) {
        for (int x : {b.lo[0], b.lo[1], b.lo[2], b.hi[0], b.hi[1], b.hi[2]}) lohi.push_back(x);
        n += (long long)(b.n(0) + 6) * (b.n(1) + 6) * (b.n(2) + 6);
    }
    out.resize((size_t)n);
    mbg_status st = mbg_geometry_flags(&cfg_.geom, &params_, lev, (int)grids_[lev].size(), lohi.data(), out.data(),
                                       ctx_ ? mbg_stream(ctx_) : nullptr);
    if (st != MBG_OK) err = mbg_last_error(nullptr);
    return st;
}

mbg_status LBM::gpu_tags(std::vector<std::vector<uint8_t>>& dense)
{
    const int nlev = (int)grids_.size();
    dense.assign(cfg_.max_level, {});
    std::vector<mbg_tag> tags;
    for (const auto& t : cfg_.tags) {
        mbg_tag g{};
        g.field = t.field_index;
        g.kind = t.kind;
        g.value = t.value;
        g.has_box = t.has_box ? 1 : 0;
        for (int d = 0; d < 3; ++d) { g.box_lo[d] = t.box_lo[d]; g.box_hi[d] = t.box_hi[d]; }
        g.start_time = t.start_time;
        g.end_time = t.end_time;
        g.max_level = t.max_level;
        tags.push_back(g);
    }
    if ((int)tags.size() > MBG_MAX_TAGS) { err = "tagging: at most 8 refinement indicators"; return MBG_EINVAL; }
    for (int lev = 0; lev < std::min(nlev, cfg_.max_level); ++lev) {
        long long ncell = 0;
        for (const Box& b : grids_[lev]) ncell += b.vol();
        std::vector<uint8_t> t((size_t)ncell);
        mbg_status st = mbg_tag_cells(ctx_, lev, tags.data(), (int)tags.size(), time_, t.data());
        if (st != MBG_OK) { err = mbg_last_error(ctx_); return st; }
        const int n[3] = {cfg_.n_cell[0] << lev, cfg_.n_cell[1] << lev, cfg_.n_cell[2] << lev};
        auto& D = dense[lev];
        D.assign((size_t)n[0] * n[1] * n[2], 0);
        long long off = 0;
        for (const Box& b : grids_[lev])
            for (int k = b.lo[2]; k <= b.hi[2]; ++k)
                for (int j = b.lo[1]; j <= b.hi[1]; ++j)
                    for (int i = b.lo[0]; i <= b.hi[0]; ++i, ++off)
                        D[((size_t)k * n[1] + j) * n[0] + i] = t[(size_t)off];
    }
    return MBG_OK;
}

static bool same_grids(const std::vector<std::vector<Box>>& a, const std::vector<std::vector<Box>>& b)
{
    if (a.size() != b.size()) return false;
    for (size_t l = 0; l < a.size(); ++l) {
        if (a[l].size() != b[l].size()) return false;
        for (size_t n = 0; n < a[l].size(); ++n)
            for (int d = 0; d < 3; ++d)
                if (a[l][n].lo[d] != b[l][n].lo[d] || a[l][n].hi[d] != b[l][n].hi[d]) return false;
    }
    return true;
}

mbg_status LBM::regrid()
{
    if (!ctx_) { err = "regrid: the driver is not initialised"; return MBG_ESTATE; }
    if (cfg_.max_level <= 0) return MBG_OK;
    std::vector<std::vector<uint8_t>> dense;
    mbg_status st = gpu_tags(dense);
    if (st != MBG_OK) return st;
    const std::vector<std::vector<Box>> old = grids_;
    if (!make_grids(err, &dense)) return MBG_EINVAL;
    if (same_grids(old, grids_)) return MBG_OK;
    const int nlev = (int)grids_.size();
    flags_.resize(nlev);
    std::vector<int> nbox, lohi;
    std::vector<uint8_t> fl;
    for (int lev = 1; lev < nlev; ++lev) {
        if ((st = level_flags_gpu(lev, flags_[lev])) != MBG_OK) return st;
        nbox.push_back((int)grids_[lev].size());
        for (const Box& b : grids_[lev])
            for (int x : {b.lo[0], b.lo[1], b.lo[2], b.hi[0], b.hi[1], b.hi[2]}) lohi.push_back(x);
        fl.insert(fl.end(), flags_[lev].begin(), flags_[lev].end());
    }
    st = mbg_regrid(ctx_, 1, nlev - 1, nbox.data(), lohi.data(), fl.data());
    if (st != MBG_OK) err = mbg_last_error(ctx_);
    return st;
}

mbg_status LBM::init_data()
{
    mbg_status st = prepare();
    if (st != MBG_OK) return st;
    if ((st = build_context()) != MBG_OK) return st;
    if (cfg_.restart.empty() && has_field_tags()) {
        // InitFromScratch tags each level on its initial data
        // (MakeNewLevelFromScratch, then ErrorEst): tag the initial state on
        // the GPU, rebuild the grids and start again from the IC until the
        // grids stop changing (at most max_level rounds)
        for (int it = 0; it < cfg_.max_level; ++it) {
            std::vector<std::vector<uint8_t>> dense;
            if ((st = gpu_tags(dense)) != MBG_OK) return st;
            const std::vector<std::vector<Box>> old = grids_;
            if (!make_grids(err, &dense)) return MBG_EINVAL;
            if (same_grids(old, grids_)) break;
            flags_.assign(grids_.size(), {});
            for (size_t lev = 0; lev < grids_.size(); ++lev) make_flags((int)lev);
            if ((st = build_context()) != MBG_OK) return st;
        }
    }
    if (!cfg_.restart.empty()) {
        // LBM::init_data's restart branch (Source/LBM.cpp:177-182)
        st = read_checkpoint();
        if (st != MBG_OK) return st;
        if (cfg_.compute_forces) write_forces(false);
    } else {
        for (int lev = (int)grids_.size() - 2; lev >= 0; --lev) {
            st = mbg_average_down(ctx_, lev, 0);
            if (st != MBG_OK) { err = mbg_last_error(ctx_); return st; }
        }
        step_ = 0;
        time_ = 0.0;
        if (cfg_.chk_int > 0) {
            st = write_checkpoint(numbered(cfg_.chk_file));
            if (st != MBG_OK) return st;
        }
        if (cfg_.compute_forces) write_forces(true);
    }
    last_regrid_step_ = step_;
    if (cfg_.plot_int > 0) {
        st = write_plot_file(numbered(cfg_.plot_file));
        if (st != MBG_OK) return st;
    }
    return MBG_OK;
}

// amrex::Concatenate(root, step, file_name_digits)
std::string LBM::numbered(const std::string& root) const
{
    char num[32];
    std::snprintf(num, sizeof num, "%0*d", cfg_.file_name_digits, step_);
    return root + num;
}

void LBM::write_forces(bool init)
{
    if (mbg_eb_forces(ctx_, last_forces.data()) != MBG_OK) return;
    std::ofstream f(cfg_.forces_file, init ? std::ios::trunc : std::ios::app);
    f.precision(16);
    f << step_ << " " << time_ << " " << last_forces[0] << " " << last_forces[1] << " " << last_forces[2] << "\n";
}

mbg_status LBM::evolve(int nsteps)
{
    // LBM::evolve (Source/LBM.cpp:398-448): nsteps <= 0 runs to max_step /
    // stop_time and then writes the last plotfile if it is not written yet
    const bool to_end = nsteps <= 0;
    const int last = to_end ? cfg_.max_step : step_ + nsteps;
    while (step_ < last && time_ < cfg_.stop_time) {
        // the regrid branch of time_step(0) (Source/LBM.cpp:456-479): before
        // a coarse step whose count is a multiple of amr.regrid_int
        if (cfg_.regrid_int > 0 && cfg_.max_level > 0 && step_ > last_regrid_step_ &&
            step_ % cfg_.regrid_int == 0) {
            mbg_status sr = regrid();
            if (sr != MBG_OK) return sr;
            last_regrid_step_ = step_;
        }
        mbg_status st = mbg_step(ctx_, 1);
        if (st != MBG_OK) { err = mbg_last_error(ctx_); return st; }
        ++step_;
        time_ += 1.0;
        if (cfg_.compute_forces) write_forces(false);
        if (cfg_.plot_int > 0 && step_ % cfg_.plot_int == 0) {
            st = write_plot_file(numbered(cfg_.plot_file));
            if (st != MBG_OK) return st;
        }
        if (cfg_.chk_int > 0 && step_ % cfg_.chk_int == 0) {
            st = write_checkpoint(numbered(cfg_.chk_file));
            if (st != MBG_OK) return st;
        }
    }
    if (to_end && cfg_.plot_int > 0 && step_ > last_plot_step_) {
        mbg_status st = write_plot_file(numbered(cfg_.plot_file));
        if (st != MBG_OK) return st;
    }
    return mbg_synchronize(ctx_);
}

// ---------------------------------------------------------------------------
// plotfile and checkpoint (Source/LBM.cpp:1613-1916)
// ---------------------------------------------------------------------------
namespace {

const char* const MACRO_NAMES[19] = {"rho", "vel_x", "vel_y", "vel_z", "vel_mag", "two_rho_e", "QCorrX",
                                     "QCorrY", "QCorrZ", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz",
                                     "qx", "qy", "qz", "temperature"};
const char* const DERIVED_NAMES[7] = {"vort_x", "vort_y", "vort_z", "vort_mag", "dQCorrX", "dQCorrY", "dQCorrZ"};

std::string two_digits(const char* pre, int q)
{
    char b[16];
    std::snprintf(b, sizeof b, "%s%02d", pre, q);
    return b;
}

bool mkdir_p(const std::string& d)
{
    if (mkdir(d.c_str(), 0755) == 0) return true;
    struct stat st;
    return errno == EEXIST && stat(d.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

std::vector<int> lohi_of(const std::vector<Box>& ba)
{
    std::vector<int> v;
    for (const Box& b : ba)
        for (int x : {b.lo[0], b.lo[1], b.lo[2], b.hi[0], b.hi[1], b.hi[2]}) v.push_back(x);
    return v;
}

}  // namespace

mbg_status LBM::write_plot_file(const std::string& name)
{
    if (!ctx_) { err = "write_plot_file: the driver is not initialised"; return MBG_ESTATE; }
    // variable list of LBM::LBM (Source/LBM.cpp:14-82): macro, f, g, derived, flags
    std::vector<std::string> names(MACRO_NAMES, MACRO_NAMES + 19);
    if (cfg_.save_streaming) {
        for (int q = 0; q < mbg::NQ; ++q) names.push_back(two_digits("f_", q));
        for (int q = 0; q < mbg::NQ; ++q) names.push_back(two_digits("g_", q));
    }
    if (cfg_.save_derived) names.insert(names.end(), DERIVED_NAMES, DERIVED_NAMES + 7);
    names.push_back("is_fluid");
    names.push_back("eb_boundary");
    const int nc = (int)names.size();
    const int nlev = (int)grids_.size();
    std::vector<std::vector<double>> data(nlev);
    std::vector<const double*> ptrs(nlev);
    std::vector<int> nbox(nlev), steps(nlev), lohi;
    for (int lev = 0; lev < nlev; ++lev) {
        const std::vector<Box>& ba = grids_[lev];
        long long ncell = 0;
        for (const Box& b : ba) ncell += b.vol();
        std::vector<double> mac((size_t)ncell * 19), f, g, der;
        mbg_status st = mbg_get_macro(ctx_, lev, mac.data());
        if (st == MBG_OK && cfg_.save_streaming) {
            f.resize((size_t)ncell * mbg::NQ);
            g.resize((size_t)ncell * mbg::NQ);
            st = mbg_get_state(ctx_, lev, f.data(), g.data());
        }
        if (st == MBG_OK && cfg_.save_derived) {
            der.resize((size_t)ncell * 7);
            st = mbg_get_derived(ctx_, lev, der.data());
        }
        if (st != MBG_OK) { err = mbg_last_error(ctx_); return st; }
        std::vector<double>& D = data[lev];
        D.resize((size_t)ncell * nc);
        long long off = 0, foff = 0;
        for (const Box& b : ba) {
            const long long v = b.vol();
            double* dst = D.data() + off * nc;
            int c = 0;
            auto put = [&](const double* src, int n) {
                std::memcpy(dst + (size_t)c * v, src, (size_t)n * v * sizeof(double));
                c += n;
            };
            put(mac.data() + off * 19, 19);
            if (cfg_.save_streaming) {
                put(f.data() + off * mbg::NQ, mbg::NQ);
                put(g.data() + off * mbg::NQ, mbg::NQ);
            }
            if (cfg_.save_derived) put(der.data() + off * 7, 7);
            // is_fluid components 0 and 1 of the valid cells
            long long cell = 0;
            for (int k = 0; k < b.n(2); ++k)
                for (int j = 0; j < b.n(1); ++j)
                    for (int i = 0; i < b.n(0); ++i, ++cell) {
                        const uint8_t fl = flags_[lev][foff + ((long long)(k + 3) * (b.n(1) + 6) + (j + 3)) *
                                                                  (b.n(0) + 6) + (i + 3)];
                        dst[(size_t)c * v + cell] = (fl & 1) ? 1.0 : 0.0;
                        dst[(size_t)(c + 1) * v + cell] = (fl & 2) ? 1.0 : 0.0;
                    }
            off += v;
            foff += (long long)(b.n(0) + 6) * (b.n(1) + 6) * (b.n(2) + 6);
        }
        ptrs[lev] = D.data();
        nbox[lev] = (int)ba.size();
        steps[lev] = step_ << lev;
        std::vector<int> l = lohi_of(ba);
        lohi.insert(lohi.end(), l.begin(), l.end());
    }
    std::vector<const char*> cn;
    for (const std::string& n : names) cn.push_back(n.c_str());
    mbg_status st = mbg_write_plotfile(name.c_str(), nlev, nbox.data(), lohi.data(), cfg_.n_cell, cfg_.prob_lo,
                                       cfg_.prob_hi, nc, cn.data(), ptrs.data(), time_, steps.data());
    if (st != MBG_OK) { err = mbg_last_error(nullptr); return st; }
    last_plot_step_ = step_;
    return MBG_OK;
}

// LBM::write_checkpoint_file (Source/LBM.cpp:1692-1783): Header, then f and
// g of every level as VisMF multifabs Level_<l>/f_00 and Level_<l>/g_00
mbg_status LBM::write_checkpoint(const std::string& name)
{
    if (!ctx_) { err = "write_checkpoint: the driver is not initialised"; return MBG_ESTATE; }
    const int nlev = (int)grids_.size();
    if (!mkdir_p(name)) { err = "write_checkpoint: cannot create directory " + name; return MBG_EINVAL; }
    {
        std::ofstream h(name + "/Header", std::ios::trunc);
        if (!h) { err = "write_checkpoint: cannot open " + name + "/Header"; return MBG_EINVAL; }
        h.precision(17);
        h << "Checkpoint file for LBM\n" << nlev - 1 << "\n";
        for (int l = 0; l < nlev; ++l) h << (step_ << l) << " ";
        h << "\n";
        for (int l = 0; l < nlev; ++l) h << 1.0 / (double)(1 << l) << " ";
        h << "\n";
        for (int l = 0; l < nlev; ++l) h << time_ << " ";
        h << "\n";
        for (int l = 0; l < nlev; ++l) {
            const std::vector<Box>& ba = grids_[l];
            h << "(" << ba.size() << " 0\n";
            for (const Box& b : ba)
                h << "((" << b.lo[0] << "," << b.lo[1] << "," << b.lo[2] << ") (" << b.hi[0] << "," << b.hi[1] << ","
                  << b.hi[2] << ") (0,0,0))\n";
            h << ")\n";
        }
        h.close();
        if (!h) { err = "write_checkpoint: write failed: " + name + "/Header"; return MBG_EINVAL; }
    }
    for (int lev = 0; lev < nlev; ++lev) {
        const std::string ld = name + "/Level_" + std::to_string(lev);
        if (!mkdir_p(ld)) { err = "write_checkpoint: cannot create directory " + ld; return MBG_EINVAL; }
        long long ncell = 0;
        for (const Box& b : grids_[lev]) ncell += b.vol();
        std::vector<double> f((size_t)ncell * mbg::NQ), g((size_t)ncell * mbg::NQ);
        mbg_status st = mbg_get_state(ctx_, lev, f.data(), g.data());
        if (st != MBG_OK) { err = mbg_last_error(ctx_); return st; }
        const std::vector<int> lohi = lohi_of(grids_[lev]);
        const int nb = (int)grids_[lev].size();
        st = mbg_write_multifab((ld + "/f_00").c_str(), nb, lohi.data(), mbg::NQ, f.data());
        if (st == MBG_OK) st = mbg_write_multifab((ld + "/g_00").c_str(), nb, lohi.data(), mbg::NQ, g.data());
        if (st != MBG_OK) { err = mbg_last_error(nullptr); return st; }
    }
    return MBG_OK;
}

// LBM::read_checkpoint_file (Source/LBM.cpp:1785-1916) onto the static
// grids the inputs build: the Header's box arrays must be those grids
mbg_status LBM::read_checkpoint()
{
    const std::string& dir = cfg_.restart;
    std::ifstream in(dir + "/Header");
    if (!in) { err = "amr.restart: cannot read " + dir + "/Header"; return MBG_EINVAL; }
    std::string line;
    std::getline(in, line);
    int finest = -1;
    in >> finest;
    std::getline(in, line);
    const int nlev = (int)grids_.size();
    if (finest != nlev - 1) {
        err = "amr.restart: the checkpoint has " + std::to_string(finest + 1) + " levels, the inputs build " +
              std::to_string(nlev);
        return MBG_EINVAL;
    }
    std::vector<std::vector<double>> rows(3);
    for (int r = 0; r < 3; ++r) {
        std::getline(in, line);
        std::istringstream ls(line);
        double v;
        while (ls >> v) rows[r].push_back(v);
        if ((int)rows[r].size() != nlev) { err = "amr.restart: malformed Header in " + dir; return MBG_EINVAL; }
    }
    for (int l = 0; l < nlev; ++l) {
        int n = -1, hash = 0;
        char c = 0;
        in >> c >> n >> hash;
        if (c != '(' || n != (int)grids_[l].size()) {
            err = "amr.restart: level " + std::to_string(l) + " of the checkpoint has other grids than the inputs "
                  "build (run-time regridding is not supported)";
            return MBG_EINVAL;
        }
        std::getline(in, line);
        for (int b = 0; b < n; ++b) {
            std::getline(in, line);
            int v[9];
            if (std::sscanf(line.c_str(), " ((%d,%d,%d) (%d,%d,%d) (%d,%d,%d))", &v[0], &v[1], &v[2], &v[3], &v[4],
                            &v[5], &v[6], &v[7], &v[8]) != 9) {
                err = "amr.restart: malformed box in " + dir + "/Header";
                return MBG_EINVAL;
            }
            const Box& B = grids_[l][b];
            if (v[0] != B.lo[0] || v[1] != B.lo[1] || v[2] != B.lo[2] || v[3] != B.hi[0] || v[4] != B.hi[1] ||
                v[5] != B.hi[2]) {
                err = "amr.restart: level " + std::to_string(l) + " box " + std::to_string(b) +
                      " of the checkpoint differs from the grids the inputs build";
                return MBG_EINVAL;
            }
        }
        std::getline(in, line);   // ")"
    }
    for (int lev = 0; lev < nlev; ++lev) {
        const std::string ld = dir + "/Level_" + std::to_string(lev);
        long long ncell = 0;
        for (const Box& b : grids_[lev]) ncell += b.vol();
        std::vector<double> f((size_t)ncell * mbg::NQ), g((size_t)ncell * mbg::NQ);
        const std::vector<int> lohi = lohi_of(grids_[lev]);
        const int nb = (int)grids_[lev].size();
        mbg_status st = mbg_read_multifab((ld + "/f_00").c_str(), nb, lohi.data(), mbg::NQ, f.data());
        if (st == MBG_OK) st = mbg_read_multifab((ld + "/g_00").c_str(), nb, lohi.data(), mbg::NQ, g.data());
        if (st != MBG_OK) { err = mbg_last_error(nullptr); return st; }
        // fill_f_inside_eb (Source/LBM.cpp:1278-1298): solid cells start at 0
        long long off = 0, foff = 0;
        for (const Box& b : grids_[lev]) {
            const long long v = b.vol();
            long long cell = 0;
            for (int k = 0; k < b.n(2); ++k)
                for (int j = 0; j < b.n(1); ++j)
                    for (int i = 0; i < b.n(0); ++i, ++cell) {
                        const uint8_t fl = flags_[lev][foff + ((long long)(k + 3) * (b.n(1) + 6) + (j + 3)) *
                                                                  (b.n(0) + 6) + (i + 3)];
                        if (fl & 1) continue;
                        for (int q = 0; q < mbg::NQ; ++q) {
                            f[(size_t)(off * mbg::NQ + q * v + cell)] = 0.0;
                            g[(size_t)(off * mbg::NQ + q * v + cell)] = 0.0;
                        }
                    }
            off += v;
            foff += (long long)(b.n(0) + 6) * (b.n(1) + 6) * (b.n(2) + 6);
        }
        st = mbg_set_state(ctx_, lev, f.data(), g.data());
        if (st != MBG_OK) { err = mbg_last_error(ctx_); return st; }
    }
    step_ = (int)rows[0][0];
    time_ = rows[2][0];
    return MBG_OK;
}

}  // namespace mbgdrv
