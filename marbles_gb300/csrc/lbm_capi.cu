// lbm_capi.cu -- C ABI of the host drop-in driver (mbg_lbm_*).
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>

#include "lbm_driver.h"

struct mbg_lbm {
    mbgdrv::LBM lbm;
    std::string err;
};

static std::string g_lbm_err;

extern "C" {

mbg_status mbg_lbm_create(const char* inputs_text, int n_overrides, const char* const* overrides, mbg_lbm** out)
{
    if (!inputs_text || !out) { g_lbm_err = "mbg_lbm_create: null argument"; return MBG_EINVAL; }
    *out = nullptr;
    mbgdrv::Inputs in;
    std::string e;
    if (!in.parse_text(inputs_text, e)) { g_lbm_err = e; return MBG_EINVAL; }
    for (int i = 0; i < n_overrides; ++i)
        if (!in.parse_override(overrides[i], e)) { g_lbm_err = e; return MBG_EINVAL; }
    auto* h = new (std::nothrow) mbg_lbm();
    if (!h) { g_lbm_err = "out of host memory"; return MBG_ENOMEM; }
    try {
        if (!h->lbm.configure(in, e)) {
            g_lbm_err = e;
            delete h;
            return MBG_EINVAL;
        }
    } catch (const std::exception& ex) {
        g_lbm_err = std::string("inputs: ") + ex.what();
        delete h;
        return MBG_EINVAL;
    }
    *out = h;
    return MBG_OK;
}

mbg_status mbg_lbm_init(mbg_lbm* h)
{
    if (!h) return MBG_EINVAL;
    mbg_status st = h->lbm.init_data();
    if (st != MBG_OK) h->err = h->lbm.err;
    return st;
}

mbg_status mbg_lbm_evolve(mbg_lbm* h, int nsteps)
{
    if (!h || !h->lbm.context()) return MBG_ESTATE;
    mbg_status st = h->lbm.evolve(nsteps);
    if (st != MBG_OK) h->err = h->lbm.err;
    return st;
}

mbg_ctx* mbg_lbm_context(mbg_lbm* h) { return h ? h->lbm.context() : nullptr; }

mbg_status mbg_lbm_prepare(mbg_lbm* h)
{
    if (!h) return MBG_EINVAL;
    mbg_status st = h->lbm.prepare();
    if (st != MBG_OK) h->err = h->lbm.err;
    return st;
}

mbg_status mbg_lbm_initial_state(mbg_lbm* h, int lev, double* f, double* g)
{
    if (!h || !f || !g) return MBG_EINVAL;
    mbg_status st = h->lbm.prepare();
    if (st != MBG_OK) { h->err = h->lbm.err; return st; }
    if (lev < 0 || lev >= (int)h->lbm.grids().size()) return MBG_ESTATE;
    std::vector<double> F, G;
    h->lbm.initial_state(lev, F, G);
    std::memcpy(f, F.data(), F.size() * sizeof(double));
    std::memcpy(g, G.data(), G.size() * sizeof(double));
    return MBG_OK;
}

int mbg_lbm_num_levels(const mbg_lbm* h) { return h ? (int)h->lbm.grids().size() : 0; }

mbg_status mbg_lbm_level_boxes(const mbg_lbm* h, int lev, int* lohi, int cap, int* nbox)
{
    if (!h || !nbox) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)h->lbm.grids().size()) return MBG_ESTATE;
    const auto& g = h->lbm.grids()[lev];
    *nbox = (int)g.size();
    if (lohi)
        for (int n = 0; n < (int)g.size() && n < cap; ++n)
            for (int d = 0; d < 3; ++d) { lohi[6 * n + d] = g[n].lo[d]; lohi[6 * n + 3 + d] = g[n].hi[d]; }
    return MBG_OK;
}

mbg_status mbg_lbm_level_flags(const mbg_lbm* h, int lev, uint8_t* out, long long cap, long long* n)
{
    if (!h || !n) return MBG_EINVAL;
    if (lev < 0 || lev >= (int)h->lbm.flags().size()) return MBG_ESTATE;
    const auto& f = h->lbm.flags()[lev];
    *n = (long long)f.size();
    if (out) std::memcpy(out, f.data(), (size_t)std::min<long long>(cap, (long long)f.size()));
    return MBG_OK;
}

mbg_status mbg_lbm_write_plotfile(mbg_lbm* h, const char* name)
{
    if (!h || !name) return MBG_EINVAL;
    mbg_status st = h->lbm.write_plot_file(name);
    if (st != MBG_OK) h->err = h->lbm.err;
    return st;
}

mbg_status mbg_lbm_write_checkpoint(mbg_lbm* h, const char* name)
{
    if (!h || !name) return MBG_EINVAL;
    mbg_status st = h->lbm.write_checkpoint(name);
    if (st != MBG_OK) h->err = h->lbm.err;
    return st;
}

mbg_status mbg_lbm_step_time(const mbg_lbm* h, int* step, double* time)
{
    if (!h) return MBG_EINVAL;
    if (step) *step = h->lbm.step();
    if (time) *time = h->lbm.time();
    return MBG_OK;
}

mbg_status mbg_lbm_regrid(mbg_lbm* h)
{
    if (!h) return MBG_EINVAL;
    mbg_status st = h->lbm.regrid();
    if (st != MBG_OK) h->err = h->lbm.err;
    return st;
}

const char* mbg_lbm_last_error(const mbg_lbm* h) { return h ? h->err.c_str() : g_lbm_err.c_str(); }

void mbg_lbm_destroy(mbg_lbm* h) { delete h; }

}  // extern "C"
