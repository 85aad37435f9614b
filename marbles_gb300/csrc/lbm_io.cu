// lbm_io.cu -- AMReX-format output and restart input of the drop-in driver
// (host code only): the multi-level plotfile the reference writes with
// amrex::WriteMultiLevelPlotfile (Source/LBM.cpp:1677-1690) and the VisMF
// multifabs of its checkpoints (Source/LBM.cpp:1692-1916), so that VisIt,
// yt, Amrvis and the reference's own restart read them.
//
// Formats (AMReX's published on-disk layout):
//   <dir>/Header            "HyperCLaw-V1.1", the variable names, geometry,
//                           refinement ratios, domains, steps, cell sizes and,
//                           per level, the boxes in physical coordinates
//   <dir>/Level_<l>/Cell_H  a VisMF header (version 1): the box array, one
//                           "FabOnDisk" entry per box and per-box minima and
//                           maxima of every component
//   <dir>/Level_<l>/Cell_D_00000
//                           the boxes' FABs one after another: an ASCII line
//                           "FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (1 2 3 4 5
//                           6 7 8)))(box) ncomp" then ncomp x cells IEEE
//                           doubles, little endian, each component contiguous
//                           with i fastest
// Multifabs are written without ghost cells (ngrow 0); the reader also
// accepts files with ghost cells and keeps the valid region.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/marbles_gb300.h"

void mbg_set_global_error(const std::string& msg);

namespace {

const char* FAB_REAL_DESC = "((8, (64 11 52 0 1 12 0 1023)),(8, (1 2 3 4 5 6 7 8)))";

mbg_status io_fail(const std::string& m)
{
    mbg_set_global_error(m);
    return MBG_EINVAL;
}

bool host_little_endian()
{
    const uint16_t one = 1;
    unsigned char c;
    std::memcpy(&c, &one, 1);
    return c == 1;
}

bool make_dir(const std::string& d)
{
    if (mkdir(d.c_str(), 0755) == 0) return true;
    if (errno != EEXIST) return false;
    struct stat st;
    return stat(d.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

std::string box_str(const int* b)
{
    char s[128];
    std::snprintf(s, sizeof s, "((%d,%d,%d) (%d,%d,%d) (0,0,0))", b[0], b[1], b[2], b[3], b[4], b[5]);
    return s;
}

long long box_vol(const int* b)
{
    return (long long)(b[3] - b[0] + 1) * (b[4] - b[1] + 1) * (b[5] - b[2] + 1);
}

std::string fmt17(double v)
{
    char s[64];
    std::snprintf(s, sizeof s, "%.17g", v);
    return s;
}

// the box array as AMReX's BoxArray::writeOn prints it
void write_box_array(std::ostream& os, int nbox, const int* lohi)
{
    os << "(" << nbox << " 0\n";
    for (int n = 0; n < nbox; ++n) os << box_str(lohi + 6 * n) << "\n";
    os << ")";
}

bool parse_box(const std::string& s, size_t& pos, int b[6])
{
    // ((lo0,lo1,lo2) (hi0,hi1,hi2) (t0,t1,t2))
    int t[3];
    const size_t open = s.find("((", pos);
    if (open == std::string::npos) return false;
    const int k = std::sscanf(s.c_str() + open, "((%d,%d,%d) (%d,%d,%d) (%d,%d,%d))", &b[0], &b[1], &b[2], &b[3],
                              &b[4], &b[5], &t[0], &t[1], &t[2]);
    if (k != 9) return false;
    const size_t close = s.find("))", open);
    if (close == std::string::npos) return false;
    pos = close + 2;
    return true;
}

// VisMF::Write equivalent: <prefix>_H and <prefix>_D_00000
mbg_status write_multifab(const std::string& prefix, int nbox, const int* lohi, int ncomp, const double* data)
{
    if (!host_little_endian()) return io_fail("AMReX output: big-endian hosts are not supported");
    const std::string dname = prefix + "_D_00000";
    std::FILE* fd = std::fopen(dname.c_str(), "wb");
    if (!fd) return io_fail("cannot open " + dname + " for writing");
    std::vector<long long> offsets(nbox);
    std::vector<double> mins((size_t)nbox * ncomp), maxs((size_t)nbox * ncomp);
    long long pos = 0, off = 0;
    for (int n = 0; n < nbox; ++n) {
        const int* b = lohi + 6 * n;
        const long long vol = box_vol(b);
        std::string hdr = std::string("FAB ") + FAB_REAL_DESC + box_str(b) + " " + std::to_string(ncomp) + "\n";
        offsets[n] = pos;
        const double* src = data + off * ncomp;
        if (std::fwrite(hdr.data(), 1, hdr.size(), fd) != hdr.size() ||
            std::fwrite(src, sizeof(double), (size_t)vol * ncomp, fd) != (size_t)vol * ncomp) {
            std::fclose(fd);
            return io_fail("write failed: " + dname);
        }
        pos += (long long)hdr.size() + vol * ncomp * (long long)sizeof(double);
        for (int c = 0; c < ncomp; ++c) {
            double lo = std::numeric_limits<double>::infinity(), hi = -lo;
            for (long long i = 0; i < vol; ++i) {
                const double v = src[(size_t)c * vol + i];
                lo = v < lo ? v : lo;
                hi = v > hi ? v : hi;
            }
            mins[(size_t)n * ncomp + c] = lo;
            maxs[(size_t)n * ncomp + c] = hi;
        }
        off += vol;
    }
    if (std::fclose(fd) != 0) return io_fail("write failed: " + dname);
    const std::string hname = prefix + "_H";
    std::ofstream h(hname, std::ios::trunc);
    if (!h) return io_fail("cannot open " + hname + " for writing");
    h << "1\n0\n" << ncomp << "\n0\n";
    write_box_array(h, nbox, lohi);
    h << "\n" << nbox << "\n";
    const std::string base = dname.substr(dname.find_last_of('/') + 1);
    for (int n = 0; n < nbox; ++n) h << "FabOnDisk: " << base << " " << offsets[n] << "\n";
    h << "\n" << nbox << "," << ncomp << "\n";
    for (int n = 0; n < nbox; ++n) {
        for (int c = 0; c < ncomp; ++c) h << fmt17(mins[(size_t)n * ncomp + c]) << ",";
        h << "\n";
    }
    h << "\n" << nbox << "," << ncomp << "\n";
    for (int n = 0; n < nbox; ++n) {
        for (int c = 0; c < ncomp; ++c) h << fmt17(maxs[(size_t)n * ncomp + c]) << ",";
        h << "\n";
    }
    h.close();
    if (!h) return io_fail("write failed: " + hname);
    return MBG_OK;
}

bool read_file(const std::string& name, std::string& out)
{
    std::ifstream in(name, std::ios::binary);
    if (!in) return false;
    std::ostringstream ss;
    ss << in.rdbuf();
    out = ss.str();
    return true;
}

// VisMF::Read equivalent for the boxes given (which must be the file's):
// valid cells of every component, [box][comp][k][j][i]
mbg_status read_multifab(const std::string& prefix, int nbox, const int* lohi, int ncomp, double* data)
{
    std::string H;
    if (!read_file(prefix + "_H", H)) return io_fail("cannot read " + prefix + "_H");
    std::istringstream hs(H);
    int version = 0, how = 0, nc = 0, ngrow = 0;
    hs >> version >> how >> nc;
    std::string ng_tok;
    hs >> ng_tok;   // "0" or "(3,3,3)"-style
    if (ng_tok.size() && ng_tok[0] == '(') {
        int g0 = 0;
        std::sscanf(ng_tok.c_str(), "(%d", &g0);
        ngrow = g0;
    } else {
        ngrow = std::atoi(ng_tok.c_str());
    }
    if (version != 1) return io_fail(prefix + "_H: VisMF header version " + std::to_string(version) + " unsupported");
    if (nc != ncomp)
        return io_fail(prefix + "_H: " + std::to_string(nc) + " components, expected " + std::to_string(ncomp));
    // box array
    size_t pos = (size_t)hs.tellg();
    const size_t lp = H.find('(', pos);
    if (lp == std::string::npos) return io_fail(prefix + "_H: no box array");
    int nb = 0;
    std::sscanf(H.c_str() + lp, "(%d", &nb);
    if (nb != nbox)
        return io_fail(prefix + "_H: " + std::to_string(nb) + " boxes, expected " + std::to_string(nbox));
    pos = H.find('\n', lp);
    for (int n = 0; n < nbox; ++n) {
        int b[6];
        if (!parse_box(H, pos, b)) return io_fail(prefix + "_H: malformed box " + std::to_string(n));
        for (int d = 0; d < 6; ++d)
            if (b[d] != lohi[6 * n + d])
                return io_fail(prefix + "_H: box " + std::to_string(n) + " differs from the level's grids");
    }
    // FabOnDisk entries
    std::vector<std::string> files(nbox);
    std::vector<long long> offs(nbox);
    size_t q = pos;
    for (int n = 0; n < nbox; ++n) {
        q = H.find("FabOnDisk:", q);
        if (q == std::string::npos) return io_fail(prefix + "_H: missing FabOnDisk entry");
        char fname[512];
        long long o = 0;
        if (std::sscanf(H.c_str() + q, "FabOnDisk: %511s %lld", fname, &o) != 2)
            return io_fail(prefix + "_H: malformed FabOnDisk entry");
        files[n] = fname;
        offs[n] = o;
        q += 10;
    }
    const std::string dir = prefix.substr(0, prefix.find_last_of('/') + 1);
    long long off = 0;
    for (int n = 0; n < nbox; ++n) {
        const int* b = lohi + 6 * n;
        const long long vol = box_vol(b);
        std::FILE* fd = std::fopen((dir + files[n]).c_str(), "rb");
        if (!fd) return io_fail("cannot read " + dir + files[n]);
        if (std::fseek(fd, (long)offs[n], SEEK_SET) != 0) {
            std::fclose(fd);
            return io_fail("seek failed in " + files[n]);
        }
        char line[512];
        if (!std::fgets(line, sizeof line, fd) || std::strncmp(line, "FAB ", 4) != 0) {
            std::fclose(fd);
            return io_fail(files[n] + ": no FAB header at offset " + std::to_string(offs[n]));
        }
        if (!std::strstr(line, "(8, (1 2 3 4 5 6 7 8))") || !std::strstr(line, "(64 11 52 0 1 12 0 1023)")) {
            std::fclose(fd);
            return io_fail(files[n] + ": only little-endian IEEE double FABs are supported");
        }
        // the FAB's own box (grown by ngrow when the file carries ghosts)
        int fb[6];
        size_t lpos = 0;
        const std::string ls(line);
        const size_t bstart = ls.find(")))");
        lpos = bstart == std::string::npos ? 0 : bstart + 3;
        if (!parse_box(ls, lpos, fb)) {
            std::fclose(fd);
            return io_fail(files[n] + ": malformed FAB box");
        }
        for (int d = 0; d < 3; ++d)
            if (fb[d] != b[d] - ngrow || fb[d + 3] != b[d + 3] + ngrow) {
                std::fclose(fd);
                return io_fail(files[n] + ": FAB box does not match the box grown by " + std::to_string(ngrow));
            }
        const int gx = fb[3] - fb[0] + 1, gy = fb[4] - fb[1] + 1, gz = fb[5] - fb[2] + 1;
        std::vector<double> buf((size_t)gx * gy * gz);
        double* dst = data + off * ncomp;
        const int nx = b[3] - b[0] + 1, ny = b[4] - b[1] + 1, nz = b[5] - b[2] + 1;
        for (int c = 0; c < ncomp; ++c) {
            if (std::fread(buf.data(), sizeof(double), buf.size(), fd) != buf.size()) {
                std::fclose(fd);
                return io_fail(files[n] + ": short read");
            }
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    std::memcpy(dst + (size_t)c * vol + ((size_t)k * ny + j) * nx,
                                buf.data() + ((size_t)(k + ngrow) * gy + (j + ngrow)) * gx + ngrow,
                                (size_t)nx * sizeof(double));
        }
        std::fclose(fd);
        off += vol;
    }
    return MBG_OK;
}

}  // namespace

extern "C" {

mbg_status mbg_write_multifab(const char* prefix, int nbox, const int* lohi, int ncomp, const double* data)
{
    if (!prefix || nbox < 0 || (nbox > 0 && (!lohi || !data)) || ncomp < 1)
        return io_fail("mbg_write_multifab: bad argument");
    return write_multifab(prefix, nbox, lohi, ncomp, data);
}

mbg_status mbg_read_multifab(const char* prefix, int nbox, const int* lohi, int ncomp, double* data)
{
    if (!prefix || nbox < 0 || (nbox > 0 && (!lohi || !data)) || ncomp < 1)
        return io_fail("mbg_read_multifab: bad argument");
    return read_multifab(prefix, nbox, lohi, ncomp, data);
}

mbg_status mbg_write_plotfile(const char* dir, int nlev, const int* nbox, const int* lohi, const int* n_cell,
                              const double* prob_lo, const double* prob_hi, int ncomp,
                              const char* const* varnames, const double* const* data, double time,
                              const int* level_steps)
{
    if (!dir || nlev < 1 || !nbox || !lohi || !n_cell || !prob_lo || !prob_hi || ncomp < 1 || !varnames || !data ||
        !level_steps)
        return io_fail("mbg_write_plotfile: bad argument");
    const std::string root(dir);
    if (!make_dir(root)) return io_fail("mbg_write_plotfile: cannot create directory " + root);
    std::ofstream h(root + "/Header", std::ios::trunc);
    if (!h) return io_fail("mbg_write_plotfile: cannot open " + root + "/Header");
    h << "HyperCLaw-V1.1\n" << ncomp << "\n";
    for (int c = 0; c < ncomp; ++c) h << varnames[c] << "\n";
    h << "3\n" << fmt17(time) << "\n" << nlev - 1 << "\n";
    h << fmt17(prob_lo[0]) << " " << fmt17(prob_lo[1]) << " " << fmt17(prob_lo[2]) << "\n";
    h << fmt17(prob_hi[0]) << " " << fmt17(prob_hi[1]) << " " << fmt17(prob_hi[2]) << "\n";
    for (int l = 0; l + 1 < nlev; ++l) h << 2 << " ";
    h << "\n";
    for (int l = 0; l < nlev; ++l) {
        const int r = 1 << l;
        const int dom[6] = {0, 0, 0, n_cell[0] * r - 1, n_cell[1] * r - 1, n_cell[2] * r - 1};
        h << box_str(dom) << " ";
    }
    h << "\n";
    for (int l = 0; l < nlev; ++l) h << level_steps[l] << " ";
    h << "\n";
    std::vector<std::vector<double>> dx(nlev, std::vector<double>(3));
    for (int l = 0; l < nlev; ++l) {
        for (int d = 0; d < 3; ++d) {
            dx[l][d] = (prob_hi[d] - prob_lo[d]) / ((double)n_cell[d] * (1 << l));
            h << fmt17(dx[l][d]) << (d < 2 ? " " : "\n");
        }
    }
    h << "0\n0\n";
    long long boff = 0;
    for (int l = 0; l < nlev; ++l) {
        h << l << " " << nbox[l] << " " << fmt17(time) << "\n" << level_steps[l] << "\n";
        for (int n = 0; n < nbox[l]; ++n) {
            const int* b = lohi + 6 * (boff + n);
            for (int d = 0; d < 3; ++d)
                h << fmt17(prob_lo[d] + b[d] * dx[l][d]) << " " << fmt17(prob_lo[d] + (b[d + 3] + 1) * dx[l][d])
                  << "\n";
        }
        h << "Level_" << l << "/Cell\n";
        boff += nbox[l];
    }
    h.close();
    if (!h) return io_fail("mbg_write_plotfile: write failed: " + root + "/Header");
    boff = 0;
    for (int l = 0; l < nlev; ++l) {
        const std::string ld = root + "/Level_" + std::to_string(l);
        if (!make_dir(ld)) return io_fail("mbg_write_plotfile: cannot create directory " + ld);
        mbg_status st = write_multifab(ld + "/Cell", nbox[l], lohi + 6 * boff, ncomp, data[l]);
        if (st != MBG_OK) return st;
        boff += nbox[l];
    }
    return MBG_OK;
}

}  // extern "C"
