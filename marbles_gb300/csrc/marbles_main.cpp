// marbles_main.cpp -- command-line driver with the reference executable's
// calling convention (Source/main.cpp:10-25):
//     marbles_gb300 <inputs file> [key=value ...]
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/marbles_gb300.h"

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s <inputs file> [key=value ...]\n", argv[0]);
        return 2;
    }
    std::ifstream f(argv[1]);
    if (!f) {
        std::fprintf(stderr, "cannot open inputs file %s\n", argv[1]);
        return 2;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    std::vector<const char*> ov(argv + 2, argv + argc);
    mbg_lbm* h = nullptr;
    if (mbg_lbm_create(ss.str().c_str(), (int)ov.size(), ov.data(), &h) != MBG_OK) {
        std::fprintf(stderr, "error: %s\n", mbg_lbm_last_error(nullptr));
        return 1;
    }
    if (mbg_lbm_init(h) != MBG_OK || mbg_lbm_evolve(h, 0) != MBG_OK) {
        std::fprintf(stderr, "error: %s\n", mbg_lbm_last_error(h));
        mbg_lbm_destroy(h);
        return 1;
    }
    mbg_lbm_destroy(h);
    return 0;
}
