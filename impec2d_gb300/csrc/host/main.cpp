// Impec2D command-line driver: `Impec2D [config.cfg]`, as the reference's main
// (src/Driver.cpp:58-87) but single-process: one engine per GPU.
#include <cstdio>
#include <string>

#include "impec2d.h"

int main(int argc, char** argv) {
    std::string cfg = argc > 1 ? argv[1] : "parallel.cfg";
    impec_status s = impec_run_cfg(cfg.c_str(), 0);
    if (s != IMPEC_OK) {
        std::fprintf(stderr, "Impec2D: %s failed with status %d\n", cfg.c_str(), (int)s);
        return 1;
    }
    return 0;
}
