// yk_run_main.cpp -- `yk_run input.toml [out_dir]`: the drop-in for the
// reference's `./out input.toml` (code/src/main.cu:73-86, code/runbw.sh:14).
#include <cstdio>

#include "yukawa.h"

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "No input file provided.\nExiting.\n");
        return 1;
    }
    const int rc = yk_run_toml(argv[1], argc > 2 ? argv[2] : "");
    if (rc != YK_OK) {
        std::fprintf(stderr, "yk_run: %s (status %d)\n", yk_last_error(), rc);
        return 2;
    }
    return 0;
}
