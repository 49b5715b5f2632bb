// ps_cli.cpp -- ps_gb300, a process-level drop-in for the BOINC app
// period_search (period_search/period_search_BOINC.cpp:147-954).
//
// Reads period_search_in, resumes from period_search_state when present,
// writes or appends period_search_out, all in the working directory (or the
// directory given with --dir).  Exit codes follow the reference: 0 success,
// 2 a size limit, 4 singular ellipsoid fit, 255 (-1) input missing,
// 1 output/checkpoint failure; CUDA problems exit with 10.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "ps_gb300.h"

int main(int argc, char **argv)
{
    ps_options opt{};
    std::string dir = ".";
    int checkpoint_rows = 64;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--device") && i + 1 < argc) opt.device = std::atoi(argv[++i]);
        else if (!std::strcmp(argv[i], "--dir") && i + 1 < argc) dir = argv[++i];
        else if (!std::strcmp(argv[i], "--form") && i + 1 < argc) {
            const char *f = argv[++i];
            opt.form = !std::strcmp(f, "mixed") ? PS_FORM_MIXED : PS_FORM_FP64;
        } else if (!std::strcmp(argv[i], "--checkpoint-rows") && i + 1 < argc)
            checkpoint_rows = std::atoi(argv[++i]);
        else {
            std::fprintf(stderr, "usage: %s [--device N] [--dir D] [--form fp64|mixed] [--checkpoint-rows K]\n",
                         argv[0]);
            return 1;
        }
    }
    std::string in = dir + "/period_search_in", out = dir + "/period_search_out",
                state = dir + "/period_search_state";
    ps_status st = ps_run_files(in.c_str(), out.c_str(), state.c_str(), &opt, checkpoint_rows);
    if (st != PS_OK) std::fprintf(stderr, "ps_gb300: %s\n", ps_status_string(st));
    switch (st) {
    case PS_OK: return 0;
    case PS_ERR_LIMIT: return 2;
    case PS_ERR_SINGULAR: return 4;
    case PS_ERR_IO: return std::fopen(in.c_str(), "r") ? 1 : 255;
    default: return 10;
    }
}
