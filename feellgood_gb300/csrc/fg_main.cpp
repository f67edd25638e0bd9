// fggpu: command-line driver, `fggpu [--seed N] [-v] settings.yml` (or "-" for stdin),
// the counterpart of the reference's `feellgood` executable (src/main.cpp:103-286).
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>

#include "../../include/fggpu.h"

static void on_signal(int) { fg_run_request_stop(); }

int main(int argc, char **argv) {
    unsigned int seed = std::random_device{}();
    int verbose = 0;
    const char *file = nullptr;
    for (int i = 1; i < argc; i++) {
        if (!std::strcmp(argv[i], "--seed") && i + 1 < argc) seed = (unsigned)std::strtoul(argv[++i], nullptr, 10);
        else if (!std::strcmp(argv[i], "-v") || !std::strcmp(argv[i], "--verbose")) verbose = 1;
        else if (!std::strcmp(argv[i], "-h") || !std::strcmp(argv[i], "--help")) {
            std::printf("usage: fggpu [--seed N] [-v] settings.yml|-\n");
            return 0;
        } else file = argv[i];
    }
    if (!file) {
        std::fprintf(stderr, "usage: fggpu [--seed N] [-v] settings.yml|-\n");
        return 1;
    }
    std::signal(SIGINT, on_signal);
    std::signal(SIGTERM, on_signal);
    std::printf("random seed:       %u\nsettings file:     %s\n", seed, file);
    fg_run_report rep;
    const int s = fg_run(file, seed, verbose, &rep);
    if (s != FG_OK) {
        std::fprintf(stderr, "%s\n", fg_run_last_error());
        return 1;
    }
    std::printf("%lld time steps in %.3f s, per time step: %g s\n", rep.steps, rep.wall_s,
                rep.steps ? rep.wall_s / rep.steps : 0.0);
    return 0;
}
