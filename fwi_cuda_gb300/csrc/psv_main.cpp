// seis_fwi: the reference's program (src/h_main.cpp: simulate_PSV() between
// two clock reads, then "total time taken") on the GB300 engine.  Reads
// bin/*.bin (and io/*.bin for FWI) under the working directory, or under the
// directory given as the first argument, and writes the reference's output
// files there (psv_simulate_PSV).  An optional second argument caps the FWI
// iterations (0, the default, keeps the reference's cap).  The reference's
// program runs its CPU path, so the imaging sign is the CPU one.  Where the
// reference prints and exits 0 on an error, this prints the status and
// exits 1.
#include <chrono>
#include <cstdio>
#include <cstdlib>

#include "fwi_psv.h"

int main(int argc, char **argv)
{
    const char *dir = argc > 1 ? argv[1] : ".";
    const int max_iter = argc > 2 ? std::atoi(argv[2]) : 0;
    const auto t0 = std::chrono::steady_clock::now();
    const int st = psv_simulate_PSV(dir, max_iter, -1, nullptr);
    const double s =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st != PSV_OK) {
        std::fprintf(stderr, "seis_fwi: %s: %s\n", psv_error_string(st), psv_last_error());
        return 1;
    }
    std::printf("total time taken %g\n", s);
    return 0;
}
