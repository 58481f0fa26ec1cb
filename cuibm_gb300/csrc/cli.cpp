// The command-line program (src/cuIBM.cu:25-75 main): reads the case folder and the
// command-line overrides, creates and initialises the solver, steps it until nt,
// writing the output after every step, and shuts it down - through the C ABI only.
//
//   cuibm -caseFolder <folder> [-nu V] [-dt V] [-nt N] [-nsave N] [-deviceNumber D] ...
//
// Exit status 0 on success, else the failing call's status (message on stderr), where
// the reference would call exit(-1) from inside the solver.
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/cuibm.h"

static int report(const char *what, int st, const cuibm_ctx *ctx)
{
    std::fprintf(stderr, "cuibm: %s failed (status %d): %s\n", what, st,
                 ctx ? cuibm_last_error(ctx) : cuibm_case_error());
    return st;
}

int main(int argc, char **argv)
{
    std::string folder = ".";
    std::vector<const char *> overrides;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "-caseFolder" && i + 1 < argc) {
            folder = argv[++i];
            continue;
        }
        overrides.push_back(argv[i]);
    }
    cuibm_ctx *ctx = nullptr;
    int st = cuibm_create(folder.c_str(), (int)overrides.size(), overrides.data(), &ctx);
    if (st != CUIBM_OK) return report("reading the case", st, nullptr);
    cuibm_info info;
    if ((st = cuibm_initialise(ctx)) != CUIBM_OK || (st = cuibm_get_info(ctx, &info)) != CUIBM_OK) {
        report("initialise", st, ctx);
        cuibm_destroy(ctx);
        return st;
    }
    std::printf("cuibm: %s, %d x %d cells, solver type %d, %d steps of %g\n", folder.c_str(), info.nx, info.ny,
                info.solver_type, info.nt, info.dt);
    while (!cuibm_finished(ctx)) {
        if ((st = cuibm_step(ctx, 1)) != CUIBM_OK || (st = cuibm_write_data(ctx)) != CUIBM_OK) {
            report("time step", st, ctx);
            cuibm_shutdown(ctx);
            cuibm_destroy(ctx);
            return st;
        }
    }
    int itv = 0, itp = 0;
    cuibm_get_iterations(ctx, &itv, &itp);
    std::printf("cuibm: done; last step's iterations: velocity %d, Poisson %d\n", itv, itp);
    cuibm_shutdown(ctx);
    cuibm_destroy(ctx);
    return 0;
}
