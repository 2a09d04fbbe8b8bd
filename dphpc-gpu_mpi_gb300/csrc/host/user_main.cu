// user_main.cu — the entry of an executable built around a converted program (the reference's
// gpumpicc output linked with libgpu_main, gpu_libs/gpu_main/main.cu): the program's
// `__device__ int __gpu_main(int, char**)` (source_converter/converter.cpp:49-65) becomes program
// GPUMPI_P_USER of the rank kernel, and main() hands the command line to the launcher, gpumpi_main.
// Compiled only by the program builder (build.py --program), together with the runtime's objects.
#include "rt_kernel.cuh"

#include <cstdio>

#include "gpumpi.h"

extern __device__ int __gpu_main(int argc, char* argv[]);

namespace {
struct UserMain {
    static __device__ int run(const gpumpi_params& p) { return __gpu_main((int)p.i[0], (char**)p.p[0]); }
};
}  // namespace

extern const gpumpi_prog_entry g_user_programs[] = {
    GPUMPI_PROGRAM(GPUMPI_P_USER, "user", UserMain),
};
extern const int g_num_user_programs = 1;

// A program written out by the source converter (gpumpi/converter.py) holds its globals in arrays of one
// element per rank and records their length here; hand-written programs define nothing.
extern "C" const int gpumpi_program_max_ranks __attribute__((weak));

int main(int argc, char** argv) {
    if (&gpumpi_program_max_ranks != nullptr) {
        gpumpi_config cfg;
        gpumpi_config_init(&cfg);
        gpumpi_parse_args(argc, argv, &cfg);
        if (cfg.nranks > gpumpi_program_max_ranks) {
            fprintf(stderr, "gpumpi: %d ranks requested, but the program was converted for at most %d "
                            "(its per-rank globals hold that many; convert it with GPU_MPI_MAX_RANKS raised)\n",
                    cfg.nranks, gpumpi_program_max_ranks);
            return 1;
        }
    }
    return gpumpi_main(argc, argv, GPUMPI_P_USER);
}
