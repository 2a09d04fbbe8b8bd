// user_main.cu — the entry of an executable built around a converted program (the reference's
// gpumpicc output linked with libgpu_main, gpu_libs/gpu_main/main.cu): the program's
// `__device__ int __gpu_main(int, char**)` (source_converter/converter.cpp:49-65) becomes program
// GPUMPI_P_USER of the rank kernel, and main() hands the command line to the launcher, gpumpi_main.
// Compiled only by the program builder (build.py --program), together with the runtime's objects.
#include "rt_kernel.cuh"

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

int main(int argc, char** argv) { return gpumpi_main(argc, argv, GPUMPI_P_USER); }
