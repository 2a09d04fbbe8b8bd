// prog_apps.cu — application programs built on the MPI surface (filled in below).
#include "rt_kernel.cuh"

extern const gpumpi_prog_entry g_app_programs[] = {
    {-1, "none", nullptr, nullptr, nullptr},
};
extern const int g_num_app_programs = 0;
