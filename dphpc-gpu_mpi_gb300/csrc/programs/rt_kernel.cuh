// rt_kernel.cuh — the persistent rank kernel and its launcher, for translation units that define
// device programs (the built-in ones here; a converted program's __gpu_main in the same way).
//
// Replaces gpu_libs/gpu_main/main.cu:102-130 (__gpu_main_caller, one thread per rank) and the test
// harness kernel of tests/test_runner.cuh:11-24.  Block b < nranks runs the program as MPI rank b on
// its thread 0 while the other threads serve the block tasks the MPI calls dispatch; blocks >= nranks
// are copy-engine blocks.  The launch is cooperative, so all blocks are guaranteed co-resident (the
// reference checks this by hand, main.cu:188-208).
#pragma once
#include <cuda_runtime.h>

#include "gpumpi.h"
#include "mpi.h.cuh"

namespace gpumpi {
__device__ void helper_loop();
__device__ int is_rank_block();
__device__ void rank_begin();
__device__ void rank_finish(int rc);
__device__ void engine_main();
}  // namespace gpumpi

__device__ MPI_Op gpumpi_predefined_op(int code);

// At most 64 registers per thread (256 threads x 4 blocks, or 128 x 8, fill an SM's register file):
// the rank count a launch can co-host is set by this.  The runtime's device functions are compiled
// with the same cap; the bound keeps a program's own code (inlined into the kernel) from raising it.
template <class P>
__global__ void __launch_bounds__(256, 4) gpumpi_rank_kernel(gpumpi_params prm) {
    if (threadIdx.x != 0) {
        gpumpi::helper_loop();
        return;
    }
    if (gpumpi::is_rank_block()) {
        gpumpi::rank_begin();
        int rc = P::run(prm);
        gpumpi::rank_finish(rc);
    } else {
        gpumpi::engine_main();
    }
}

typedef cudaError_t (*gpumpi_launch_fn)(int grid, int block, size_t smem, cudaStream_t s, const gpumpi_params* p);
typedef cudaError_t (*gpumpi_occ_fn)(int* blocks_per_sm, int block, size_t smem);
typedef cudaError_t (*gpumpi_attr_fn)(cudaFuncAttributes* attr);

struct gpumpi_prog_entry {
    int id;
    const char* name;
    gpumpi_launch_fn launch;
    gpumpi_occ_fn occupancy;
    gpumpi_attr_fn attributes;
};

template <class P>
cudaError_t gpumpi_launch_prog(int grid, int block, size_t smem, cudaStream_t s, const gpumpi_params* p) {
    gpumpi_params copy = *p;
    void* args[] = {(void*)&copy};
    return cudaLaunchCooperativeKernel((const void*)gpumpi_rank_kernel<P>, dim3(grid), dim3(block), args, smem, s);
}

template <class P>
cudaError_t gpumpi_occ_prog(int* blocks_per_sm, int block, size_t smem) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, gpumpi_rank_kernel<P>, block, smem);
}

template <class P>
cudaError_t gpumpi_attr_prog(cudaFuncAttributes* attr) {
    return cudaFuncGetAttributes(attr, gpumpi_rank_kernel<P>);
}

#define GPUMPI_PROGRAM(ID, NAME, TYPE) \
    { ID, NAME, &gpumpi_launch_prog<TYPE>, &gpumpi_occ_prog<TYPE>, &gpumpi_attr_prog<TYPE> }
