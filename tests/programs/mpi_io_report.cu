// A plain MPI program in the converter's output form (main renamed __gpu_main) that writes files and
// prints through the standard C names: each rank sums the squares of its strided share of [0, n), writes
// its partial sum into a shared file at its own offset with MPI-IO, and rank 0 prints the total with
// fprintf(stdout, ...).  GPUMPI_STDIO_NAMES maps FILE, stdout and fprintf onto the host-performed stdio.
// Arguments: [output file] [n].
#define GPUMPI_STDIO_NAMES
#include <mpi.h.cuh>
#include <gpumpi_stdio.h.cuh>

__device__ long long parse_count(const char* s) {
    long long v = 0;
    while (*s >= '0' && *s <= '9') v = v * 10 + (*s++ - '0');
    return v;
}

__device__ int __gpu_main(int argc, char* argv[]) {
    MPI_Init(&argc, &argv);
    int rank = 0, size = 1;
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    const char* out = argc > 1 ? argv[1] : "partial_sums.bin";
    const long long n = argc > 2 ? parse_count(argv[2]) : 1000;
    double mine = 0.0;
    for (long long i = rank; i < n; i += size) mine += (double)i * (double)i;
    MPI_File fh;
    int rc = MPI_File_open(MPI_COMM_WORLD, out, MPI_MODE_CREATE | MPI_MODE_WRONLY, MPI_INFO_NULL, &fh);
    if (rc == MPI_SUCCESS) {
        rc = MPI_File_write_at(fh, (MPI_Offset)rank * (MPI_Offset)sizeof(double), &mine, 1, MPI_DOUBLE,
                               MPI_STATUS_IGNORE);
        MPI_File_close(&fh);
    }
    double total = 0.0;
    MPI_Reduce(&mine, &total, 1, MPI_DOUBLE, MPI_SUM, 0, MPI_COMM_WORLD);
    if (rank == 0) fprintf(stdout, "sum of squares below %lld over %d ranks: %.1f\n", n, size, total);
    MPI_Finalize();
    return rc == MPI_SUCCESS ? 0 : 2;
}
