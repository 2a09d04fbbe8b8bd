// A plain MPI program in the converter's output form (main renamed __gpu_main) that uses the calls a
// classic pi example makes around its computation: every rank reports where it runs on stderr
// (MPI_Get_processor_name, fprintf), rank 0 takes the interval count from its arguments, broadcasts it,
// times the run with MPI_Wtime and prints the estimate, its error against the known value and the elapsed
// wall time on stdout, then flushes.  The integral is 4 / (1 + x^2) over [0, 1] by the midpoint rule,
// each rank summing every size-th interval.  Output goes through the host channel (GPUMPI_STDIO_NAMES).
// Arguments: [intervals].
#define GPUMPI_STDIO_NAMES
#include <mpi.h.cuh>
#include <gpumpi_stdio.h.cuh>

__device__ int parse_int(const char* s) {
    int v = 0;
    while (*s >= '0' && *s <= '9') v = v * 10 + (*s++ - '0');
    return v;
}

__device__ int __gpu_main(int argc, char* argv[]) {
    const double known_pi = 3.141592653589793238462643;
    MPI_Init(&argc, &argv);
    int rank = 0, size = 1, len = 0;
    char host[MPI_MAX_PROCESSOR_NAME];
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    MPI_Get_processor_name(host, &len);
    fprintf(stderr, "rank %d of %d runs on %s\n", rank, size, host);

    int intervals = 0;
    double t0 = 0.0;
    if (rank == 0) {
        intervals = argc > 1 ? parse_int(argv[1]) : 10000;
        t0 = MPI_Wtime();
    }
    MPI_Bcast(&intervals, 1, MPI_INT, 0, MPI_COMM_WORLD);
    const double h = 1.0 / (double)intervals;
    double part = 0.0;
    for (int i = rank + 1; i <= intervals; i += size) {
        const double x = h * ((double)i - 0.5);
        part += 4.0 / (1.0 + x * x);
    }
    part *= h;
    double pi = 0.0;
    MPI_Reduce(&part, &pi, 1, MPI_DOUBLE, MPI_SUM, 0, MPI_COMM_WORLD);
    if (rank == 0) {
        const double err = pi > known_pi ? pi - known_pi : known_pi - pi;
        printf("pi estimate %.16f, error %.16f\n", pi, err);
        printf("elapsed %f s\n", MPI_Wtime() - t0);
        fflush(stdout);
    }
    MPI_Finalize();
    return 0;
}
