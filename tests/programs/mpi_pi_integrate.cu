// A plain MPI program in the form the reference's source converter produces (main renamed
// __gpu_main, every function __device__): pi by the midpoint rule on 4 / (1 + x^2) over [0, 1].
// Rank 0 broadcasts the interval count, every rank sums its strided share, MPI_Reduce adds the shares
// on rank 0, which prints the result.  A per-rank global (the converter's __gpu_global(var) form) counts
// each rank's terms; their sum, reduced to rank 0, must be the interval count.
// Arguments: [intervals] [rank that fails on purpose].
#include <mpi.h.cuh>

#include <cstdio>

__device__ long long terms[4096];  // one slot per rank: a converted program's global

__device__ long long parse_ll(const char* s) {
    long long v = 0;
    bool neg = false;
    if (*s == '-') {
        neg = true;
        s++;
    }
    while (*s >= '0' && *s <= '9') v = v * 10 + (*s++ - '0');
    return neg ? -v : v;
}

__device__ int __gpu_main(int argc, char* argv[]) {
    MPI_Init(&argc, &argv);
    int rank = 0, size = 1;
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    long long n = 0;
    if (rank == 0) n = argc > 1 ? parse_ll(argv[1]) : 100000;
    MPI_Bcast(&n, 1, MPI_LONG_LONG, 0, MPI_COMM_WORLD);
    const int fail_rank = argc > 2 ? (int)parse_ll(argv[2]) : -1;
    const double h = 1.0 / (double)n;
    double sum = 0.0;
    __gpu_global(terms) = 0;
    for (long long i = rank; i < n; i += size) {
        const double x = h * ((double)i + 0.5);
        sum += 4.0 / (1.0 + x * x);
        __gpu_global(terms)++;
    }
    double mine = h * sum, pi = 0.0;
    long long all_terms = 0;
    MPI_Reduce(&mine, &pi, 1, MPI_DOUBLE, MPI_SUM, 0, MPI_COMM_WORLD);
    MPI_Reduce(&__gpu_global(terms), &all_terms, 1, MPI_LONG_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
    if (rank == 0) printf("pi %.15f ranks %d intervals %lld terms %lld\n", pi, size, n, all_terms);
    MPI_Finalize();
    return rank == fail_rank ? 3 : 0;
}
