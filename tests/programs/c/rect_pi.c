/* Pi by the midpoint rule on 4 / (1 + x^2) over [0, 1], the way classic MPI examples compute it: every
 * rank names its processor, rank 0 reads the interval count from argv and broadcasts it, each rank sums
 * every size-th interval, MPI_Reduce adds the parts on rank 0, which prints the estimate, its error and
 * the elapsed time.  Plain C: built by gpumpicc (source converter + runtime). */
#include "mpi.h"
#include <stdio.h>
#include <stdlib.h>
#include <math.h>

double height(double);

double height(double x)
{
    return 4.0 / (1.0 + x * x);
}

int main(int argc, char *argv[])
{
    int intervals, me, ranks, k, len;
    const double reference_pi = 3.141592653589793238462643;
    double part, pi, width, acc, mid;
    double t_start = 0.0, t_end;
    char where[MPI_MAX_PROCESSOR_NAME];

    MPI_Init(&argc, &argv);
    MPI_Comm_size(MPI_COMM_WORLD, &ranks);
    MPI_Comm_rank(MPI_COMM_WORLD, &me);
    MPI_Get_processor_name(where, &len);
    fprintf(stdout, "rank %d/%d on %s\n", me, ranks, where);
    fflush(stdout);

    intervals = argc > 1 ? atoi(argv[1]) : 10000;
    if (me == 0)
        t_start = MPI_Wtime();
    MPI_Bcast(&intervals, 1, MPI_INT, 0, MPI_COMM_WORLD);

    width = 1.0 / (double)intervals;
    acc = 0.0;
    for (k = me + 1; k <= intervals; k += ranks) {
        mid = width * ((double)k - 0.5);
        acc += height(mid);
    }
    part = width * acc;
    MPI_Reduce(&part, &pi, 1, MPI_DOUBLE, MPI_SUM, 0, MPI_COMM_WORLD);

    if (me == 0) {
        t_end = MPI_Wtime();
        printf("pi = %.16f, error = %.16f\n", pi, fabs(pi - reference_pi));
        printf("time = %f\n", t_end - t_start);
        fflush(stdout);
    }
    MPI_Finalize();
}
