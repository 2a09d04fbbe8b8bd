/* C idioms a C++ compiler rejects, which the converter must rewrite: implicit conversions from void*,
 * identifiers that are C++ keywords, old-style definitions (in oldstyle_lib.c), plus string and number
 * functions of the C library and a derived datatype.  Rank 0 sends 100 chars as one contiguous type to
 * rank 1; every rank builds records on the heap, and the ranks' checksums are summed.  Prints one line
 * from rank 0; returns the number of failed checks. */
#include "mpi.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "oldstyle.h"

static int failures = 0;

static void expect(int cond, const char *what, int rank)
{
    if (!cond) {
        printf("rank %d: %s\n", rank, what);
        failures++;
    }
}

int main(int argc, char **argv)
{
    int rank, size, i, new = 0, class = 0;
    char this[100];
    MPI_Datatype hundred;
    MPI_Status status;
    record *recs;
    int *counts;
    long total = 0, mine;

    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);

    MPI_Type_contiguous(100, MPI_CHAR, &hundred);
    MPI_Type_commit(&hundred);
    for (i = 0; i < 100; i++)
        this[i] = (char)(rank == 0 ? 'A' + i % 26 : 0);
    if (size > 1) {
        if (rank == 0)
            MPI_Send(this, 1, hundred, 1, 123, MPI_COMM_WORLD);
        else if (rank == 1)
            MPI_Recv(this, 1, hundred, 0, 123, MPI_COMM_WORLD, &status);
    }
    if (rank <= 1 && size > 1)
        expect(this[27] == 'B' && this[99] == 'A' + 99 % 26, "contiguous type transfer", rank);
    MPI_Type_free(&hundred);

    recs = malloc(3 * sizeof(record));
    counts = calloc(4, sizeof(int));
    for (i = 0; i < 3; i++) {
        recs[i].id = rank * 10 + i;
        recs[i].value = scaled(0.5, i + 1);
        strcpy(recs[i].label, "rec");
        strcat(recs[i].label, i == 0 ? "-a" : "-b");
        counts[i] = (int)strlen(recs[i].label);
    }
    expect(strcmp(recs[0].label, "rec-a") == 0 && strncmp(recs[2].label, "rec-b", 5) == 0, "string functions", rank);
    expect(counts[1] == 5 && counts[3] == 0, "calloc zeroes", rank);
    expect(atoi("  -42x") == -42 && strtol("0x1f", NULL, 0) == 31 && atof("2.5e2") == 250.0, "number parsing", rank);
    expect(strchr("abc", 'c') != NULL && strstr("needle in hay", "in") != NULL, "searching", rank);
    new = recs[2].id;
    class = lib_calls;
    expect(new == rank * 10 + 2 && class == 3, "keyword identifiers", rank);

    mine = checksum(recs[rank % 3].label) + rank;
    MPI_Allreduce(&mine, &total, 1, MPI_LONG, MPI_SUM, MPI_COMM_WORLD);
    free(recs);
    free(counts);
    if (rank == 0)
        printf("oldstyle: %d ranks, total %ld, failures %d\n", size, total, failures);
    MPI_Finalize();
    return failures;
}
