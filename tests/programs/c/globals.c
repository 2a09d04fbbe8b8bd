/* Per-rank globals after conversion: every variable with static storage must behave as if each rank were
 * its own process.  Each rank stores rank-dependent values into every kind of global, waits for all
 * ranks, then checks that it reads back its own values and that untouched elements keep their
 * initializers.  Returns the number of failed checks (0 = all good). */
#include <mpi.h>
#include <stdio.h>

extern int counter;
extern int counter;
int counter = 7;
double weights[3] = { 0.5, 1.5, 2.5 };
int *slots[2] = { NULL, NULL }, grid[2][4] = { { 1, 2, 3, 4 }, { 5, 6, 7, 8 } };
static long hidden = -3;
struct pair { int a, b; } couple = { 10, 20 };
int (*op_ptr)(int, int);
char tag = 'x';

#define CHECK(c) do { if (!(c)) { printf("rank %d: check failed: %s\n", rank, #c); bad++; } } while (0)
#define WEIGHT0 weights[0]

int add(int x, int y) { return x + y; }
int mul(int x, int y) { return x * y; }

int bump(void)
{
    static int calls = 100;
    calls += 1;
    return calls;
}

int shadow(int counter)
{
    return counter * 2;   /* the parameter, not the global */
}

int main(void)
{
    int rank = -1, bad = 0, size = 0;
    MPI_Init(0, 0);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);

    CHECK(counter == 7);
    CHECK(weights[2] == 2.5);
    CHECK(grid[1][3] == 8);
    CHECK(hidden == -3);
    CHECK(couple.b == 20);
    CHECK(tag == 'x');

    counter = rank;
    WEIGHT0 = rank + 0.25;
    slots[1] = &counter;
    grid[0][rank % 4] = 100 + rank;
    hidden = -rank;
    couple.a = rank * 3;
    op_ptr = (rank % 2) ? mul : add;
    tag = (char)('a' + rank % 26);
    bump();
    bump();
    {
        int counter = -1;         /* a local shadowing the global */
        counter += 1;
        CHECK(counter == 0);
    }
    for (int weights = 0; weights < 1; weights++)   /* shadowing in a for-init */
        CHECK(weights == 0);

    MPI_Barrier(MPI_COMM_WORLD);

    CHECK(counter == rank);
    CHECK(shadow(21) == 42);
    CHECK(weights[0] == rank + 0.25);
    CHECK(weights[1] == 1.5);
    CHECK(slots[1] == &counter);
    CHECK(*slots[1] == rank);
    CHECK(slots[0] == NULL);
    CHECK(grid[0][rank % 4] == 100 + rank);
    CHECK(grid[1][0] == 5);
    CHECK(hidden == -rank);
    CHECK(couple.a == rank * 3 && couple.b == 20);
    CHECK(op_ptr(6, 7) == ((rank % 2) ? 42 : 13));
    CHECK(tag == (char)('a' + rank % 26));
    CHECK(bump() == 103);

    int total = 0;
    MPI_Allreduce(&counter, &total, 1, MPI_INT, MPI_SUM, MPI_COMM_WORLD);
    CHECK(total == size * (size - 1) / 2);
    if (rank == 0)
        printf("globals: %d ranks, %s\n", size, bad ? "FAILED" : "ok");
    MPI_Finalize();
    return bad;
}
