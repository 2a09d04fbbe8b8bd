"""Generate tests/golden/reference_tests.json: the known answers of the reference's own GPU tests.

Each case restates, in plain Python integer arithmetic, the expected values that a reference test
checks (file:line of the reference's tests/ directory given per case).  Nothing here calls the oracle:
the oracle is checked against these vectors (tests/test_oracle_golden.py), and the GPU path is checked
against both.  Run:  python tests/golden/make_golden.py
"""
import json
from pathlib import Path


def wrap16(v):
    v &= 0xFFFF
    return v - 0x10000 if v >= 0x8000 else v


def main():
    cases = {}

    # tests/cuda_mpi_test.cu:5-36 — rank 0 sends int 3456 to rank 1 (tag 15)
    cases["single_int"] = {"ranks": 2, "recv": {"1": [3456]}}

    # tests/cuda_mpi_test.cu:38-73 — 16-int array 0..15 from rank 0 to rank 1
    cases["transfer_array"] = {"ranks": 2, "recv": {"1": list(range(16))}}

    # tests/cuda_mpi_test.cu:75-127 — bidirectional exchange, rank0 sends i, rank1 sends -i
    cases["send_recv"] = {"ranks": 2, "recv": {"0": [-i for i in range(16)], "1": list(range(16))}}

    # tests/cuda_mpi_test.cu:129-174 — 5 messages of 1,2,4,8,16 ints with tags 10..14 into the same
    # buffer; the final buffer holds the last (16-int) message: (other+1)*i
    cases["repeat_send_recv"] = {"ranks": 2, "recv": {str(r): [((1 - r) + 1) * i for i in range(16)]
                                                       for r in range(2)}}

    # tests/cuda_mpi_test.cu:177-233 — 3-rank ring, both directions, 5 sizes; final buffers hold
    # (prev+1)*i and (next+1)*i
    cases["network_flood"] = {"ranks": 3, "prev": {str(r): [(((r + 2) % 3) + 1) * i for i in range(16)]
                                                   for r in range(3)},
                              "next": {str(r): [(((r + 1) % 3) + 1) * i for i in range(16)] for r in range(3)}}

    # tests/cuda_mpi_test.cu:235-317 — 10 ranks, 20 repeats x 16 ints to every other rank;
    # receiver r's block from sender s, repeat k, element i == i*k*r
    cases["all_to_all"] = {"ranks": 10, "repeats": 20, "elems": 16,
                           "formula": "remote[s][k][i] = i*k*r for s != r"}

    # tests/collectives_test.cu:6-54 — MPI_Reduce int16 PROD, 5 ranks, 14 elements, (r+1)(i+1),
    # int16 wrap-around at every step
    exp = []
    for i in range(14):
        e = 1
        for r in range(5):
            e = wrap16(e * (r + 1) * (i + 1))
        exp.append(e)
    cases["reduce_int16_prod"] = {"ranks": 5, "count": 14, "root": 0, "expected": exp}

    # tests/collectives_test.cu:57-98 — MPI_Allreduce fp64 SUM, 7 ranks, 17 elements, tol 1e-5
    cases["allreduce_f64_sum"] = {"ranks": 7, "count": 17, "tol": 1e-5,
                                  "expected": [float(sum((r + 1) * (i + 1) for r in range(7))) for i in range(17)]}

    # tests/collectives_test.cu:100-141 — MPI_Allgather 7 ranks x 7 ints, (r+1)(i+1)
    cases["allgather_int"] = {"ranks": 7, "count": 7,
                              "expected": [(r + 1) * (i + 1) for r in range(7) for i in range(7)]}

    # tests/collectives_test.cu:144-196 — MPI_Scatter root 2, 5 ranks, 4 ints each; rank gets its rank
    cases["scatter_int"] = {"ranks": 5, "count": 4, "root": 2,
                            "expected": {str(r): [r] * 4 for r in range(5)}}

    # tests/collectives_test.cu:199-288 — MPI_Scatterv root 2, 5 ranks, sizes i+1 packed; rank gets
    # rank+1 copies of its rank
    cases["scatterv_int"] = {"ranks": 5, "root": 2, "sizes": [i + 1 for i in range(5)],
                             "expected": {str(r): [r] * (r + 1) for r in range(5)}}

    # tests/communicator_test.cu:5-25 — MPI_Comm_rank(MPI_COMM_WORLD) == grid rank, 5 ranks
    cases["comm_rank"] = {"ranks": 5, "expected": list(range(5))}

    # tests/communicator_test.cu:27-90 — three dup'ed communicators keep same-tag traffic apart
    cases["comm_dup_isolation"] = {"ranks": 2,
                                   "rank0_data_10_20": [-(i + 1) for i in range(10, 20)],
                                   "rank1_data_0_10": [i + 1 for i in range(10)],
                                   "rank1_data_20_30": [i + 1 for i in range(20, 30)]}

    # tests/communicator_test.cu:93-152 — Comm_split colours/keys over 10 ranks
    colors, keys, newrank, newsize = [], [], [], []
    for rank in range(10):
        if rank < 3:
            c, k, nr, ns = 0, rank, rank, 3
        elif rank < 6:
            c, k, nr, ns = 1, 6 - rank, 5 - rank, 3
        elif rank < 9:
            c, k, nr, ns = 2, 1, rank - 5, 4
        else:
            c, k, nr, ns = 2, 0, 0, 4
        colors.append(c); keys.append(k); newrank.append(nr); newsize.append(ns)
    cases["comm_split"] = {"ranks": 10, "colors": colors, "keys": keys, "newrank": newrank, "newsize": newsize}

    # tests/sample_test.cu — MPI_Init / MPI_Finalize on 5 ranks
    cases["sample"] = {"ranks": 5}

    out = Path(__file__).resolve().parent / "reference_tests.json"
    out.write_text(json.dumps(cases, indent=1, sort_keys=True) + "\n")
    print(out)


if __name__ == "__main__":
    main()
