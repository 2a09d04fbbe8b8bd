"""Writes tests/golden/reference_device_api.json: the names of the __device__ MPI functions that the
reference's public headers declare (gpu_libs/gpu_mpi/{mpi,communicator,group,io}.cuh), so the CPU suite
can check that include/mpi.h.cuh declares each of them without reading the reference at test time.

Run from the repository root with the reference checked out beside it:
    python tests/golden/make_api_list.py /path/to/dphpc-gpu_mpi
"""
import json
import re
import sys
from pathlib import Path

HEADERS = ["mpi.cuh", "communicator.cuh", "group.cuh", "io.cuh"]


def declared(text: str) -> list:
    # a declaration: `__device__ <return type> MPI_Name(` (possibly with the name on the same line only)
    return sorted(set(re.findall(r"__device__[^;(]*?\b(MPI_\w+)\s*\(", text)))


def main():
    ref = Path(sys.argv[1]) / "gpu_libs" / "gpu_mpi"
    out = {h: declared((ref / h).read_text()) for h in HEADERS}
    dst = Path(__file__).resolve().parent / "reference_device_api.json"
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(dst, {k: len(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
