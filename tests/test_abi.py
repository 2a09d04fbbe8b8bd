"""CPU: the C-ABI library builds for sm_103a, loads, and exports every entry point include/gpumpi.h
declares (no compute call: there is no GPU here)."""
import ctypes
import re
import shutil
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "gpumpi.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const char\*|int|double|long long)\s+(gpumpi_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def built():
    if not shutil.which("nvcc") and not Path("/usr/local/cuda/bin/nvcc").exists():
        pytest.skip("nvcc not available")
    import gpumpi
    return gpumpi.build()


def test_header_and_python_mirror_agree():
    import gpumpi
    assert declared_functions() == sorted(gpumpi.EXPORTS)


def test_tuning_keys_match_the_header():
    import gpumpi
    text = (ROOT / "include" / "gpumpi.h").read_text()
    keys = dict(re.findall(r"^#define GPUMPI_(TUNE_\w+) (\d+)", text, re.M))
    assert keys and all(getattr(gpumpi, k) == int(v) for k, v in keys.items())


def test_library_exports_every_declared_symbol(built):
    L = ctypes.CDLL(str(built))
    for name in declared_functions():
        assert hasattr(L, name), name


def test_config_defaults_and_arg_parsing(built):
    import gpumpi
    L = gpumpi.lib()
    c = gpumpi.Config()
    assert L.gpumpi_config_init(ctypes.byref(c)) == 0
    assert c.pending_requests == 1024 and c.engine_blocks == -1 and c.eager_bytes == 1024
    argv = [b"prog", b"x", b"---gpumpi", b"-n", b"64", b"-b", b"128", b"-e", b"40", b"-s", b"4096"]
    arr = (ctypes.c_char_p * len(argv))(*argv)
    pos = L.gpumpi_parse_args(len(argv), arr, ctypes.byref(c))
    assert pos == 2 and c.nranks == 64 and c.threads_per_block == 128 and c.pending_requests == 40
    assert c.stack_bytes == 4096
    arr2 = (ctypes.c_char_p * 2)(b"prog", b"x")
    assert L.gpumpi_parse_args(2, arr2, ctypes.byref(c)) == -1


def test_abi_constants_match_reference_order():
    # datatype enum order of gpu_libs/gpu_mpi/mpi_types_list.cuh:3-33 and op order of mpi_operators_list.cuh
    text = (ROOT / "include" / "gpumpi_abi.h").read_text()
    vals = dict(re.findall(r"#define GPUMPI_(\w+)\s+(-?\d+)", text))
    order = ["CHAR", "SHORT", "INT", "LONG", "LONG_LONG_INT", "LONG_LONG", "SIGNED_CHAR", "UNSIGNED_CHAR",
             "UNSIGNED_SHORT", "UNSIGNED", "UNSIGNED_LONG", "UNSIGNED_LONG_LONG", "FLOAT", "DOUBLE", "LONG_DOUBLE",
             "WCHAR", "C_BOOL", "INT8_T", "INT16_T", "INT32_T", "INT64_T", "UINT8_T", "UINT16_T", "UINT32_T",
             "UINT64_T", "C_COMPLEX", "C_FLOAT_COMPLEX", "C_DOUBLE_COMPLEX", "C_LONG_DOUBLE_COMPLEX", "BYTE"]
    assert [int(vals[k]) for k in order] == list(range(30))
    ops = ["MAX", "MIN", "SUM", "PROD", "LAND", "BAND", "LOR", "BOR", "LXOR", "BXOR", "MAXLOC", "MINLOC"]
    assert [int(vals["OP_" + k]) for k in ops] == list(range(12))
    assert vals["SUCCESS"] == "0" and vals["ERR_OTHER"] == "1"


def test_product_path_has_no_oracle_dependency():
    # the product package must never import or link the oracle
    pkg = ROOT / "dphpc-gpu_mpi_gb300"
    for p in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cuh")):
        t = p.read_text()
        for pat in ("import oracle", "from oracle", "liboracle", "oracle/", "gpumpi_oracle"):
            assert pat not in t, (p, pat)


def test_device_header_declares_the_reference_surface():
    """Every __device__ MPI function the reference's headers declare (mpi.cuh, communicator.cuh,
    group.cuh, io.cuh; names recorded in tests/golden/reference_device_api.json by make_api_list.py) is declared
    by include/mpi.h.cuh, so a converted program that calls any of them links."""
    import json
    names = json.loads((ROOT / "tests" / "golden" / "reference_device_api.json").read_text())
    text = (ROOT / "include" / "mpi.h.cuh").read_text()
    ours = set(re.findall(r"__device__[^;(]*?\b(MPI_\w+)\s*\(", text))
    for header in ("mpi.cuh", "communicator.cuh", "group.cuh", "io.cuh"):
        # io.cuh's MPI_File_View is the constructor of the reference's internal view struct, not an API call
        missing = sorted(set(names[header]) - ours - {"MPI_File_View"})
        assert not missing, (header, missing)
    # the typedefs the keyval functions take
    for t in ("MPI_Copy_function", "MPI_Delete_function"):
        assert re.search(r"typedef\s+int\s+" + t + r"\s*\(", text), t
