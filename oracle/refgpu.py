"""Builds and runs the REFERENCE gpu_mpi runtime (lilyyangyn/dphpc-gpu_mpi) on the GPU, for comparison.

COMPARATOR / TEST INFRASTRUCTURE ONLY: used by bench.py's reference-runtime leg (and nothing in the
product).  The reference's own sources are never committed here:

* stage(): where the reference checkout exists (REFERENCE_SRC, default /root/reference), copies its
  toolchain test programs (plain C MPI programs, for the source converter's tests) into
  baseline/_ref/toolchain/ and its runtime sources - gpu_libs/gpu_libc, gpu_libs/gpu_mpi, gpu_libs/gpu_main (without main.cu, whose
  launcher is replaced by oracle/refgpu/driver.cu) and common/ - unchanged into baseline/_ref/src/
  (git-ignored; it travels with the working tree to the GPU machine, which has no reference checkout);
* build(): compiles those sources for sm_103a with relocatable device code, exactly as the reference's
  CMake build does for its own targets (gpu_libs/CMakeLists.txt: separable compilation, every source
  directory on the include path), plus the driver and the oracle's generators, into
  oracle/_ref/ref_gpumpi_bench;
* run_allreduce() / run_alltoallv(): run it as a separate process (its own device heap limit, and a
  host time limit), and check its output against the oracle.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
STAGE = ROOT / "baseline" / "_ref" / "src"
OUT = HERE / "_ref"
EXE = OUT / "ref_gpumpi_bench"
DRIVER = HERE / "refgpu" / "driver.cu"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_DIRS = ["gpu_libs/gpu_libc", "gpu_libs/gpu_libc/sys", "gpu_libs/gpu_mpi", "gpu_libs/gpu_main", "common"]


def reference_root() -> Path:
    return Path(os.environ.get("REFERENCE_SRC", "/root/reference"))


def stage() -> bool:
    """Copies the reference runtime sources into baseline/_ref/src (when the checkout is present), and
    its toolchain test programs into baseline/_ref/toolchain."""
    stage_toolchain()
    ref = reference_root()
    if not (ref / "gpu_libs" / "gpu_mpi" / "mpi.cu").exists():
        return STAGE.exists()
    for d in ("gpu_libs/gpu_libc", "gpu_libs/gpu_mpi", "gpu_libs/gpu_main", "common"):
        dst = STAGE / d
        if dst.exists():
            shutil.rmtree(dst)
        shutil.copytree(ref / d, dst, ignore=shutil.ignore_patterns("main.cu", "CMakeLists.txt", "*.md"))
    return True


TOOLCHAIN = ROOT / "baseline" / "_ref" / "toolchain"
# the reference's own plain C MPI programs that its toolchain tests convert and run (toolchain_tests/)
TOOLCHAIN_PROGRAMS = ["pi/cpi.c", "global_var/global_var.c", "datatype/contiguous.c", "basicIO/basicIO.c",
                      "basicIO/file_view1.c", "basicIO/file_view2.c"]


# NPB IS and DT (the integer sort and data traffic benchmarks of the NAS Parallel Benchmarks, which the
# reference's toolchain tests convert and run: toolchain_tests/npb/is_test.sh, dt_test.sh): their sources,
# the common files they link, and NPB's own parameter generator with its configuration template
NPB = "npb/NPB3.4.1/NPB3.4-MPI"
NPB_FILES = [f"{NPB}/{p}" for p in (
    "IS/is.c", "DT/dt.c", "DT/DGraph.c", "DT/DGraph.h", "common/c_print_results.c", "common/c_timers.c",
    "common/c_timers.h", "common/randdp.c", "sys/setparams.c", "config/make.def.template")]
NPB_SOURCES = {"is": ["IS/is.c", "common/c_print_results.c", "common/c_timers.c"],
               "dt": ["DT/dt.c", "DT/DGraph.c", "common/c_print_results.c", "common/c_timers.c", "common/randdp.c"]}


def stage_toolchain() -> bool:
    """Copies the reference's toolchain test programs (and NPB IS and DT) unchanged into
    baseline/_ref/toolchain/ (git-ignored) for the source converter's tests: they are the converter's inputs in
    the reference, so converting, building and running them here checks the converter against the reference's
    own programs."""
    ref = reference_root() / "toolchain_tests"
    files = TOOLCHAIN_PROGRAMS + NPB_FILES
    if not all((ref / p).exists() for p in files):
        return all((TOOLCHAIN / p).exists() for p in files)
    for p in files:
        (TOOLCHAIN / p).parent.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(ref / p, TOOLCHAIN / p)
    return True


def npb_prepare(dst: Path, bench: str, cls: str = "S") -> list:
    """Copies the staged NPB tree to dst and writes `bench`'s npbparams.h for class `cls` the way NPB's build
    does (sys/setparams, compiled with the host C compiler, run in the benchmark's directory with the
    configuration template as config/make.def); returns the benchmark's source files under dst."""
    shutil.copytree(TOOLCHAIN / "npb", dst / "npb")
    mpi = dst / NPB
    shutil.copyfile(mpi / "config" / "make.def.template", mpi / "config" / "make.def")
    cc = shutil.which("gcc") or shutil.which("cc")
    subprocess.run([cc, "-o", str(mpi / "sys" / "setparams"), str(mpi / "sys" / "setparams.c")], check=True,
                   capture_output=True)
    bdir = mpi / bench.upper()
    subprocess.run([str(mpi / "sys" / "setparams"), bench, cls], cwd=bdir, check=True, capture_output=True)
    return [mpi / p for p in NPB_SOURCES[bench]]


def sources() -> list:
    out = []
    for d in ("gpu_libs/gpu_libc", "gpu_libs/gpu_libc/sys", "gpu_libs/gpu_mpi", "gpu_libs/gpu_main", "common"):
        out += sorted((STAGE / d).glob("*.cu"))
    return out


def build(force: bool = False) -> Path:
    if not STAGE.exists() and not stage():
        raise FileNotFoundError("reference runtime sources are not staged (baseline/_ref/src)")
    deps = sources() + [DRIVER, HERE / "gpumpi_oracle.c"]
    if not force and EXE.exists() and all(p.stat().st_mtime <= EXE.stat().st_mtime for p in deps):
        return EXE
    objdir = OUT / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = []
    for d in LIB_DIRS:
        inc += ["-I", str(STAGE / d)]
    flags = ARCH + ["-O3", "-std=c++17", "-rdc=true", "-w"] + inc

    def compile_one(src: Path) -> Path:
        obj = objdir / (src.parent.name + "_" + src.stem + ".o")
        r = subprocess.run([nvcc, *flags, "-c", str(src), "-o", str(obj)], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-4000:]}")
        return obj

    srcs = sources() + [DRIVER]
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    gen = objdir / "oracle_gen.o"
    subprocess.run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-c", str(HERE / "gpumpi_oracle.c"),
                    "-o", str(gen)], check=True)
    tmp = OUT / "ref_gpumpi_bench.tmp"
    r = subprocess.run([nvcc, *ARCH, "-rdc=true", *map(str, objs), str(gen), "-o", str(tmp), "-lpthread"],
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, EXE)
    return EXE


def _run(args: list, limit_s: float) -> dict:
    try:
        r = subprocess.run([str(EXE), *map(str, args), str(limit_s)], capture_output=True, text=True,
                           timeout=limit_s + 60)
    except subprocess.TimeoutExpired:
        return {"error": f"no answer within {limit_s + 60:.0f} s"}
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if not lines:
        return {"error": f"exit {r.returncode}: {(r.stderr or r.stdout)[-400:]}"}
    return json.loads(lines[-1])


def run_allreduce(n: int, count: int, iters: int = 2, seed: int = 2026, limit_s: float = 120.0) -> dict:
    """The reference's MPI_Allreduce(fp32 SUM) among n ranks; result checked against the oracle."""
    from oracle import oracle
    with tempfile.TemporaryDirectory() as td:
        out = Path(td) / "row0.bin"
        res = _run(["allreduce", n, count, iters, seed, out], limit_s)
        if "error" in res:
            return res
        got = np.fromfile(out, dtype=np.float32)
    x = oracle.fill_f32(seed, n * count).reshape(n, count)
    ref = oracle.reduce(x, 12, 2)
    # the reference folds in rank order too (mpi.cu:209-225), so its result is bit-identical
    res["bit_exact_vs_oracle"] = bool(np.array_equal(got.view(np.uint32), ref.view(np.uint32))) and res["rows_identical"]
    return res


def alltoallv_checksums(recv: np.ndarray) -> np.ndarray:
    """Per receiving rank: sum over its elements e_k of (uint32)e_k * (k + 1), mod 2^64 (the driver's)."""
    k = np.arange(1, recv.shape[1] + 1, dtype=np.uint64)
    return (recv.view(np.uint32).astype(np.uint64) * k[None, :]).sum(1, dtype=np.uint64)


def run_alltoallv(sc: np.ndarray, iters: int = 2, seed: int = 99, limit_s: float = 120.0) -> dict:
    """The reference's MPI_Alltoallv(int32) with counts sc[r][s] >= 1; placement checked against the oracle."""
    from oracle import oracle
    n = sc.shape[0]
    sc = np.ascontiguousarray(sc, dtype=np.int32)
    with tempfile.TemporaryDirectory() as td:
        cf = Path(td) / "counts.bin"
        sc.tofile(cf)
        out = Path(td) / "sums.bin"
        res = _run(["alltoallv", n, cf, iters, seed, out], limit_s)
        if "error" in res:
            return res
        sums = np.fromfile(out, dtype=np.uint64)
    rc = sc.T.copy()
    sd = (np.cumsum(sc, 1) - sc).astype(np.int32)
    rd = (np.cumsum(rc, 1) - rc).astype(np.int32)
    S, R = int(sc.sum(1).max()), int(rc.sum(1).max())
    x = oracle.fill_i32(seed, n * S).reshape(n, S)
    ref = oracle.alltoallv(x, sc, sd, R, rc, rd, threads=os.cpu_count() or 1)
    res["bit_exact_vs_oracle"] = bool(np.array_equal(sums, alltoallv_checksums(ref)))
    return res


if __name__ == "__main__":
    import sys
    if len(sys.argv) > 1 and sys.argv[1] == "stage":
        print(stage())
    else:
        print(build(force="--force" in sys.argv))
