"""Builds libgpumpi.so (the block-rank MPI runtime + its C ABI) for sm_103a, in-tree.

nvcc compiles the translation units in parallel with relocatable device code and links them into
one shared library (device link included).  Output: dphpc-gpu_mpi_gb300/_build/libgpumpi.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libgpumpi.so"
SOURCES = [
    CSRC / "api" / "mpi_api.cu",
    CSRC / "programs" / "prog_tests.cu",
    CSRC / "programs" / "prog_hot.cu",
    CSRC / "programs" / "prog_apps.cu",
    CSRC / "host" / "host.cu",
    CSRC / "host" / "noalloc.cu",
    CSRC / "host" / "host_io.cu",
    CSRC / "selector" / "mlp.cu",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def common_flags() -> list[str]:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-rdc=true", "-maxrregcount=64",
                   "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"), "-I", str(CSRC / "runtime"),
                   "-I", str(CSRC / "programs")]


def _deps() -> list[Path]:
    out = list(SOURCES)
    for d in ("runtime", "programs", "api", "host", "selector"):
        out += list((CSRC / d).glob("*.cuh"))
    out += list((ROOT / "include").glob("*.h")) + list((ROOT / "include").glob("*.cuh"))
    return out


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    nv = nvcc()
    flags = common_flags()
    if verbose:
        flags += ["-Xptxas", "-v"]

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        cmd = [nv, *flags, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr[-8000:]}")
        if verbose and r.stderr:
            (BUILD / (src.stem + ".ptxas.txt")).write_text(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = BUILD / "libgpumpi.so.tmp"
    cmd = [nv, *ARCH, "-shared", "-rdc=true", *map(str, objs), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-8000:]}")
    os.replace(tmp, LIB)
    return LIB


def build_program(sources: list, out: Path, extra_flags: list | None = None) -> Path:
    """Builds an executable from a converted MPI program (the reference's gpumpicc step): the user's
    sources define `__device__ int __gpu_main(int, char**)` and include <mpi.h.cuh>; they are compiled with
    the runtime's flags and device-linked with the runtime's objects and csrc/host/user_main.cu (main() ->
    gpumpi_main).  Run it as `out [program args] ---gpumpi -n RANKS [...]`."""
    build()
    nv = nvcc()
    flags = common_flags() + list(extra_flags or [])
    udir = BUILD / "user"
    udir.mkdir(parents=True, exist_ok=True)
    objs = []
    for k, src in enumerate([Path(x) for x in sources] + [CSRC / "host" / "user_main.cu"]):
        obj = udir / f"{k}_{src.stem}.o"
        r = subprocess.run([nv, *flags, "-c", str(src), "-o", str(obj)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-8000:]}")
        objs.append(obj)
    runtime = [BUILD / (src.stem + ".o") for src in SOURCES]
    out = Path(out)
    r = subprocess.run([nv, *ARCH, "-rdc=true", *map(str, runtime + objs), "-o", str(out)], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-8000:]}")
    return out


if __name__ == "__main__":
    if "--program" in sys.argv:
        # build.py --program a.cu [b.cu ...] -o OUT
        args = sys.argv[sys.argv.index("--program") + 1:]
        out = args[args.index("-o") + 1] if "-o" in args else "a.out"
        srcs = [a for i, a in enumerate(args) if a != "-o" and (i == 0 or args[i - 1] != "-o")]
        print(build_program(srcs, Path(out)))
    else:
        print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
