"""gpumpicc: builds a C MPI program into an executable whose ranks are thread blocks of one GPU.

The reference's compiler wrapper (scripts/gpumpicc.py) runs its clang source converter on the sources and
the project's headers, renames includes to their `.cuh` forms and links the result with the runtime's
libraries through nvcc.  This one runs the token-level converter (gpumpi/converter.py) into a work
directory and links the converted sources with the runtime's objects (build.py: build_program).

    python -m gpumpi.gpumpicc prog.c [more.c ...] -o prog [-I dir] [-D NAME[=V]] [--max-ranks N]
    ./prog [program arguments] ---gpumpi -n RANKS [-b THREADS] ...

The project directory (headers converted with the sources) is $GPU_MPI_PROJECT as in the reference, else
the first source's directory.  The rank capacity of the per-rank globals is --max-ranks, else
$GPU_MPI_MAX_RANKS, else 1024; the executable refuses to start more ranks than that.
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

from . import converter

PKG = Path(__file__).resolve().parent.parent


def _build_module():
    spec = importlib.util.spec_from_file_location("gpumpi_build", PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def compile_program(sources, out, include_dirs=(), defines=(), max_ranks=None, workdir=None,
                    extra_types=(), project=None) -> Path:
    """Converts `sources` (C files, with the project's headers they include) and links them into the
    executable `out`; returns its path."""
    out = Path(out).resolve()
    work = Path(workdir) if workdir else out.parent / (out.name + ".gpumpi")
    converted = converter.convert_files(sources, work, max_ranks, include_dirs, project=project,
                                        extra_types=extra_types)
    flags = []
    for d in [*(Path(s).resolve().parent for s in sources), work, *include_dirs]:
        flags += ["-I", str(Path(d).resolve())]
    for d in defines:
        flags += ["-D" + d]
    return _build_module().build_program(converted, out, flags)


def main(argv=None) -> int:
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("sources", nargs="+")
    ap.add_argument("-o", dest="out", default="a.out")
    ap.add_argument("-I", dest="include_dirs", action="append", default=[])
    ap.add_argument("-D", dest="defines", action="append", default=[])
    ap.add_argument("--max-ranks", type=int, default=None)
    ap.add_argument("--workdir", default=None, help="where the converted sources go (default OUT.gpumpi/)")
    ap.add_argument("--type", dest="types", action="append", default=[], help="extra typedef name")
    ap.add_argument("--project", default=None, help="project directory (default $GPU_MPI_PROJECT)")
    a = ap.parse_args(argv)
    try:
        print(compile_program(a.sources, a.out, a.include_dirs, a.defines, a.max_ranks, a.workdir, a.types,
                              a.project))
    except (converter.ConversionError, RuntimeError) as e:
        print(f"gpumpicc: {e}", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
