"""GPU: a converted MPI program (main renamed __gpu_main, the reference's converter contract) built into an
executable by the program builder and run through the launcher, `prog [args] ---gpumpi -n RANKS`, as the
reference's gpumpicc output runs (gpu_libs/gpu_main/main.cu)."""
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "dphpc-gpu_mpi_gb300"))


@pytest.fixture(scope="module")
def pi_exe(tmp_path_factory, gpulib):   # gpulib: skips without a GPU
    import build
    out = tmp_path_factory.mktemp("prog") / "mpi_pi"
    return build.build_program([ROOT / "tests" / "programs" / "mpi_pi_integrate.cu"], out)


def expected_pi(n: int, ranks: int) -> float:
    h = 1.0 / n
    total = 0.0
    for r in range(ranks):   # canonical rank order, as MPI_Reduce folds here
        s = 0.0
        for i in range(r, n, ranks):
            x = h * (i + 0.5)
            s += 4.0 / (1.0 + x * x)
        total += h * s
    return total


@pytest.mark.parametrize("ranks,n", [(1, 1000), (64, 200000), (300, 30000)])
def test_converted_program_runs(pi_exe, ranks, n):
    r = subprocess.run([str(pi_exe), str(n), "---gpumpi", "-n", str(ranks)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    line = [l for l in r.stdout.splitlines() if l.startswith("pi ")][-1].split()
    assert int(line[3]) == ranks and int(line[5]) == n and int(line[7]) == n   # per-rank globals summed
    # fused multiply-adds on the device may round the terms differently: a relative tolerance
    assert abs(float(line[1]) - expected_pi(n, ranks)) <= 1e-12 * 3.2


def test_failing_rank_gives_exit_status_1(pi_exe):
    # a rank returning non-zero makes the launcher exit with 1 and name the rank (main.cu:126-129,320)
    r = subprocess.run([str(pi_exe), "1000", "5", "---gpumpi", "-n", "8"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 1 and "rank 5 returned 3" in r.stderr, (r.returncode, r.stderr)


def test_bad_options_fail_cleanly(pi_exe):
    r = subprocess.run([str(pi_exe), "1000", "---gpumpi", "-n", "8", "-b", "48"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 1 and "threads_per_block" in r.stderr


@pytest.fixture(scope="module")
def io_exe(tmp_path_factory, gpulib):
    import build
    out = tmp_path_factory.mktemp("prog") / "mpi_io_report"
    return build.build_program([ROOT / "tests" / "programs" / "mpi_io_report.cu"], out)


@pytest.mark.parametrize("ranks", [1, 16, 100])
def test_converted_program_writes_files_and_prints(io_exe, tmp_path, ranks):
    # fprintf(stdout, ...) and MPI_File_write_at from ranks, performed by the launcher's host channel
    import numpy as np
    n = 1000
    out = tmp_path / "partial.bin"
    r = subprocess.run([str(io_exe), str(out), str(n), "---gpumpi", "-n", str(ranks)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    total = float(sum(i * i for i in range(n)))
    assert f"sum of squares below {n} over {ranks} ranks: {total:.1f}" in r.stdout
    parts = np.fromfile(out, dtype=np.float64)
    assert parts.tolist() == [float(sum(i * i for i in range(k, n, ranks))) for k in range(ranks)]


@pytest.fixture(scope="module")
def report_exe(tmp_path_factory, gpulib):
    import build
    out = tmp_path_factory.mktemp("prog") / "mpi_pi_report"
    return build.build_program([ROOT / "tests" / "programs" / "mpi_pi_report.cu"], out)


def expected_pi_report(n: int, ranks: int) -> float:
    """The program's sum in its own order: per rank every size-th interval from rank + 1, times h, then
    the ranks' parts in rank order (the canonical MPI_Reduce fold)."""
    h = 1.0 / n
    total = 0.0
    for r in range(ranks):
        s = 0.0
        for i in range(r + 1, n + 1, ranks):
            x = h * (i - 0.5)
            s += 4.0 / (1.0 + x * x)
        total += h * s
    return total


@pytest.mark.parametrize("ranks,n", [(1, 10000), (16, 100000), (100, 100000)])
def test_converted_pi_program_reports_through_host_streams(report_exe, ranks, n):
    # MPI_Get_processor_name, MPI_Wtime, fprintf(stderr), printf and fflush(stdout) from ranks, performed
    # by the launcher's host channel while the kernel runs
    import math
    r = subprocess.run([str(report_exe), str(n), "---gpumpi", "-n", str(ranks)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    where = sorted(l for l in r.stderr.splitlines() if l.startswith("rank "))
    assert where == sorted(f"rank {k} of {ranks} runs on GB300 block-rank" for k in range(ranks))
    est = [l for l in r.stdout.splitlines() if l.startswith("pi estimate ")]
    assert len(est) == 1, r.stdout
    pi, err = (float(x) for x in est[0][len("pi estimate "):].replace(", error", "").split())
    assert abs(pi - expected_pi_report(n, ranks)) <= 1e-12 * 3.2
    assert abs(err - abs(pi - math.pi)) <= 1e-15
    secs = [l for l in r.stdout.splitlines() if l.startswith("elapsed ")]
    assert len(secs) == 1 and 0.0 <= float(secs[0].split()[1]) < 60.0


# ---- plain C programs through gpumpicc (source converter + program builder) ----

CPROGS = ROOT / "tests" / "programs" / "c"


def gpumpicc(sources, out, max_ranks=None):
    from gpumpi import gpumpicc as cc
    return cc.compile_program([CPROGS / s for s in sources], out, max_ranks=max_ranks)


@pytest.fixture(scope="module")
def c_programs(tmp_path_factory, gpulib):
    d = tmp_path_factory.mktemp("cprog")
    return {"rect_pi": gpumpicc(["rect_pi.c"], d / "rect_pi"),
            "globals": gpumpicc(["globals.c"], d / "globals"),
            "globals8": gpumpicc(["globals.c"], d / "globals8", max_ranks=8),
            "oldstyle": gpumpicc(["oldstyle.c", "oldstyle_lib.c"], d / "oldstyle")}


@pytest.mark.parametrize("ranks,n", [(1, 10000), (7, 10000), (64, 100000)])
def test_c_pi_program_runs_unchanged(c_programs, ranks, n):
    # a classic C pi program: atoi, fabs, fprintf(stdout)/printf/fflush, MPI_Get_processor_name, MPI_Wtime
    import math
    r = subprocess.run([str(c_programs["rect_pi"]), str(n), "---gpumpi", "-n", str(ranks)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    where = sorted(l for l in r.stdout.splitlines() if l.startswith("rank "))
    assert where == sorted(f"rank {k}/{ranks} on GB300 block-rank" for k in range(ranks))
    est = [l for l in r.stdout.splitlines() if l.startswith("pi = ")]
    assert len(est) == 1, r.stdout
    pi, err = (float(x) for x in est[0][len("pi = "):].replace(", error =", "").split())
    assert abs(pi - expected_pi_report(n, ranks)) <= 1e-12 * 3.2
    assert abs(err - abs(pi - math.pi)) <= 1e-15


@pytest.mark.parametrize("ranks", [1, 8, 100])
def test_c_globals_are_per_rank(c_programs, ranks):
    r = subprocess.run([str(c_programs["globals"]), "---gpumpi", "-n", str(ranks)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, (r.stdout, r.stderr)
    assert f"globals: {ranks} ranks, ok" in r.stdout


def test_c_program_refuses_more_ranks_than_it_was_converted_for(c_programs):
    ok = subprocess.run([str(c_programs["globals8"]), "---gpumpi", "-n", "8"], capture_output=True, text=True,
                        timeout=120)
    assert ok.returncode == 0 and "globals: 8 ranks, ok" in ok.stdout, ok.stderr
    r = subprocess.run([str(c_programs["globals8"]), "---gpumpi", "-n", "9"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 1 and "converted for at most 8" in r.stderr


def _checksum(text: str) -> int:
    s = 0
    for ch in text:
        s = (s * 31 + ord(ch)) & 0xFFFFFFFF
    return s - (1 << 32) if s >= 1 << 31 else s


@pytest.mark.parametrize("ranks", [1, 2, 5])
def test_c_oldstyle_program(c_programs, ranks):
    # K&R definitions, implicit void* conversions, C++-keyword identifiers, libc strings and numbers,
    # a contiguous datatype, two translation units sharing a global through a project header
    r = subprocess.run([str(c_programs["oldstyle"]), "---gpumpi", "-n", str(ranks)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, (r.stdout, r.stderr)
    labels = ["rec-a", "rec-b", "rec-b"]
    total = sum(_checksum(labels[k % 3]) + k for k in range(ranks))
    assert f"oldstyle: {ranks} ranks, total {total}, failures 0" in r.stdout, r.stdout


# ---- the reference's own toolchain programs (toolchain_tests/, staged unchanged by oracle/refgpu.py) ----

def _toolchain():
    sys.path.insert(0, str(ROOT))
    from oracle import refgpu
    return refgpu


@pytest.fixture(scope="module")
def ref_programs(tmp_path_factory, gpulib):
    refgpu = _toolchain()
    if not all((refgpu.TOOLCHAIN / p).exists() for p in refgpu.TOOLCHAIN_PROGRAMS):
        pytest.skip("the reference's toolchain programs are not staged")
    from gpumpi import gpumpicc as cc
    d = tmp_path_factory.mktemp("refprog")
    return {Path(p).stem: cc.compile_program([refgpu.TOOLCHAIN / p], d / Path(p).stem, max_ranks=256)
            for p in refgpu.TOOLCHAIN_PROGRAMS}


@pytest.mark.parametrize("ranks,n", [(4, 10000), (33, 100000)])
def test_reference_cpi_runs_converted(ref_programs, ranks, n):
    # toolchain_tests/pi/test.sh runs `./pi ---gpumpi -g 4 -b 1 -s 8192`
    import math
    r = subprocess.run([str(ref_programs["cpi"]), str(n), "---gpumpi", "-n", str(ranks)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    procs = sorted(l for l in r.stdout.splitlines() if l.startswith("Process "))
    assert procs == sorted(f"Process {k} of {ranks} is on GB300 block-rank" for k in range(ranks))
    est = [l for l in r.stdout.splitlines() if l.startswith("pi is approximately ")]
    assert len(est) == 1, r.stdout
    pi, err = (float(x) for x in est[0][len("pi is approximately "):].replace(", Error is", "").split())
    assert abs(pi - expected_pi_report(n, ranks)) <= 1e-12 * 3.2
    assert abs(err - abs(pi - math.pi)) <= 1e-15
    assert any(l.startswith("wall clock time = ") for l in r.stdout.splitlines())


@pytest.mark.parametrize("ranks", [4, 64, 256])
def test_reference_global_var_runs_converted(ref_programs, ranks):
    # toolchain_tests/global_var/test.sh runs it on 4 ranks; it returns 1 and prints "error ..." when a
    # per-rank global does not behave as a process's global
    r = subprocess.run([str(ref_programs["global_var"]), "---gpumpi", "-n", str(ranks)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0 and "error" not in r.stdout, (r.stdout, r.stderr)


def test_reference_contiguous_runs_converted(ref_programs):
    r = subprocess.run([str(ref_programs["contiguous"]), "---gpumpi", "-n", "2"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("ranks", [1, 4, 16])
def test_reference_io_programs_run_converted(ref_programs, tmp_path, ranks):
    import numpy as np
    for name in ("basicIO", "file_view1", "file_view2"):
        r = subprocess.run([str(ref_programs[name]), "---gpumpi", "-n", str(ranks)], capture_output=True, text=True,
                           timeout=120, cwd=tmp_path)
        assert r.returncode == 0, (name, r.stderr)
    assert (tmp_path / "test.out").read_bytes() == b"hello world from GPUMPI IO"
    v1 = np.fromfile(tmp_path / "test_file_view1.out", dtype=np.int32)
    assert v1.tolist() == list(range(100)) * ranks      # each rank's 100 ints at rank * 400 bytes
    # two blocks of 50 ints per rank, 50 * ranks ints apart (the buffer itself is uninitialised)
    assert (tmp_path / "test_file_view2.out").stat().st_size == 2 * 50 * ranks * 4


def _npb(tmp_path_factory, bench):
    refgpu = _toolchain()
    if not all((refgpu.TOOLCHAIN / p).exists() for p in refgpu.NPB_FILES):
        pytest.skip("NPB is not staged")
    from gpumpi import gpumpicc as cc
    d = tmp_path_factory.mktemp("npb_" + bench)
    srcs = refgpu.npb_prepare(d, bench, "S")   # npbparams.h from NPB's own setparams
    return cc.compile_program(srcs, d / f"{bench}.S.x", max_ranks=64, project=d / "npb")


@pytest.fixture(scope="module")
def npb_is(tmp_path_factory, gpulib):
    return _npb(tmp_path_factory, "is")


@pytest.fixture(scope="module")
def npb_dt(tmp_path_factory, gpulib):
    return _npb(tmp_path_factory, "dt")


@pytest.mark.parametrize("ranks,strict", [(2, None), (8, None), (16, None), (3, "off")])
def test_npb_is_class_s_verifies(npb_is, tmp_path, ranks, strict):
    # toolchain_tests/npb/is_test.sh: `make IS CLASS=S` through gpumpicc, then `./bin/is.S.x ---gpumpi -g 2`.
    # IS verifies its own sort.  With 3 ranks and NPB_NPROCS_STRICT=off (read through getenv, answered by
    # the launcher's environment) IS runs on the largest power of two and the third rank leaves through
    # MPI_Finalize and exit(0)
    import os
    env = {**os.environ, "NPB_NPROCS_STRICT": strict} if strict else None
    r = subprocess.run([str(npb_is), "---gpumpi", "-n", str(ranks)], capture_output=True, text=True, timeout=300,
                       cwd=tmp_path, env=env)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "Verification    =               SUCCESSFUL" in r.stdout, r.stdout[-3000:]
    assert " Class           =                        S" in r.stdout


def test_npb_is_exit_status_reaches_the_launcher(npb_is, tmp_path):
    # without NPB_NPROCS_STRICT, 3 ranks are refused: every rank calls MPI_Abort and exit(1), ends with
    # status 1, and the launcher exits with 1
    import os
    env = {k: v for k, v in os.environ.items() if k != "NPB_NPROCS_STRICT"}
    r = subprocess.run([str(npb_is), "---gpumpi", "-n", "3", "--timeout", "5"], capture_output=True, text=True,
                       timeout=300, cwd=tmp_path, env=env)
    assert r.returncode == 1, (r.stdout[-2000:], r.stderr[-2000:])
    assert "is not a power of two" in r.stdout


@pytest.mark.parametrize("graph,ranks", [("BH", 5), ("WH", 5), ("SH", 32)])
def test_npb_dt_class_s_verifies(npb_dt, tmp_path, graph, ranks):
    # toolchain_tests/npb/dt_test.sh: `make DT CLASS=S` through gpumpicc, then
    # `./bin/dt.S.x BH ---gpumpi -g 5 -b 1 -s 16000 -p 80000000`; DT checks its own result
    r = subprocess.run([str(npb_dt), graph, "---gpumpi", "-n", str(ranks), "-s", "16000"], capture_output=True,
                       text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "Verification    =               SUCCESSFUL" in r.stdout, (r.stdout[-3000:], r.stderr[-3000:])
