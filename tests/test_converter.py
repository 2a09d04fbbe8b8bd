"""CPU tests of the source converter (gpumpi/converter.py), the counterpart of the reference's clang tool
(source_converter/converter.cpp): each rewrite on small inputs, and the converted test programs
compiling for sm_103a (nvcc cross-compiles without a GPU)."""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from gpumpi import converter as cv
from oracle import refgpu

ROOT = Path(__file__).resolve().parents[1]
PROGS = ROOT / "tests" / "programs" / "c"


def conv(src: str, n: int = 4) -> str:
    out = cv.convert_source(src, max_ranks=n)
    assert out.startswith(cv.PRELUDE)
    return out[len(cv.PRELUDE):]


def squash(s: str) -> str:
    return re.sub(r"\s+", " ", s).strip()


def test_functions_get_device_and_main_is_renamed():
    out = squash(conv("double f(double);\nstatic int g(void) { return 1; }\nint main() { return g(); }\n", 8))
    assert "__device__ double f(double);" in out
    assert "__device__ static int g(void) { return 1; }" in out
    assert "__device__ int __gpu_main(int argc, char** argv) { return g(); return 0; }" in out
    assert "__device__ int __gpu_max_threads() { return 8; }" in out
    assert 'extern "C" const int gpumpi_program_max_ranks = 8;' in out


def test_main_keeps_its_own_parameters():
    out = squash(conv("int main(int ac, char **av) { return ac; }"))
    assert "__device__ int __gpu_main(int ac, char **av) { return ac; return 0; }" in out


def test_globals_become_per_rank_arrays_with_repeated_initializers():
    out = squash(conv("int a = -1, *p, m[2][2] = {{1,2},{3,4}};\nextern int e;\nstatic char c;\n", 3))
    assert "__device__ int a[3] = {-1, -1, -1}, *p[3], m[3][2][2] = {{{1,2},{3,4}}, {{1,2},{3,4}}, {{1,2},{3,4}}};" in out
    assert "__device__ extern int e[3];" in out
    assert "__device__ static char c[3];" in out


def test_references_are_wrapped_unless_shadowed():
    src = """int g = 1; int h[4];
int f(int g) { return g + h[0]; }
int k(void) { int r = g; { int h = 2; r += h; } for (int g = 0; g < 1; g++) r += g; return r + g; }
"""
    out = squash(conv(src))
    assert "__device__ int f(int g) { return g + __gpu_global(h)[0]; }" in out
    assert ("int r = __gpu_global(g); { int h = 2; r += h; } for (int g = 0; g < 1; g++) r += g; "
            "return r + __gpu_global(g); }") in out


def test_member_names_labels_and_tags_are_not_references():
    src = """struct s { int g; } v; int g;
int f(void) { struct s g2; g2.g = g; v.g = 1; goto g_end; g_end: return v.g; }
"""
    out = squash(conv(src))
    assert "g2.g = __gpu_global(g); __gpu_global(v).g = 1; goto g_end; g_end: return __gpu_global(v).g;" in out


def test_function_static_becomes_per_rank():
    out = squash(conv("int f(void) { static int n = 5; n++; return n; }", 2))
    assert "static int n[2] = {5, 5}; __gpu_global(n)++; return __gpu_global(n);" in out


def test_old_style_definition_gets_a_prototype_list():
    out = squash(conv("int f(a, b, c) double a; char *b; { return a + b[0] + c; }"))
    assert "__device__ int f(double a, char *b, int c ) { return a + b[0] + c; }" in out


def test_allocations_get_casts():
    src = """typedef struct node { int v; } node;
node *head; int **grid;
void f(int n) { double *x = malloc(n * sizeof(double)); node *t; t = calloc(1, sizeof(node));
  head = malloc(8); grid = malloc(8); grid[0] = malloc(4); }
"""
    out = squash(conv(src))
    assert "double *x = (double *)malloc(n * sizeof(double));" in out
    assert "t = (node *)calloc(1, sizeof(node));" in out
    assert "__gpu_global(head) = (node *)malloc(8);" in out
    assert "__gpu_global(grid) = (int **)malloc(8); __gpu_global(grid)[0] = (int *)malloc(4);" in out


def test_unsized_arrays_get_the_extent_their_initializer_implies():
    src = """static const char *names[] = {"a", "b", "c",};
int tab[] = { [5] = 1, 2, [1] = 3 };
char msg[] = "hi\\n" "there";
int g(void) { static int loc[] = {1, 2, 3}; return loc[2] + tab[6] + msg[0] + names[2][0]; }
"""
    out = squash(conv(src, 2))
    assert '__device__ static const char *names[2][3] = {{"a", "b", "c",}, {"a", "b", "c",}};' in out
    assert "__device__ int tab[2][7] =" in out
    assert "__device__ char msg[2][9] =" in out
    assert "static int loc[2][3] = {{1, 2, 3}, {1, 2, 3}};" in out


def test_extern_array_of_unknown_extent_takes_its_definitions(tmp_path):
    (tmp_path / "def.c").write_text("double table[] = {1.0, 2.0, 3.0};\nint rows = 3;\n")
    (tmp_path / "use.c").write_text("extern double table[];\nextern int rows;\n"
                                    "double last(void) { return table[rows - 1]; }\n")
    out = cv.convert_files([tmp_path / "use.c", tmp_path / "def.c"], tmp_path / "conv", max_ranks=4)
    assert "__device__ extern double table[4][3];" in squash(out[0].read_text())
    assert "__device__ double table[4][3] =" in squash(out[1].read_text())
    with pytest.raises(cv.ConversionError):
        cv.convert_source("extern double other[];\ndouble f(void) { return other[0]; }\n", max_ranks=2)


def test_initializers_naming_globals_use_each_ranks_copy():
    src = ("int base = 3;\nint arr[4];\nint *pb = &base, *pa = arr + 1;\n"
           "struct S { int *p; int n; } s = { &base, sizeof(arr) };\nint f(void) { static int *q = &base; return *q; }\n")
    out = squash(conv(src, 2))
    assert "__device__ int *pb[2] = {&base[0], &base[1]}, *pa[2] = {arr[0] + 1, arr[1] + 1};" in out
    assert "s[2] = {{ &base[0], sizeof(arr[0]) }, { &base[1], sizeof(arr[1]) }};" in out
    assert "static int *q[2] = {&base[0], &base[1]};" in out


def test_globals_in_array_dimensions_mean_one_ranks_copy():
    out = squash(conv("double src[] = {1, 2, 3};\ndouble copy[sizeof(src) / sizeof(src[0])];\n", 2))
    assert "__device__ double copy[2][sizeof(src[0]) / sizeof(src[0][0])];" in out


def test_const_definitions_keep_external_linkage():
    out = squash(conv("const int N = 4;\nstatic const int M = 2;\nconst char *name = \"x\";\n"
                      "char * const fixed = 0;\nextern const int K;\nint f(void) { return N + M + K; }\n", 2))
    assert "__device__ extern const int N[2] = {4, 4};" in out
    assert "__device__ static const int M[2] = {2, 2};" in out
    assert '__device__ const char *name[2] = {"x", "x"};' in out       # a pointer to const: already external
    assert "__device__ extern char * const fixed[2] = {0, 0};" in out
    assert "__device__ extern const int K[2];" in out


@pytest.mark.skipif(shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists(),
                    reason="no nvcc")
def test_tables_shared_across_files_device_link(tmp_path):
    # const and unsized file-scope arrays defined in one file and used through extern declarations in
    # another: both converted, compiled for sm_103a and device-linked (every symbol resolves)
    import build as gbuild
    (tmp_path / "tabdef.c").write_text('const int primes[] = {2, 3, 5, 7, 11, 13};\n'
                                       'const char *words[] = {"alpha", "beta", "gamma"};\n'
                                       'char banner[] = "tables";\nconst double scale = 0.5;\n')
    (tmp_path / "tabuse.c").write_text('extern const int primes[];\nextern const char *words[];\n'
                                       'extern char banner[];\nextern const double scale;\n'
                                       'double score(int r) { return (primes[r % 6] + words[r % 3][0] + '
                                       'banner[0]) * scale; }\n')
    out = cv.convert_files([tmp_path / "tabuse.c", tmp_path / "tabdef.c"], tmp_path / "conv", max_ranks=8)
    objs = []
    for f in out:
        o = f.with_suffix(".o")
        r = subprocess.run([gbuild.nvcc(), *gbuild.common_flags(), "-c", str(f), "-o", str(o)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]
        objs.append(str(o))
    r = subprocess.run([gbuild.nvcc(), *gbuild.ARCH, "-dlink", *objs, "-o", str(tmp_path / "dlink.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_void_pointer_members_get_casts():
    # the reference's converter casts every implicit conversion from void*; here: values of void* struct
    # members reaching typed pointers through assignment, initialisation, return and call arguments
    src = """typedef struct { int id; void *head, *tail; } Arc;
typedef struct node { Arc **in; void *feat; } Node;
typedef struct { double *v; } Arr;
double total(Arr *a, int w);
Arr *feat_of(Node *n) { return n->feat; }
double f(Arc *ar, Node *nd, int j) {
  Node *h = ar->head, *t;
  t = nd->in[j]->tail;
  void *keep = ar->tail;
  return total(nd->feat, j) + total(feat_of(h), 0);
}
"""
    out = squash(conv(src))
    assert "Arr *feat_of(Node *n) { return (Arr *)n->feat; }" in out
    assert "Node *h = (Node *)ar->head, *t;" in out
    assert "t = (Node *)nd->in[j]->tail;" in out
    assert "void *keep = ar->tail;" in out
    assert "return total((Arr *)nd->feat, j) + total(feat_of(h), 0);" in out


def test_cxx_keywords_are_renamed():
    out = squash(conv("int f(int class) { int new = class, this = 1; return new + this; }"))
    assert "int f(int __decl_class) { int __decl_new = __decl_class, __decl_this = 1; return __decl_new + __decl_this; }" in out


def test_includes_and_macros():
    src = """#include "mpi.h"
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
int total;
#define TOTAL total
#define ADD(total, x) ((total) + (x))
"""
    out = conv(src)
    assert "#include <mpi.h.cuh>" in out and "#include <gpumpi_stdio.h.cuh>" in out
    assert "#include <gpumpi_libc.h.cuh>" in out and "#include <math.h>" in out
    assert "#define TOTAL __gpu_global(total)" in out
    assert "#define ADD(total, x) ((total) + (x))" in out   # a macro parameter, not the global


def test_typedef_names_parse_as_types():
    src = "typedef unsigned long long u64; u64 count = 3; MPI_Status st;\nint f(void) { u64 x = count; return (int)x; }"
    out = squash(conv(src, 2))
    assert "__device__ u64 count[2] = {3, 3}; __device__ MPI_Status st[2];" in out
    assert "u64 x = __gpu_global(count);" in out


def test_max_ranks_from_environment(monkeypatch):
    monkeypatch.setenv(cv.MAX_RANKS_ENV, "16")
    assert cv.max_ranks_from_env() == 16
    monkeypatch.setenv(cv.MAX_RANKS_ENV, "zero")
    with pytest.raises(cv.ConversionError):
        cv.max_ranks_from_env()


def test_unbalanced_input_is_an_error():
    with pytest.raises(cv.ConversionError):
        cv.convert_source("int f( { return 0; }")


def test_project_headers_are_converted(tmp_path):
    out = cv.convert_files([PROGS / "oldstyle.c", PROGS / "oldstyle_lib.c"], tmp_path, max_ranks=4)
    assert [p.name for p in out] == ["oldstyle.cu", "oldstyle_lib.cu"]
    hdr = (tmp_path / "oldstyle.h.cuh").read_text()
    assert "__device__ extern int lib_calls[4];" in hdr
    assert '#include "oldstyle.h.cuh"' in out[0].read_text()
    assert "__device__ int lib_calls[4] = {0, 0, 0, 0};" in out[1].read_text()


@pytest.mark.skipif(shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists(),
                    reason="no nvcc")
@pytest.mark.parametrize("progs", [["rect_pi.c"], ["globals.c"], ["oldstyle.c", "oldstyle_lib.c"]])
def test_converted_programs_compile_for_sm103a(tmp_path, progs):
    import build as gbuild
    out = cv.convert_files([PROGS / p for p in progs], tmp_path, max_ranks=64)
    for f in out:
        r = subprocess.run([gbuild.nvcc(), *gbuild.common_flags(), "-I", str(tmp_path), "-I", str(PROGS), "-c",
                            str(f), "-o", str(f.with_suffix(".o"))], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]


# the reference's own toolchain test programs (staged unchanged, git-ignored, by oracle/refgpu.py)

@pytest.mark.skipif(not all((refgpu.TOOLCHAIN / p).exists() for p in refgpu.TOOLCHAIN_PROGRAMS),
                    reason="the reference's toolchain programs are not staged")
@pytest.mark.parametrize("prog", refgpu.TOOLCHAIN_PROGRAMS)
def test_reference_toolchain_programs_convert_and_compile(tmp_path, prog):
    import build as gbuild
    (out,) = cv.convert_files([refgpu.TOOLCHAIN / prog], tmp_path, max_ranks=64)
    r = subprocess.run([gbuild.nvcc(), *gbuild.common_flags(), "-I", str(tmp_path), "-c", str(out), "-o",
                        str(out.with_suffix(".o"))], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.skipif(not all((refgpu.TOOLCHAIN / p).exists() for p in refgpu.NPB_FILES),
                    reason="NPB is not staged")
@pytest.mark.parametrize("bench", ["is", "dt"])
def test_npb_converts_and_compiles(tmp_path, bench):
    # NPB IS and DT class S, npbparams.h from NPB's own setparams, converted with their project headers
    import build as gbuild
    srcs = refgpu.npb_prepare(tmp_path, bench, "S")
    out = cv.convert_files(srcs, tmp_path / "conv", max_ranks=8, project=tmp_path / "npb")
    assert (tmp_path / "conv" / "npbparams.h.cuh").exists() and (tmp_path / "conv" / "c_timers.h.cuh").exists()
    for f in out:
        r = subprocess.run([gbuild.nvcc(), *gbuild.common_flags(), "-I", str(tmp_path / "conv"), "-c", str(f), "-o",
                            str(f.with_suffix(".o"))], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]
