"""Source converter: turns a C MPI program into code that runs with one MPI rank per thread block.

The reference project does this with a clang tool (source_converter/converter.cpp).  Neither this
machine nor the GPU machine has clang or LLVM, so this module does the same rewrites over a C token
stream, with a scope-aware pass over function bodies instead of an AST:

* every function declaration and definition gets `__device__` (converter.cpp:49-75);
* `main` becomes `__gpu_main(int argc, char** argv)`, `return 0;` is made explicit at its end (C99 main
  returns 0 when it falls off its end; `__gpu_main` is an ordinary function), and after it come
  `__device__ int __gpu_max_threads()` (converter.cpp:52-64) and a host constant the launcher reads to
  refuse more ranks than the per-rank arrays hold;
* old-style (K&R) parameter lists become prototype parameter lists (converter.cpp:77-108);
* a variable with static storage (file scope, `extern`, or `static` inside a function) becomes an array
  with one element per rank: `__device__ T name[MAX_RANKS]` with its C initializer repeated for every
  rank (converter.cpp:118-144), and every reference to it becomes `__gpu_global(name)`, the calling
  rank's element (converter.cpp:145-164) -- in function bodies, honouring local declarations and
  parameters that shadow it, and in `#define` bodies; in rank r's copy of an initializer a variable it
  names (an address constant such as `&base`) becomes rank r's element `base[r]`; an array of unknown
  extent gets the extent its initializer, or for `extern`, its definition in another converted file,
  implies; a `const` object defined at file scope is defined `extern` (external in C, internal in C++);
* results of malloc/calloc/realloc stored into typed pointers get an explicit cast, the implicit
  `void*` conversion being invalid in CUDA C++ (the reference casts every implicit bit cast,
  converter.cpp:112-116);
* identifiers that are C++ keywords (`class`, `new`, `this`, ...) get the prefix `__decl_`
  (converter.cpp:166-171 renames `class`);
* `#include` lines: <mpi.h> / "mpi.h" -> <mpi.h.cuh>, <stdio.h> -> <gpumpi_stdio.h.cuh> (files and
  streams through the host channel), <stdlib.h> / <string.h> -> <gpumpi_libc.h.cuh>; headers of the
  project are converted too and included as `name.h.cuh` (the reference's gpumpicc.py renames the same
  way).

Limits (as for the reference's tool, plus those of working on tokens): an `extern` array of unknown
extent whose definition is not converted with it is refused; macros are rewritten where they are defined, so a macro whose body names a global is rewritten for every
use; block-scope function prototypes are left alone; the program is expected to be C (C++ classes are
not converted).  Output files: `x.c` -> `x.cu`, a project header `y.h` -> `y.h.cuh`.
"""
from __future__ import annotations

import os
import re
from dataclasses import dataclass, field
from pathlib import Path

MAX_RANKS_ENV = "GPU_MPI_MAX_RANKS"   # the reference's variables (converter.cpp:24-25)
PROJECT_ENV = "GPU_MPI_PROJECT"
DEFAULT_MAX_RANKS = 1024


class ConversionError(Exception):
    pass


def max_ranks_from_env() -> int:
    v = os.environ.get(MAX_RANKS_ENV)
    if v is None:
        return DEFAULT_MAX_RANKS
    try:
        n = int(v)
    except ValueError:
        n = 0
    if n <= 0:
        raise ConversionError(f"{MAX_RANKS_ENV} should contain a positive number of ranks")
    return n


# ------------------------------------------------------------------------------------------------
# tokens
# ------------------------------------------------------------------------------------------------
_TOKEN = re.compile(r"""
  (?P<nl>\n)
| (?P<ws>(?:[ \t\r\f\v]|\\\n)+)
| (?P<comment>//(?:[^\n\\]|\\.)*|/\*.*?\*/)
| (?P<str>(?:u8|[uUL])?"(?:\\.|[^"\\\n])*")
| (?P<chr>(?:u8|[uUL])?'(?:\\.|[^'\\\n])*')
| (?P<num>\.?[0-9](?:[eEpP][+-]|[0-9A-Za-z_.])*)
| (?P<id>[A-Za-z_][A-Za-z_0-9]*)
| (?P<op>\.\.\.|<<=|>>=|->|\+\+|--|<<|>>|<=|>=|==|!=|&&|\|\||[-+*/%&|^]=|\#\#|[][{}();,.<>+\-*/%&|^!~?:=\#])
| (?P<other>.)
""", re.S | re.X)

STORAGE = {"typedef", "extern", "static", "auto", "register", "_Thread_local", "inline", "__inline",
           "__inline__", "_Noreturn"}
QUALS = {"const", "volatile", "restrict", "__restrict", "__restrict__", "_Atomic"}
BASE = {"void", "char", "short", "int", "long", "float", "double", "signed", "unsigned", "_Bool", "_Complex",
        "__int128"}
TAGS = {"struct", "union", "enum"}
ATTRS = {"__attribute__", "__declspec", "__extension__", "__asm__", "asm"}
C_KEYWORDS = STORAGE | QUALS | BASE | TAGS | {
    "break", "case", "continue", "default", "do", "else", "for", "goto", "if", "return", "sizeof", "switch",
    "while", "_Alignas", "_Alignof", "_Generic", "_Static_assert"}
CXX_KEYWORDS = {"class", "new", "delete", "this", "template", "typename", "namespace", "operator", "private",
                "protected", "public", "virtual", "friend", "explicit", "mutable", "catch", "try", "throw",
                "using", "nullptr", "export", "reinterpret_cast", "static_cast", "dynamic_cast",
                "const_cast", "typeid", "decltype", "constexpr", "noexcept", "thread_local", "alignof",
                "alignas", "char16_t", "char32_t", "static_assert"}
KNOWN_TYPES = {
    "MPI_Comm", "MPI_Datatype", "MPI_Status", "MPI_Request", "MPI_Op", "MPI_Group", "MPI_Aint", "MPI_Offset",
    "MPI_File", "MPI_Info", "MPI_Fint", "MPI_Errhandler", "MPI_User_function", "MPI_Copy_function",
    "MPI_Delete_function", "FILE", "va_list", "bool", "wchar_t", "div_t", "ldiv_t", "lldiv_t", "fpos_t"}
ALLOCATORS = {"malloc", "calloc", "realloc", "aligned_alloc"}
INCLUDE_MAP = {"mpi.h": "mpi.h.cuh", "stdio.h": "gpumpi_stdio.h.cuh", "stdlib.h": "gpumpi_libc.h.cuh",
               "string.h": "gpumpi_libc.h.cuh"}
PRELUDE = ("#define GPUMPI_STDIO_NAMES\n#define GPUMPI_LIBC_NAMES\n#include <gpumpi_libc.h.cuh>\n"
           "#include <mpi.h.cuh>\n#include <gpumpi_stdio.h.cuh>\n")


@dataclass
class Tok:
    kind: str
    text: str


def tokenize(src: str) -> list[Tok]:
    """Lossless token list; a preprocessor directive (from a line-initial '#' to the end of its logical
    line) is one token of kind 'dir'."""
    raw = [Tok(m.lastgroup, m.group()) for m in _TOKEN.finditer(src)]
    out: list[Tok] = []
    line_start = True
    i = 0
    while i < len(raw):
        t = raw[i]
        if line_start and t.kind == "op" and t.text == "#":
            j = i
            while j < len(raw) and raw[j].kind != "nl":
                j += 1
            out.append(Tok("dir", "".join(x.text for x in raw[i:j])))
            i = j
            continue
        if t.kind == "nl":
            line_start = True
        elif t.kind not in ("ws", "comment"):
            line_start = False
        out.append(t)
        i += 1
    return out


def c_string_length(lit: str) -> int:
    """Characters of a narrow C string literal's contents (escape sequences count as one)."""
    body = lit[lit.index('"') + 1:-1]
    n, i = 0, 0
    while i < len(body):
        if body[i] == "\\" and i + 1 < len(body):
            i += 1
            if body[i] == "x":
                i += 1
                while i < len(body) and body[i] in "0123456789abcdefABCDEF":
                    i += 1
            elif body[i] in "01234567":
                j = i
                while i < len(body) and i < j + 3 and body[i] in "01234567":
                    i += 1
            else:
                i += 1
        else:
            i += 1
        n += 1
    return n


def is_sig(t: Tok) -> bool:
    return t.kind not in ("ws", "nl", "comment", "dir")


# ------------------------------------------------------------------------------------------------
# declarations
# ------------------------------------------------------------------------------------------------
@dataclass
class Declarator:
    start: int            # sig index range [start, end) of the declarator, initializer included
    end: int
    name: int | None      # sig index of the declared identifier
    is_function: bool
    init: int | None      # sig index of the first initializer token
    stars: int
    brackets: int


@dataclass
class Declaration:
    start: int            # sig index of the first specifier
    spec_end: int         # sig index after the specifiers
    storage: set
    decls: list
    type_text: str        # specifiers without storage classes (for casts)


class Converter:
    def __init__(self, src: str, max_ranks: int, extra_types=(), is_main_file=True, globals_in=None,
                 include_map=None, structs_in=None, functions_in=None, array_sizes_in=None):
        self.toks = tokenize(src)
        self.sig = [i for i, t in enumerate(self.toks) if is_sig(t)]
        self.max_ranks = max_ranks
        self.types = set(KNOWN_TYPES) | set(extra_types)
        self.is_main_file = is_main_file
        self.globals: dict[str, tuple] = dict(globals_in or {})   # name -> (type_text, stars, brackets)
        self.include_map = include_map or {}
        self.prefix: dict[int, str] = {}
        self.suffix: dict[int, str] = {}
        self.repl: dict[int, str] = {}
        self.match = self._match_brackets()
        self.saw_main = False
        self.structs: dict[str, dict] = dict(structs_in or {})  # struct key -> member -> (type, stars, brackets)
        self.functions: dict[str, tuple] = dict(functions_in or {})  # name -> (return type, parameters or None)
        # name -> first extent of a file-scope array defined with one (an `extern T x[];` elsewhere needs it)
        self.array_sizes: dict[str, str] = dict(array_sizes_in or {})
        self._ret = None                       # return type of the function being converted

    # ---- token helpers (k = sig index) ----
    def t(self, k: int) -> str:
        return self.toks[self.sig[k]].text if 0 <= k < len(self.sig) else ""

    def kind(self, k: int) -> str:
        return self.toks[self.sig[k]].kind if 0 <= k < len(self.sig) else ""

    def is_id(self, k: int) -> bool:
        return self.kind(k) == "id"

    def _match_brackets(self) -> dict:
        m, stack = {}, []
        pairs = {")": "(", "]": "[", "}": "{"}
        for k in range(len(self.sig)):
            x = self.t(k)
            if self.kind(k) != "op":
                continue
            if x in "([{":
                stack.append(k)
            elif x in ")]}":
                if not stack or self.t(stack[-1]) != pairs[x]:
                    raise ConversionError(f"unbalanced '{x}' near token {k}")
                o = stack.pop()
                m[o], m[k] = k, o
        if stack:
            raise ConversionError(f"unclosed '{self.t(stack[-1])}'")
        return m

    def add_prefix(self, k: int, s: str):
        i = self.sig[k]
        self.prefix[i] = self.prefix.get(i, "") + s

    def add_suffix(self, k: int, s: str):
        i = self.sig[k]
        self.suffix[i] = s + self.suffix.get(i, "")

    def replace(self, k: int, s: str):
        self.repl[self.sig[k]] = s

    def raw_text(self, a: int, b: int) -> str:
        """Source text from sig token a through sig token b (inclusive), everything between included."""
        return "".join(t.text for t in self.toks[self.sig[a]:self.sig[b] + 1])

    def is_type_name(self, name: str) -> bool:
        return name in self.types or (name.endswith("_t") and name not in self.globals)

    # ---- declaration parsing over [a, b) ----
    def parse_declaration(self, a: int, b: int) -> Declaration:
        k = a
        storage, has_base, type_parts = set(), False, []
        while k < b:
            x = self.t(k)
            if x in STORAGE:
                storage.add(x)
                k += 1
            elif x in QUALS or x in BASE:
                has_base = has_base or x in BASE
                type_parts.append(x)
                k += 1
            elif x in TAGS:
                has_base = True
                j = k + 1
                if self.is_id(j):
                    j += 1
                if self.t(j) == "{":
                    j = self.match[j] + 1
                type_parts.append(self.raw_text(k, j - 1))
                k = j
            elif x in ATTRS:
                k += 1
                if self.t(k) == "(":
                    k = self.match[k] + 1
            elif self.is_id(k) and not has_base and self.is_type_name(x):
                has_base = True
                type_parts.append(x)
                k += 1
            else:
                break
        spec_end = k
        decls = []
        s = k
        while s < b:
            e, init = s, None
            while e < b and self.t(e) != ",":
                x = self.t(e)
                if x == "=" and init is None:
                    init = e + 1
                if x in ("(", "[", "{"):
                    e = self.match[e]
                e += 1
            decls.append(self._declarator(s, e, init))
            s = e + 1
        return Declaration(a, spec_end, storage, decls, " ".join(type_parts))

    def _declarator(self, s: int, e: int, init) -> Declarator:
        stop = (init - 1) if init is not None else e
        name, stars, k = None, 0, s
        while k < stop:
            x = self.t(k)
            if x == "*":
                stars += 1
            elif x in ATTRS:
                if self.t(k + 1) == "(":
                    k = self.match[k + 1]
            elif self.is_id(k) and x not in QUALS:
                name = k
                break
            k += 1
        is_fn, brackets = False, 0
        if name is not None:
            j = name + 1
            is_fn = self.t(j) == "("
            while j < stop and self.t(j) == "[":
                brackets += 1
                j = self.match[j] + 1
        return Declarator(s, e, name, is_fn, init, stars, brackets)

    def starts_declaration(self, k: int) -> bool:
        x = self.t(k)
        if x in STORAGE or x in QUALS or x in BASE or x in TAGS:
            return True
        if self.is_id(k) and self.is_type_name(x):
            return self.is_id(k + 1) or self.t(k + 1) == "*"
        return False

    # ---- the conversion ----
    def run(self) -> str:
        self._collect_typedefs_and_globals()
        k = 0
        n = len(self.sig)
        while k < n:
            k = self._top_level_item(k)
        self._directives()
        self._rename_cxx_keywords()
        return self._emit()

    def _collect_typedefs_and_globals(self):
        """First pass: typedef names (for parsing), the file-scope variables (for references that come
        before a later tentative definition, and for macro bodies), struct members and function signatures
        (for the casts of void* values)."""
        k, n = 0, len(self.sig)
        while k < n:
            end, body = self._item_extent(k)
            if body is None and end > k:
                d = self.parse_declaration(k, end)
                self._record_structs(d)
                for dd in d.decls:
                    if dd.name is None:
                        continue
                    if "typedef" in d.storage:
                        self.types.add(self.t(dd.name))
                    elif dd.is_function:
                        self.functions[self.t(dd.name)] = (
                            (d.type_text, dd.stars, 0), self._param_infos(dd.name + 1, self.match[dd.name + 1]))
                    else:
                        self.globals[self.t(dd.name)] = (d.type_text, dd.stars, dd.brackets)
                        ext = self._first_extent(dd) if dd.brackets else None
                        if ext is not None:
                            self.array_sizes[self.t(dd.name)] = ext
            elif body is not None:
                d = self.parse_declaration(k, body[0])
                fn = next((dd for dd in d.decls if dd.name is not None and dd.is_function), None)
                if fn is not None:
                    self.functions[self.t(fn.name)] = (
                        (d.type_text, fn.stars, 0), self._param_infos(fn.name + 1, self.match[fn.name + 1]))
            k = (body[1] + 1) if body else end + 1

    # ---- types of simple expressions (the casts of void* values) ----
    @staticmethod
    def _type_key(type_text: str) -> str:
        words = [w for w in type_text.replace("{", " { ").split() if w not in QUALS]
        if words and words[0] in TAGS:
            return " ".join(words[:2]) if len(words) > 1 and words[1] != "{" else ""
        return " ".join(words)

    def _record_structs(self, d: Declaration):
        """Members of a struct/union body in the specifiers of declaration d, under `struct Tag` and under
        the typedef names that denote the struct itself; `typedef struct Tag Name;` aliases a known one."""
        k = d.start
        while k < d.spec_end:
            if self.t(k) in TAGS:
                tag = self.t(k + 1) if self.is_id(k + 1) else None
                j = k + (2 if tag else 1)
                names = [f"{self.t(k)} {tag}"] if tag else []
                if "typedef" in d.storage:
                    names += [self.t(dd.name) for dd in d.decls if dd.name is not None and dd.stars == 0
                              and dd.brackets == 0 and not dd.is_function]
                if self.t(j) == "{":
                    members, s = {}, j + 1
                    while s < self.match[j]:
                        e = s
                        while e < self.match[j] and self.t(e) != ";":
                            if self.t(e) in ("(", "[", "{"):
                                e = self.match[e]
                            e += 1
                        md = self.parse_declaration(s, e)
                        self._record_structs(md)
                        for dd in md.decls:
                            if dd.name is not None and not dd.is_function:
                                members[self.t(dd.name)] = (md.type_text, dd.stars, dd.brackets)
                        s = e + 1
                    for nm in names:
                        self.structs[nm] = members
                    k = self.match[j] + 1
                    continue
                if tag and f"{self.t(k)} {tag}" in self.structs:
                    for nm in names[1:]:
                        self.structs[nm] = self.structs[f"{self.t(k)} {tag}"]
            k += 1

    def _param_infos(self, lp: int, rp: int):
        """Parameter types of a prototype list, or None for an old-style list (types unknown here)."""
        inner = list(range(lp + 1, rp))
        if not inner or (len(inner) == 1 and self.t(inner[0]) == "void"):
            return []
        out, s = [], lp + 1
        while s < rp:
            e = s
            while e < rp and self.t(e) != ",":
                if self.t(e) in ("(", "["):
                    e = self.match[e]
                e += 1
            if self.t(s) == "...":
                break
            if e - s == 1 and self.is_id(s) and not self.is_type_name(self.t(s)) and self.t(s) not in C_KEYWORDS:
                return None   # an identifier list
            d = self.parse_declaration(s, e)
            dd = d.decls[0] if d.decls else None
            out.append((d.type_text, dd.stars if dd else 0, dd.brackets if dd else 0))
            s = e + 1
        return out

    def _chain_info(self, a: int, b: int, scopes: list):
        """Type of sig range [a, b) when it is `name` followed by member accesses and subscripts, else
        None."""
        if a >= b or not self.is_id(a):
            return None
        r = self._lookup(scopes, self.t(a))
        if r is None or r[1] is None:
            return None
        tt, st, br = r[1]
        k = a + 1
        while k < b:
            x = self.t(k)
            if x == "[":
                if self.match[k] >= b:
                    return None
                if br > 0:
                    br -= 1
                elif st > 0:
                    st -= 1
                else:
                    return None
                k = self.match[k] + 1
            elif x in ("->", ".") and self.is_id(k + 1):
                if x == "->":
                    if br > 0:
                        br -= 1
                    elif st > 0:
                        st -= 1
                    else:
                        return None
                if st or br:
                    return None
                mem = self.structs.get(self._type_key(tt))
                if mem is None or self.t(k + 1) not in mem:
                    return None
                tt, st, br = mem[self.t(k + 1)]
                k += 2
            else:
                return None
        return (tt, st, br)

    def _void_ptr(self, info) -> bool:
        return info is not None and self._type_key(info[0]) == "void" and info[1] == 1 and info[2] == 0

    def _typed_ptr(self, info) -> bool:
        return (info is not None and info[2] == 0 and info[1] >= 1 and
                not (self._type_key(info[0]) == "void" and info[1] == 1))

    def _cast_void_value(self, a: int, b: int, target, scopes: list):
        """An explicit cast to `target` before sig range [a, b) when it is a void* chain."""
        if self._typed_ptr(target) and self._void_ptr(self._chain_info(a, b, scopes)):
            i = self.sig[a]
            self.prefix[i] = self._cast_type(target[0], target[1]) + self.prefix.get(i, "")

    def _cast_call_args(self, a: int, b: int, scopes: list):
        """Arguments that are void* chains passed to typed pointer parameters of known functions."""
        for k in range(a, b):
            if not (self.is_id(k) and self.t(k + 1) == "(" and self.t(k) in self.functions):
                continue
            if self.t(k - 1) in (".", "->"):
                continue
            r = self._lookup(scopes, self.t(k))
            if r is not None and r[0] != "global":
                continue
            params = self.functions[self.t(k)][1]
            close = self.match[k + 1]
            if not params or close > b:
                continue
            s, i = k + 2, 0
            while s < close and i < len(params):
                e = s
                while e < close and self.t(e) != ",":
                    if self.t(e) in ("(", "[", "{"):
                        e = self.match[e]
                    e += 1
                self._cast_void_value(s, e, params[i], scopes)
                s, i = e + 1, i + 1

    def _item_extent(self, k: int):
        """Extent of the top-level item starting at sig index k: (index of its ';' or of the token after
        a function body, (body_open, body_close) or None)."""
        n = len(self.sig)
        j, seen_eq, prev = k, False, ""
        while j < n:
            x = self.t(j)
            if x in ("(", "["):
                j = self.match[j] + 1
                prev = ")" if x == "(" else "]"
                continue
            if x == "{":
                p1, p2 = self.t(j - 1), self.t(j - 2)
                if seen_eq or p1 in TAGS or (self.is_id(j - 1) and p2 in TAGS):
                    j = self.match[j] + 1
                    prev = "}"
                    continue
                return j, (j, self.match[j])
            if x == "=":
                seen_eq = True
            elif x == ",":
                seen_eq = False
            elif x == ";":
                # an old-style definition continues with its parameter declarations up to the body
                if self._knr_header(k, j):
                    j2 = j
                    while j2 < n and self.t(j2) != "{":
                        if self.t(j2) in ("(", "["):
                            j2 = self.match[j2]
                        j2 += 1
                    if j2 < n:
                        return j2, (j2, self.match[j2])
                return j, None
            prev = x
            j += 1
        return j, None

    def _knr_header(self, k: int, semi: int) -> bool:
        """Does [k, semi) hold `... name ( ident, ident ) decl-specifiers ...` (an old-style definition's
        header followed by its first parameter declaration)?"""
        j = k
        while j < semi:
            if self.t(j) == "(" and self.is_id(j - 1):
                close = self.match[j]
                inner = list(range(j + 1, close))
                if inner and all((self.is_id(q) and self.t(q) not in C_KEYWORDS and not self.is_type_name(self.t(q)))
                                 or self.t(q) == "," for q in inner):
                    nxt = close + 1
                    return nxt < semi and self.starts_declaration(nxt)
                j = close
            j += 1
        return False

    def _top_level_item(self, k: int) -> int:
        end, body = self._item_extent(k)
        if body is None:
            if end > k:
                self._global_declaration(k, end)
            return end + 1
        open_, close = body
        self._function_definition(k, open_, close)
        return close + 1

    def _object_const(self, d: Declaration, dd: Declarator) -> bool:
        """Whether the declared object itself is const (not only what it points to)."""
        if dd.stars == 0:
            return "const" in d.type_text.split()
        last_star = max(k for k in range(dd.start, dd.name) if self.t(k) == "*")
        return any(self.t(k) == "const" for k in range(last_star + 1, dd.name))

    def _global_declaration(self, a: int, b: int):
        d = self.parse_declaration(a, b)
        if "typedef" in d.storage or not d.decls:
            return
        if any(dd.name is not None for dd in d.decls):
            self.add_prefix(a, "__device__ ")
        # a const object at file scope has external linkage in C but internal linkage in C++: its
        # definition keeps it visible to the other files' extern declarations
        objs = [dd for dd in d.decls if dd.name is not None and not dd.is_function]
        if (objs and not ({"static", "extern"} & d.storage) and all(dd.init is not None for dd in objs)
                and any(self._object_const(d, dd) for dd in objs)):
            self.add_prefix(a, "extern ")
        for dd in d.decls:
            if dd.name is None or dd.is_function:
                continue
            self._make_per_rank(d, dd)

    def _first_extent(self, dd: Declarator):
        """The first dimension of array declarator dd as text: written in the brackets, else the element
        count of its initializer (a braced list, designators included, or a string literal); None when
        neither says."""
        lb = dd.name + 1
        if self.t(lb) != "[":
            return None
        if self.match[lb] != lb + 1:
            return self._rank_text(lb + 1, self.match[lb] - 1, 0)
        if dd.init is None:
            return None
        if self.kind(dd.init) == "str":
            n, k = 0, dd.init
            while k < dd.end and self.kind(k) == "str":
                n += c_string_length(self.t(k))
                k += 1
            return str(n + 1)
        if self.t(dd.init) != "{":
            return None
        close = self.match[dd.init]
        pos = size = 0
        k = dd.init + 1
        while k < close:
            if self.t(k) == "[":  # designator [index] = value
                idx = self.raw_text(k + 1, self.match[k] - 1).strip()
                if not re.fullmatch(r"[0-9]+[uUlL]*", idx):
                    return None
                pos = int(re.match(r"[0-9]+", idx).group())
            e = k
            while e < close and self.t(e) != ",":
                if self.t(e) in ("(", "[", "{"):
                    e = self.match[e]
                e += 1
            if e > k:
                size = max(size, pos + 1)
                pos += 1
            k = e + 1
        return str(size)

    def _rank_text(self, a: int, b: int, r: int) -> str:
        """Raw text of tokens [a, b] for rank r's copy of an initializer: a file-scope variable named in it
        (an address constant such as `&base` or an array decaying to its first element) becomes rank r's
        element of that variable, `name[r]`."""
        out, prev = [], None
        for i in range(self.sig[a], self.sig[b] + 1):
            tok = self.toks[i]
            txt = tok.text
            if tok.kind == "id" and txt in self.globals and prev not in (".", "->"):
                txt = f"{txt}[{r}]"
            if is_sig(tok):
                prev = tok.text
            out.append(txt)
        return "".join(out).strip()

    def _make_per_rank(self, d: Declaration, dd: Declarator):
        name = self.t(dd.name)
        self.add_suffix(dd.name, f"[{self.max_ranks}]")
        if self.t(dd.name + 1) == "[" and self.match[dd.name + 1] == dd.name + 2:
            # an array of unknown first extent cannot be an element type: give it the extent its
            # initializer, or (extern) its definition in another converted file, implies
            ext = self._first_extent(dd) or self.array_sizes.get(name)
            if ext is None:
                raise ConversionError(f"array '{name}' has no size here and its definition is not among the "
                                      "converted files")
            self.add_suffix(dd.name + 1, ext)
        # a global named in the dimensions (`sizeof(src) / sizeof(src[0])`) means one rank's copy of it
        k = dd.name + 1
        while self.t(k) == "[":
            for q in range(k + 1, self.match[k]):
                if self.kind(q) == "id" and self.t(q) in self.globals and self.t(q - 1) not in (".", "->"):
                    self.add_suffix(q, "[0]")
            k = self.match[k] + 1
        if dd.init is not None:
            last = dd.end - 1
            if self.t(dd.init) == "{" and self.match[dd.init] != last:
                raise ConversionError(f"initializer of '{name}' is not a single braced list")
            self.replace(dd.init, "{" + ", ".join(self._rank_text(dd.init, last, r)
                                                   for r in range(self.max_ranks)) + "}")
            for q in range(dd.init + 1, last + 1):
                self.replace(q, "")
            # drop the layout between the removed tokens (their text is inside the replacement)
            for i in range(self.sig[dd.init] + 1, self.sig[last] + 1):
                if not is_sig(self.toks[i]):
                    self.repl[i] = ""

    def _function_definition(self, a: int, open_: int, close: int):
        # declarator: find the function's name (the identifier before the '(' of its parameter list)
        d = self.parse_declaration(a, open_)
        fn = next((dd for dd in d.decls if dd.name is not None and dd.is_function), None)
        if fn is None:
            raise ConversionError(f"cannot find the name of the function defined before token {open_}")
        self.add_prefix(a, "__device__ ")
        name_k = fn.name
        lp = name_k + 1
        rp = self.match[lp]
        params = self._parameters(lp, rp, open_)   # name -> (type, stars, brackets) or None
        if self.t(name_k) == "main":
            self.saw_main = True
            self.replace(name_k, "__gpu_main")
            if d.type_text.split() and d.type_text.split()[-1] != "int":
                raise ConversionError("main must return int")
            if len(params) == 0:
                self.replace(lp, "(int argc, char** argv")
                for q in range(lp + 1, rp):
                    self.replace(q, "")
            self.add_prefix(close, "    return 0;\n")
            self.add_suffix(close, f"\n__device__ int __gpu_max_threads() {{ return {self.max_ranks}; }}\n"
                                   f"extern \"C\" const int gpumpi_program_max_ranks = {self.max_ranks};")
        scope = {p: ("local", info) for p, info in params.items()}
        self._ret = (d.type_text, fn.stars, 0)
        self._body(open_ + 1, close, [scope])
        self._ret = None

    def _parameters(self, lp: int, rp: int, body_open: int) -> dict:
        """The parameters, name -> (type text, stars, brackets); rewrites an old-style list (identifiers,
        then declarations before the body) into a prototype list."""
        inner = list(range(lp + 1, rp))
        if not inner or (len(inner) == 1 and self.t(inner[0]) == "void"):
            return {}
        if rp + 1 < body_open:   # old-style: declarations between ')' and '{'
            names = [self.t(q) for q in inner if self.is_id(q)]
            typed, infos = {}, {}
            k = rp + 1
            while k < body_open:
                e = k
                while e < body_open and self.t(e) != ";":
                    e += 1
                d = self.parse_declaration(k, e)
                spec = " ".join(x for x in self.raw_text(k, d.spec_end - 1).split() if x != "register")
                for dd in d.decls:
                    if dd.name is not None:
                        typed[self.t(dd.name)] = spec + " " + self.raw_text(dd.start, dd.end - 1).strip()
                        infos[self.t(dd.name)] = (d.type_text, dd.stars, dd.brackets)
                k = e + 1
            self.replace(lp, "(" + ", ".join(typed.get(nm, "int " + nm) for nm in names))
            for q in range(lp + 1, rp):
                self.replace(q, "")
            for q in range(rp + 1, body_open):
                self.replace(q, "")
            for i in range(self.sig[rp] + 1, self.sig[body_open]):
                if not is_sig(self.toks[i]):
                    self.repl[i] = ""
            self.add_suffix(rp, " ")
            return {nm: infos.get(nm, ("int", 0, 0)) for nm in names}
        names, s = {}, lp + 1
        while s < rp:
            e = s
            while e < rp and self.t(e) != ",":
                if self.t(e) in ("(", "["):
                    e = self.match[e]
                e += 1
            if self.t(s) != "...":
                d = self.parse_declaration(s, e)
                for dd in d.decls:
                    if dd.name is not None:
                        names[self.t(dd.name)] = (d.type_text, dd.stars, dd.brackets)
            s = e + 1
        return names

    # ---- function bodies ----
    def _lookup(self, scopes: list, name: str):
        for sc in reversed(scopes):
            if name in sc:
                return sc[name]
        if name in self.globals:
            return ("global", self.globals[name])
        return None

    def _body(self, a: int, b: int, scopes: list):
        """Statements in sig range [a, b) of a block whose scopes are `scopes` (innermost last)."""
        k = a
        while k < b:
            k = self._statement(k, b, scopes)

    def _statement(self, k: int, b: int, scopes: list) -> int:
        x = self.t(k)
        if x == "{":
            close = self.match[k]
            scopes.append({})
            self._body(k + 1, close, scopes)
            scopes.pop()
            return close + 1
        if x == ";":
            return k + 1
        if x in ("if", "while", "switch") and self.t(k + 1) == "(":
            close = self.match[k + 1]
            self._expr(k + 2, close, scopes)
            j = self._statement(close + 1, b, scopes)
            if x == "if" and self.t(j) == "else":
                j = self._statement(j + 1, b, scopes)
            return j
        if x == "for" and self.t(k + 1) == "(":
            close = self.match[k + 1]
            scopes.append({})
            s = k + 2
            first = s
            while first < close and self.t(first) != ";":
                if self.t(first) in ("(", "[", "{"):
                    first = self.match[first]
                first += 1
            if self.starts_declaration(s):
                self._local_declaration(s, first, scopes)
            else:
                self._expr(s, first, scopes)
            self._expr(first + 1, close, scopes)
            j = self._statement(close + 1, b, scopes)
            scopes.pop()
            return j
        if x == "do":
            j = self._statement(k + 1, b, scopes)
            if self.t(j) == "while" and self.t(j + 1) == "(":
                close = self.match[j + 1]
                self._expr(j + 2, close, scopes)
                return close + 2
            return j
        if x in ("case", "default"):
            j = k + 1
            while j < b and self.t(j) != ":":
                if self.t(j) in ("(", "["):
                    j = self.match[j]
                j += 1
            self._expr(k + 1, j, scopes)
            return j + 1
        if self.is_id(k) and self.t(k + 1) == ":" and x not in C_KEYWORDS:   # label
            return k + 2
        if x == "goto":
            return self._skip_to_semicolon(k, b) + 1
        end = self._skip_to_semicolon(k, b)
        if self.starts_declaration(k):
            self._local_declaration(k, end, scopes)
        elif x == "return":
            self._expr(k + 1, end, scopes)
            if self._ret is not None:
                self._cast_void_value(k + 1, end, self._ret, scopes)
        else:
            self._expr(k, end, scopes)
            self._cast_assignment(k, end, scopes)
        return end + 1

    def _skip_to_semicolon(self, k: int, b: int) -> int:
        while k < b and self.t(k) != ";":
            if self.t(k) in ("(", "[", "{"):
                k = self.match[k]
            k += 1
        return k

    def _local_declaration(self, a: int, b: int, scopes: list):
        d = self.parse_declaration(a, b)
        if "typedef" in d.storage:
            for dd in d.decls:
                if dd.name is not None:
                    self.types.add(self.t(dd.name))
            return
        is_static = "static" in d.storage or "extern" in d.storage
        for dd in d.decls:
            if dd.name is None:
                continue
            nm = self.t(dd.name)
            if dd.is_function:
                scopes[-1][nm] = ("local", None)
                continue
            info = (d.type_text, dd.stars, dd.brackets)
            # the initializer is evaluated in the scope where the name is already declared (C rules); a
            # static's initializer is a constant
            if dd.init is not None and not is_static:
                self._expr(dd.init, dd.end, scopes)
                self._cast_initializer(d, dd)
                if dd.brackets == 0:
                    self._cast_void_value(dd.init, dd.end, (d.type_text, dd.stars, 0), scopes)
            if is_static:
                if "extern" in d.storage:
                    scopes[-1][nm] = ("global", self.globals.get(nm, info))
                else:
                    self._make_per_rank(d, dd)
                    scopes[-1][nm] = ("static", info)
            else:
                scopes[-1][nm] = ("local", info)
            # array bounds inside the declarator
            q = dd.name + 1
            while q < (dd.init - 1 if dd.init is not None else dd.end) and self.t(q) == "[":
                self._expr(q + 1, self.match[q], scopes)
                q = self.match[q] + 1

    def _expr(self, a: int, b: int, scopes: list):
        """Wraps references to per-rank variables among the identifiers of sig range [a, b)."""
        for k in range(a, b):
            if not self.is_id(k):
                continue
            prev = self.t(k - 1)
            if prev in (".", "->") or prev in TAGS or prev == "goto":
                continue
            r = self._lookup(scopes, self.t(k))
            if r is not None and r[0] in ("global", "static"):
                self._wrap(k)
        self._cast_call_args(a, b, scopes)

    def _wrap(self, k: int):
        self.add_prefix(k, "__gpu_global(")
        self.add_suffix(k, ")")

    def _cast_type(self, type_text: str, stars: int) -> str:
        return f"({type_text} {'*' * stars})".replace(" )", ")")

    def _cast_initializer(self, d: Declaration, dd: Declarator):
        if dd.init is None or dd.stars == 0 or dd.brackets:
            return
        if self.t(dd.init) in ALLOCATORS and self.t(dd.init + 1) == "(":
            self.add_prefix(dd.init, self._cast_type(d.type_text, dd.stars))

    def _cast_assignment(self, a: int, b: int, scopes: list):
        """`p = malloc(...)` or `p[i] = malloc(...)` with p's declared pointer type known, or `lhs = chain`
        where the chain has type void* and lhs a typed pointer: an explicit cast."""
        if not self.is_id(a):
            return
        eq = a
        while eq < b and self.t(eq) != "=":
            if self.t(eq) in ("(", "[", "{"):
                eq = self.match[eq]
            eq += 1
        if eq < b and not (self.t(eq + 1) in ALLOCATORS and self.t(eq + 2) == "("):
            self._cast_void_value(eq + 1, b, self._chain_info(a, eq, scopes), scopes)
            return
        k, subs = a + 1, 0
        while k < b and self.t(k) == "[":
            subs += 1
            k = self.match[k] + 1
        if self.t(k) != "=" or not (self.t(k + 1) in ALLOCATORS and self.t(k + 2) == "("):
            return
        r = self._lookup(scopes, self.t(a))
        if r is None or r[1] is None:
            return
        type_text, stars, brackets = r[1]
        if subs < brackets:            # still an array
            return
        left = stars - (subs - brackets)
        if left <= 0:
            return
        self.add_prefix(k + 1, self._cast_type(type_text, left))

    # ---- directives and keywords ----
    def _directives(self):
        for i, t in enumerate(self.toks):
            if t.kind != "dir":
                continue
            m = re.match(r'(\s*#\s*include\s*)([<"])([^>"]+)([>"])(.*)$', t.text, re.S)
            if m:
                hdr = m.group(3).strip()
                new = self.include_map.get(hdr)
                if new is not None:
                    self.repl[i] = f'{m.group(1)}"{new}"{m.group(5)}'
                elif hdr in INCLUDE_MAP:
                    self.repl[i] = f"{m.group(1)}<{INCLUDE_MAP[hdr]}>{m.group(5)}"
                continue
            m = re.match(r"(\s*#\s*define\s+)([A-Za-z_]\w*)(\([^)]*\))?(.*)$", t.text, re.S)
            if m:
                params = set(re.findall(r"[A-Za-z_]\w*", m.group(3) or ""))
                body = tokenize(m.group(4))
                out, prev = [], ""
                for bt in body:
                    txt = bt.text
                    if bt.kind == "id" and txt in self.globals and txt not in params and prev not in (".", "->", "#"):
                        txt = f"__gpu_global({txt})"
                    elif bt.kind == "id" and txt in CXX_KEYWORDS:
                        txt = "__decl_" + txt
                    out.append(txt)
                    if is_sig(bt):
                        prev = bt.text
                self.repl[i] = m.group(1) + m.group(2) + (m.group(3) or "") + "".join(out)

    def _rename_cxx_keywords(self):
        for i in self.sig:
            t = self.toks[i]
            if t.kind == "id" and t.text in CXX_KEYWORDS:
                self.repl[i] = "__decl_" + self.repl.get(i, t.text)

    def _emit(self) -> str:
        parts = [PRELUDE]
        for i, t in enumerate(self.toks):
            parts.append(self.prefix.get(i, ""))
            parts.append(self.repl.get(i, t.text))
            parts.append(self.suffix.get(i, ""))
        return "".join(parts)


# ------------------------------------------------------------------------------------------------
# files
# ------------------------------------------------------------------------------------------------
_INCLUDE = re.compile(r'^\s*#\s*include\s*"([^"]+)"', re.M)


def convert_source(src: str, max_ranks: int = DEFAULT_MAX_RANKS, extra_types=(), include_map=None,
                   globals_in=None) -> str:
    """Converts one translation unit's text; see the module docstring for the rewrites."""
    return Converter(src, max_ranks, extra_types, globals_in=globals_in, include_map=include_map).run()


def _project_headers(path: Path, project: Path, include_dirs, seen: dict):
    """Project headers a file includes with "...", recursively: {header path: include text}."""
    text = path.read_text()
    for name in _INCLUDE.findall(text):
        for d in [path.parent, *include_dirs]:
            cand = (Path(d) / name).resolve()
            if cand.is_file() and str(cand).startswith(str(project)) and cand.name != "mpi.h":
                if cand not in seen:
                    seen[cand] = name
                    _project_headers(cand, project, include_dirs, seen)
                break
    return seen


def convert_files(sources, out_dir, max_ranks: int | None = None, include_dirs=(), project=None,
                  extra_types=()) -> list:
    """Converts C sources (and the project headers they include) into out_dir: x.c -> x.cu, y.h ->
    y.h.cuh (the reference's gpumpicc.py naming).  Returns the converted sources' paths."""
    max_ranks = max_ranks or max_ranks_from_env()
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    srcs = [Path(s).resolve() for s in sources]
    project = Path(project or os.environ.get(PROJECT_ENV) or srcs[0].parent).resolve()
    # first extents of the file-scope arrays defined in any of the sources (for extern declarations of
    # unknown extent in the others)
    sizes: dict[str, str] = {}
    for src in srcs:
        c = Converter(src.read_text(), max_ranks, extra_types)
        c._collect_typedefs_and_globals()
        sizes.update(c.array_sizes)
    converted = []
    for src in srcs:
        headers = _project_headers(src, project, [Path(d).resolve() for d in include_dirs], {})
        imap = {name: Path(name).name + ".cuh" for name in headers.values()}
        # typedef names, file-scope variables, struct members and function signatures of the project's
        # headers
        types, globs, structs, funcs = set(extra_types), {}, {}, {}
        for h in headers:
            c = Converter(h.read_text(), max_ranks, types, include_map=imap, structs_in=structs)
            c._collect_typedefs_and_globals()
            types |= c.types
            globs.update(c.globals)
            structs.update(c.structs)
            funcs.update(c.functions)
        known = dict(include_map=imap, globals_in=globs, structs_in=structs, functions_in=funcs,
                     array_sizes_in=sizes)
        for h in headers:
            text = Converter(h.read_text(), max_ranks, types, **known).run()
            (out_dir / (h.name + ".cuh")).write_text(text)
        out = out_dir / (src.stem + ".cu")
        out.write_text(Converter(src.read_text(), max_ranks, types, **known).run())
        converted.append(out)
    return converted


def main(argv=None) -> int:
    import argparse
    ap = argparse.ArgumentParser(description="convert C MPI sources to block-rank device code")
    ap.add_argument("sources", nargs="+")
    ap.add_argument("-o", "--out-dir", default=".")
    ap.add_argument("-I", dest="include_dirs", action="append", default=[])
    ap.add_argument("--max-ranks", type=int, default=None)
    ap.add_argument("--type", dest="types", action="append", default=[], help="extra typedef name")
    a = ap.parse_args(argv)
    try:
        for p in convert_files(a.sources, a.out_dir, a.max_ranks, a.include_dirs, extra_types=a.types):
            print(p)
    except ConversionError as e:
        print(f"gpumpi converter: {e}")
        return 1
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
