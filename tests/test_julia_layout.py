"""The Julia binding (julia/RBFFDGPU.jl) against the C ABI, without Julia.

Julia is not installed here, so the shim's `ccall`s cannot run.  What can go wrong in a
ccall binding without a compiler noticing is layout and arity, and those are checked on the
CPU:

* every plain `struct` of the shim that crosses the ABI (Options, Stats, CSC, Problem) has the
  same field names, in the same order, at the same byte offsets and sizes, as the C struct in
  include/rbffd.h (offsets from a C program compiled against the header) and as the ctypes
  mirror in _native.py; a field added on one side only fails the test;
* every `ccall` names a symbol that include/rbffd.h declares and that _native.EXPORTED lists,
  and its argument and return types match the C prototype in count and kind (pointer, 32-bit
  or 64-bit integer, double), argument by argument.

These mirror the reference's exported API (src/RadialBasisFiniteDifferences.jl:58,62:
generate_operator, hyperviscosity_operator), which the shim re-exposes over the C ABI.
"""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "radialbasisfinitedifferences.jl_gb300", "julia", "RBFFDGPU.jl")
HDR = os.path.join(ROOT, "include", "rbffd.h")

# Julia struct -> (C typedef, ctypes class name in _native.py)
STRUCTS = {"Options": ("rbffd_options", "Options"), "Stats": ("rbffd_stats", "Stats"),
           "CSC": ("rbffd_csc", "CSC"), "Problem": ("rbffd_problem", "Problem")}

JL_SCALARS = {"Cint": (4, "i32"), "Int32": (4, "i32"), "UInt32": (4, "u32"), "Cuint": (4, "u32"),
              "Int64": (8, "i64"), "UInt64": (8, "u64"), "Csize_t": (8, "u64"), "Cdouble": (8, "f64"),
              "Float64": (8, "f64"), "UInt8": (1, "u8"), "Cvoid": (0, "void"), "Cstring": (8, "ptr")}
C_SCALARS = {"int": "i32", "int32_t": "i32", "uint32_t": "u32", "int64_t": "i64", "uint64_t": "u64",
             "size_t": "u64", "double": "f64", "uint8_t": "u8", "void": "void"}


def jl_type(t):
    """(size, alignment, kind) of a Julia field or argument type."""
    t = t.strip()
    if t.startswith(("Ptr{", "Ref{")):
        return 8, 8, "ptr"
    m = re.fullmatch(r"NTuple\{(\d+),\s*(\w+)\}", t)
    if m:
        sz, kind = JL_SCALARS[m.group(2)]
        return int(m.group(1)) * sz, sz, f"{kind}[{m.group(1)}]"
    sz, kind = JL_SCALARS[t]
    return sz, max(sz, 1), kind


def split_top(s):
    """Split s at commas outside braces and parentheses."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "{(":
            depth += 1
        elif ch in "})":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def julia_structs(src):
    out = {}
    for m in re.finditer(r"^struct (\w+)\n(.*?)^end", src, re.M | re.S):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("#")[0].strip()
            if line:
                name, typ = line.split("::", 1)
                fields.append((name.strip(), typ.strip()))
        out[m.group(1)] = fields
    return out


def julia_layout(fields):
    off, lay, maxal = 0, [], 1
    for name, typ in fields:
        sz, al, _ = jl_type(typ)
        off = (off + al - 1) // al * al
        lay.append((name, off, sz))
        off += sz
        maxal = max(maxal, al)
    return lay, (off + maxal - 1) // maxal * maxal


def strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", "", s, flags=re.S)


def c_structs(hdr):
    """Field names (in order) of every `typedef struct { ... } name;` of the header."""
    out = {}
    for m in re.finditer(r"typedef struct \{(.*?)\}\s*(\w+);", strip_c_comments(hdr), re.S):
        names = []
        for decl in m.group(1).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            parts = split_top(decl)
            parts[0] = parts[0].split()[-1]
            for d in parts:
                names.append(re.sub(r"\[\d+\]", "", d.replace("*", "")).strip())
        out[m.group(2)] = names
    return out


def c_kind(decl):
    """Kind of a C return type ('ptr' for any pointer)."""
    if "*" in decl:
        return "ptr"
    toks = [t for t in decl.split() if t not in ("const", "struct", "unsigned")]
    return C_SCALARS[toks[0]] if toks else "void"


def c_param_kind(p):
    """Kind of one named C parameter (`const double *X`, `rbffd_csc out[]`, `int64_t N`)."""
    p = p.strip()
    if "*" in p or "[" in p:
        return "ptr"
    return c_kind(" ".join(p.split()[:-1]))


def c_prototypes(hdr):
    """{name: (return kind, [param kinds])} of every rbffd_* function the header declares."""
    src = re.sub(r"^#.*$", "", strip_c_comments(hdr), flags=re.M)
    out = {}
    for m in re.finditer(r"([\w \*]+?)\b(rbffd_\w+)\s*\(([^;{]*?)\)\s*;", src, re.S):
        ret, name, params = m.group(1).replace("typedef", "").strip(), m.group(2), m.group(3)
        ps = [] if params.strip() in ("", "void") else [c_param_kind(p) for p in split_top(params)]
        out[name] = (c_kind(ret), ps)
    return out


def julia_ccalls(src):
    """[(symbol, return kind, [arg kinds])] of every ccall((:sym, LIB), Ret, (T...), ...)."""
    out = []
    for m in re.finditer(r"ccall\(\(:(\w+),\s*LIB\),\s*", src):
        i = j = m.end()
        depth = 0
        while src[j] != "," or depth:  # the return type
            depth += src[j] in "{("
            depth -= src[j] in "})"
            j += 1
        ret = src[i:j].strip()
        k = e = src.index("(", j)
        depth = 0
        while True:
            depth += src[e] == "("
            depth -= src[e] == ")"
            if depth == 0:
                break
            e += 1
        args = [a for a in split_top(src[k + 1:e]) if a]
        out.append((m.group(1), jl_type(ret)[2], [jl_type(a)[2] for a in args]))
    return out


@pytest.fixture(scope="module")
def sources():
    return open(JL).read(), open(HDR).read()


@pytest.fixture(scope="module")
def c_offsets(sources, tmp_path_factory):
    """{struct: (sizeof, {field: (offsetof, sizeof)})} from a C program built against the header."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "rbffd.h"', "int main(void) {"]
    for s, names in c_structs(sources[1]).items():
        lines.append(f'printf("S {s} %zu\\n", sizeof({s}));')
        for f in names:
            lines.append(f'printf("F {s} {f} %zu %zu\\n", offsetof({s}, {f}), sizeof((({s} *)0)->{f}));')
    lines += ["return 0;", "}"]
    d = tmp_path_factory.mktemp("layout")
    (d / "layout.c").write_text("\n".join(lines))
    subprocess.run([cc, "-std=c11", "-I", os.path.dirname(HDR), str(d / "layout.c"), "-o", str(d / "layout")],
                   check=True)
    out = {}
    for line in subprocess.run([str(d / "layout")], check=True, capture_output=True, text=True).stdout.splitlines():
        t = line.split()
        if t[0] == "S":
            out[t[1]] = (int(t[2]), {})
        else:
            out[t[1]][1][t[2]] = (int(t[3]), int(t[4]))
    return out


def test_every_abi_struct_of_the_shim_is_checked(sources):
    assert set(julia_structs(sources[0])) == set(STRUCTS)


@pytest.mark.parametrize("jname", sorted(STRUCTS))
def test_struct_layout_julia_c_ctypes(pkg, sources, c_offsets, jname):
    cname, pyname = STRUCTS[jname]
    jfields = julia_structs(sources[0])[jname]
    jlay, jsize = julia_layout(jfields)
    csize, cf = c_offsets[cname]
    py = getattr(pkg._native, pyname)
    assert [f for f, _ in jfields] == c_structs(sources[1])[cname] == [f for f, _ in py._fields_], jname
    for name, off, sz in jlay:
        assert cf[name] == (off, sz), (jname, name, cf[name], (off, sz))
        fd = getattr(py, name)
        assert (fd.offset, fd.size) == (off, sz), (jname, name)
    assert jsize == csize == ctypes.sizeof(py), (jname, jsize, csize, ctypes.sizeof(py))


def test_ccall_signatures_match_the_header(pkg, sources):
    protos = c_prototypes(sources[1])
    calls = julia_ccalls(sources[0])
    assert len(calls) >= 15
    for sym, ret, args in calls:
        assert sym in protos and sym in pkg._native.EXPORTED, sym
        cret, cargs = protos[sym]
        assert ret == cret, (sym, ret, cret)
        assert args == cargs, (sym, args, cargs)


def test_header_declares_what_native_exports(pkg, sources):
    assert set(c_prototypes(sources[1])) == set(pkg._native.EXPORTED)
