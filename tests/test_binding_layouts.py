"""The ABI structs as the three hosts see them (no GPU): the field types of every
`typedef struct` of include/bemgpu.h, in order, against the Julia `struct` mirrors in
julia/BEMGPU.jl (which cannot be run here: Julia is absent) and the ctypes mirrors in
bemgpu/_lib.py.  A field added to the header and not to a binding shifts every later
field, so this is checked on the CPU before any GPU sees it."""
import ctypes
import pathlib
import re

import pytest

from bemgpu import _lib as C

ROOT = pathlib.Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "bemgpu.h"
JULIA = ROOT / "acousticscattering.jl_gb300" / "julia" / "BEMGPU.jl"

C_TYPES = {"int32_t": "i32", "int64_t": "i64", "uint64_t": "u64", "double": "f64"}
JL_TYPES = {"Int32": "i32", "Int64": "i64", "UInt64": "u64", "Float64": "f64"}
CT_TYPES = {ctypes.c_int32: "i32", ctypes.c_int64: "i64", ctypes.c_uint64: "u64",
            ctypes.c_double: "f64"}

# header struct -> (Julia struct, ctypes struct)
PAIRS = {
    "bemgpu_problem": ("Problem", C.Problem),
    "bemgpu_diagnostics": ("Diagnostics", C.Diagnostics),
    "bemgpu_hmatrix_options": ("HmatrixOptions", C.HmatrixOptions),
    "bemgpu_hmatrix_stats": ("HmatrixStats", C.HmatrixStats),
    "bemgpu_server_options": ("ServerOptions", C.ServerOptions),
    "bemgpu_server_stats": ("ServerStats", C.ServerStats),
}


def _header_structs():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef struct \{(.*?)\}\s*(\w+);", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            typ, names = decl.split(None, 1)
            for n in names.split(","):
                n = n.strip()
                count = 1
                m = re.match(r"(\w+)\[(\d+)\]", n)
                if m:
                    n, count = m.group(1), int(m.group(2))
                fields += [(n, C_TYPES[typ])] * count
        out[name] = fields
    return out


def _julia_structs():
    text = JULIA.read_text()
    out = {}
    for name, body in re.findall(r"^struct (\w+)\n(.*?)^end", text, flags=re.S | re.M):
        fields = []
        for line in body.splitlines():
            line = line.split("#")[0].strip()
            m = re.match(r"(\w+)::(\w+)$", line)
            if m and m.group(2) in JL_TYPES:
                fields.append((m.group(1), JL_TYPES[m.group(2)]))
            elif m:
                fields = None  # a non-ABI struct (handles, payloads)
                break
        if fields:
            out[name] = fields
    return out


@pytest.mark.parametrize("cname", sorted(PAIRS))
def test_julia_and_ctypes_mirror_the_header(cname):
    hdr = _header_structs()
    jl = _julia_structs()
    jname, ct = PAIRS[cname]
    want = [t for _, t in hdr[cname]]
    assert [t for _, t in jl[jname]] == want, jname
    got = []
    for _, typ in ct._fields_:
        if hasattr(typ, "_length_"):       # fixed arrays
            got += [CT_TYPES[typ._type_]] * typ._length_
        else:
            got.append(CT_TYPES[typ])
    assert got == want, ct.__name__
    # and the ctypes sizes agree with the header's natural C layout
    assert ctypes.sizeof(ct) == _c_size(want)


def _c_size(types):
    size = {"i32": 4, "i64": 8, "u64": 8, "f64": 8}
    off, align = 0, 1
    for t in types:
        s = size[t]
        off = (off + s - 1) // s * s + s
        align = max(align, s)
    return (off + align - 1) // align * align


# ------------------------------------------------------------------ function prototypes
_STRUCTS = {"bemgpu_problem": "problem", "bemgpu_diagnostics": "diagnostics",
            "bemgpu_hmatrix_options": "hmatrix_options", "bemgpu_hmatrix_stats": "hmatrix_stats",
            "bemgpu_server_options": "server_options", "bemgpu_server_stats": "server_stats"}
_SCALARS = {"int32_t": "i32", "int": "i32", "int64_t": "i64", "uint64_t": "u64",
            "double": "f64", "size_t": "u64"}
_POINTEES = {"double": "f64*", "float": "f32*", "int64_t": "i64*", "int32_t": "i32*",
             "uint64_t": "u64*", "char": "char*", "void": "ptr"}


def _c_param(decl):
    decl = re.sub(r"\bconst\b", "", decl)
    decl = re.sub(r"\*\s+\*", "**", " ".join(decl.split()))
    m = re.match(r"([\w]+)\s*(\**)\s*\w*(\[\d*\])?$", decl)
    base, stars = m.group(1), m.group(2) + ("*" if m.group(3) else "")
    if not stars:
        return _SCALARS[base]
    if len(stars) == 2:
        return "f64**" if base == "double" else "pptr"
    if base in _STRUCTS:
        return _STRUCTS[base] + "*"
    if base.startswith("bemgpu_"):
        return "ptr"  # opaque handles
    return _POINTEES[base]


def _header_prototypes():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for name, params in re.findall(r"^(?:int|void|const char \*)\s*(bemgpu_\w+)\((.*?)\);",
                                   text, flags=re.S | re.M):
        params = " ".join(params.split())
        out[name] = [] if params in ("", "void") else [_c_param(p) for p in params.split(",")]
    return out


def _ctypes_class(t):
    if t is ctypes.c_void_p:
        return "ptr"
    if t is ctypes.c_char_p:
        return "char*"
    for k, v in {ctypes.c_int32: "i32", ctypes.c_int64: "i64", ctypes.c_uint64: "u64",
                 ctypes.c_double: "f64", ctypes.c_size_t: "u64"}.items():
        if t is k:
            return v
    inner = t._type_
    if inner is ctypes.c_void_p:
        return "pptr"
    if getattr(inner, "_type_", None) is ctypes.c_double:
        return "f64**"
    for name, ct in PAIRS.items():
        if inner is ct[1]:
            return _STRUCTS[name] + "*"
    return {ctypes.c_double: "f64*", ctypes.c_float: "f32*", ctypes.c_int64: "i64*",
            ctypes.c_int32: "i32*", ctypes.c_uint64: "u64*", ctypes.c_char: "char*"}[inner]


def _julia_class(t):
    t = t.strip()
    scal = {"Cint": "i32", "Int32": "i32", "Int64": "i64", "UInt64": "u64", "Float64": "f64",
            "Csize_t": "u64"}
    if t in scal:
        return scal[t]
    m = re.match(r"(Ptr|Ref)\{(.*)\}$", t)
    inner = m.group(2)
    if inner == "Cvoid":
        return "ptr"
    if inner == "Ptr{Cvoid}":
        return "pptr"
    if inner == "Ptr{Float64}":
        return "f64**"
    jl = {j: _STRUCTS[c] + "*" for c, (j, _) in PAIRS.items()}
    if inner in jl:
        return jl[inner]
    return {"Float64": "f64*", "Float32": "f32*", "Int64": "i64*", "Int32": "i32*",
            "UInt64": "u64*", "UInt8": "char*", "Cchar": "char*"}[inner]


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "{(":
            depth += 1
        elif ch in "})":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur)
    return [p.strip() for p in parts if p.strip()]


def _julia_ccalls():
    text = JULIA.read_text()
    out = []
    for m in re.finditer(r"ccall\(\(:(bemgpu_\w+),\s*libbemgpu\),\s*(\w+),\s*\(", text):
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(text[i], 0)
            i += 1
        out.append((m.group(1), [_julia_class(t) for t in _split_top(text[m.end():i - 1])]))
    return out


def test_ctypes_signatures_match_the_header():
    protos = _header_prototypes()
    assert len(protos) > 50
    for name, (_, args) in C.SIGNATURES.items():
        assert name in protos, name
        assert [_ctypes_class(a) for a in args] == protos[name], name


def test_julia_ccalls_match_the_header():
    """Every ccall of BEMGPU.jl passes the argument types of the C prototype (an opaque
    Ptr{Cvoid} stands for any handle; a Ref of a struct for a pointer to it)."""
    protos = _header_prototypes()
    calls = _julia_ccalls()
    assert len(calls) >= 29
    for name, got in calls:
        want = protos[name]
        assert len(got) == len(want), (name, got, want)
        for g, w in zip(got, want):
            assert g == w or (g == "ptr" and w.endswith("*")), (name, got, want)
