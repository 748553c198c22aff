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
