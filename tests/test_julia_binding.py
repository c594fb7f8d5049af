"""The Julia binding sources (justpic.jl_gb300/julia/*.jl) against the C ABI
in include/justpic_gb300.h, read as text (there is no Julia here): every
``ccall`` names a declared entry point, passes as many arguments as the
prototype takes, and declares each argument with a Julia type of the same
C shape. An array of pointers (``const double* const coords[3]``, ``double*
const* F``) is a pointer to pointers on the C side, so the ccall must declare
``Ptr{Ptr{...}}`` (a tuple declared by value would be passed as an aggregate)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "justpic_gb300.h")
JULIA = os.path.join(ROOT, "justpic.jl_gb300", "julia")


def _split_top(s, sep=","):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def prototypes():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    protos = {}
    for m in re.finditer(r"\b[\w\s\*]*?\b(jp_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        params = [p for p in _split_top(" ".join(m.group(2).split())) if p and p != "void"]
        protos[m.group(1)] = params
    return protos


def c_shape(param):
    """'pp' pointer to pointers, 'p' pointer, or the scalar type."""
    p = param.strip()
    if re.search(r"\[\s*\d*\s*\]\s*$", p):
        base = re.sub(r"\w+\s*\[\s*\d*\s*\]\s*$", "", p)
        return "pp" if "*" in base else "p"
    if p.count("*") >= 2:
        return "pp"
    if "*" in p:
        return "p"
    scalar = p.rsplit(" ", 1)[0].replace("const ", "").strip()
    return {"double": "f64", "float": "f32", "int32_t": "i32", "int": "i32", "int64_t": "i64",
            "uint64_t": "u64", "uint32_t": "u32", "size_t": "u64", "uint8_t": "u8"}.get(scalar, scalar)


def julia_shape(t):
    t = t.strip()
    if re.fullmatch(r"(Ptr|Ref)\{(Ptr|Ref)\{.*\}\}", t):
        return "pp"
    if t.startswith(("Ptr{", "Ref{")) or t in ("Cstring", "Ptr"):
        return "p"
    return {"Float64": "f64", "Cdouble": "f64", "Float32": "f32", "Cfloat": "f32", "Int32": "i32",
            "Cint": "i32", "Int64": "i64", "UInt64": "u64", "Csize_t": "u64", "UInt32": "u32",
            "UInt8": "u8"}.get(t, t)


def ccalls():
    out = []
    for fn in sorted(os.listdir(JULIA)):
        if not fn.endswith(".jl"):
            continue
        text = open(os.path.join(JULIA, fn)).read()
        for m in re.finditer(r"ccall\(\(:(jp_[a-z0-9_]+),\s*lib\),\s*\w+,\s*\(", text):
            i, depth = m.end(), 1
            while depth:
                depth += {"(": 1, ")": -1}.get(text[i], 0)
                i += 1
            types = _split_top(" ".join(text[m.end():i - 1].split()))
            line = text.count("\n", 0, m.start()) + 1
            out.append((fn, line, m.group(1), types))
    return out


def test_julia_sources_have_ccalls():
    assert len(ccalls()) > 30


@pytest.mark.parametrize("fn,line,name,types", ccalls(), ids=lambda v: v if isinstance(v, str) else None)
def test_ccall_matches_the_header(fn, line, name, types):
    protos = prototypes()
    assert name in protos, f"{fn}:{line}: {name} is not declared in the header"
    params = protos[name]
    assert len(types) == len(params), f"{fn}:{line}: {name} takes {len(params)} arguments, ccall declares {len(types)}"
    for k, (p, t) in enumerate(zip(params, types)):
        assert c_shape(p) == julia_shape(t), f"{fn}:{line}: {name} argument {k + 1}: C '{p}' vs Julia '{t}'"
